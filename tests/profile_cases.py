"""Profiling harness: small stand-alone runs of one kernel family, for
profiling a single launch on a case of a few hundred MB
(python tests/profile_cases.py ...).  Not collected by pytest.

  adjoint N S [form] : N^3 field, v = (0.8, 0.5, -0.6), dt = 0.5 min(dx/|v|),
                three adjoint calls of S steps; form "closed" (default: dL/dv
                in closed form) or "stepwise" (one checkpoint segment, the
                recompute and one contraction per transposed step)
  advect N S  : N^3 sphere + noise field, v = (1, -0.7, 0.3), dt = 0.5/N,
                three advect calls of S steps
  batch C S   : C seeded instances with axes in [32, 160] (the benchmark's
                generator), three batched advects of S steps (depth 2,
                shape 4x8 with shared-memory history, whole-z tiles: the
                tuning the autotuner picks for the benchmark's batch)
  filter N I  : 2-D N x N laplacian Filter (the reference laplacian
                driver's stencil and index wrap), three iterate(I) calls
"""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def adjoint_case(n: int, steps: int, form: str = "closed") -> dict:
    import torch
    import fidibench_gb300 as fdb
    v = (0.8, 0.5, -0.6)
    dt = 0.5 * min(1.0 / n / abs(x) for x in v)
    up = fdb.Upwind(v, (1.0,) * 3, (n,) * 3)
    up.set_adjoint_form(form)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1)
    lam = torch.randn(n ** 3, device="cuda", dtype=torch.float64, generator=gen)
    for _ in range(3):
        up.init_sphere((0.5,) * 3, 0.2, 0.01, 1)
        up.adjoint(steps, dt, lam, checkpoint_every=steps)
    t = up.adjoint_timings()
    up.close()
    return t


def advect_case(n: int, steps: int) -> float:
    import fidibench_gb300 as fdb
    up = fdb.Upwind((1.0, -0.7, 0.3), (1.0,) * 3, (n,) * 3)
    up.init_sphere((0.5,) * 3, 0.2, 0.01, 1)
    for _ in range(3):
        up.advect(steps, 0.5 / n)
    cs = up.checksum()
    up.close()
    return cs


def batch_case(count: int, steps: int) -> float:
    from fidibench_gb300.batch import Batch, random_instances
    specs = random_instances(count, 20261203)
    b = Batch([(s["v"], s["L"], s["n"]) for s in specs])
    for k, s in enumerate(specs):
        b.init_sphere(k, s["center"], s["radius"], 0.0, 20261203 + k)
    b.set_tuning(depth=2, shape=4, tile_z=0)
    dts = [s["dt"] for s in specs]
    for _ in range(3):
        b.advect(steps, dts)
    cs = float(sum(b.checksums()))
    b.close()
    return cs


def filter_case(n: int, iters: int) -> float:
    import numpy as np
    from fidibench_gb300.filter import Filter, laplacian_stencil
    x = (np.arange(n, dtype=np.float64) + 0.5) / n
    s = np.sin(2.0 * np.pi * x)
    flt = Filter((n, n), [0.0, 0.0], [1.0, 1.0], laplacian_stencil(2))
    flt.set_in_data(np.ascontiguousarray((s[:, None] * s[None, :]).reshape(-1)))
    for _ in range(3):
        flt.iterate(iters)
    cs = flt.computeCheckSum("out")
    flt.close()
    return cs


def main(argv: list[str]) -> int:
    cases = {"adjoint": adjoint_case, "advect": advect_case, "batch": batch_case,
             "filter": filter_case}
    if len(argv) < 3 or argv[0] not in cases or (len(argv) > 3 and argv[0] != "adjoint"):
        print(__doc__)
        return 2
    print(cases[argv[0]](int(argv[1]), int(argv[2]), *argv[3:4]))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
