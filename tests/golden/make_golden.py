"""Generate the golden fixtures in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py

Runs the reference's own Upwind<NDIMS> (upwind/cxx/upwind.cxx, compiled by
oracle/Makefile target `ref` from the reference tree, no FMA contraction) and
the reference's Python Upwind (upwind/python/upwind.py, imported from the
reference tree) on small seeded inputs, and stores inputs and outputs as
.npz files.  The reference tree is read only by this script; the tests read
the committed .npz files, so they also run where the reference is absent.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import Port, Reference, build, cfl_dt, reference_dt  # noqa: E402
from oracle.oracle import reference_dir  # noqa: E402

REFDIR = reference_dir()
SEED = 20261203


def save(name: str, **arrays) -> None:
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", os.path.relpath(path, ROOT), os.path.getsize(path), "bytes")


def field_cases(ref: Reference, port: Port) -> None:
    rng = np.random.default_rng(SEED)
    cases = [
        # name, n, v, L, steps, cfl, init
        ("g3_7x5x6_mixed", (7, 5, 6), (1.0, -0.7, 0.3), (1.0, 1.0, 1.0), 13, 0.5, "uniform"),
        ("g3_8x8x8_c1sphere", (8, 8, 8), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), 10, 0.5, "sphere"),
        ("g3_5x9x4_negall", (5, 9, 4), (-0.9, -0.2, -1.0), (2.0, 0.5, 1.0), 21, 0.45, "uniform"),
        ("g3_1x6x3_zerov", (1, 6, 3), (0.0, 0.6, -0.0), (1.0, 1.0, 1.0), 7, 0.5, "signed"),
        ("g3_3x3x3_c2noise", (3, 3, 3), (1.0, -0.7, 0.3), (1.0, 1.0, 1.0), 100, 0.5, "sphere_noise"),
        ("g2_9x11", (9, 11), (-0.4, 0.9), (1.0, 1.0), 17, 0.5, "uniform"),
        ("g1_17", (17,), (-1.3,), (1.0,), 9, 0.8, "signed"),
        ("g4_3x4x5x6", (3, 4, 5, 6), (0.1, -0.2, 0.3, -0.4), (1.0, 1.0, 1.0, 1.0), 5, 0.5,
         "uniform"),
    ]
    for name, n, v, L, steps, cfl, init in cases:
        ntot = int(np.prod(n))
        if init == "uniform":
            f0 = rng.random(ntot)
        elif init == "signed":
            f0 = rng.standard_normal(ntot)
        elif init == "sphere":
            f0 = port.sphere_noise(n, L, [0.5 * x for x in L], 0.2 * min(L), 0.0, 0)
        else:
            f0 = port.sphere_noise(n, L, [0.5 * x for x in L], 0.2 * min(L), 0.01, SEED)
        dt = cfl_dt(n, v, L, cfl)
        fT = ref.advect(n, v, L, f0, steps, dt)
        save(name, n=np.asarray(n, np.uint64), v=np.asarray(v, np.float64),
             L=np.asarray(L, np.float64), dt=np.float64(dt), steps=np.int64(steps), f0=f0, fT=fT,
             checksum=np.float64(ref.checksum(n, fT)), std=np.float64(ref.std(n, fT)))


def driver_cases(ref: Reference) -> None:
    """The reference driver's own run (upwind.cxx:139-217): corner IC, v = 1,
    L = 1, courant 0.1, for the ctest size (128^3 x 10) and 32^3 x 10."""
    for N in (32, 128):
        n = (N, N, N)
        v = (1.0, 1.0, 1.0)
        L = (1.0, 1.0, 1.0)
        dt = reference_dt(n, v, L, 0.1)
        fT = ref.advect(n, v, L, None, 10, dt)
        idx = np.array([0, 1, 2, N, N * N, N * N + N + 1, 10, 11 * N * N, N ** 3 - 1],
                       dtype=np.int64)
        save(f"driver_{N}cube_10", n=np.asarray(n, np.uint64), dt=np.float64(dt),
             steps=np.int64(10), idx=idx, values=fT[idx], checksum=np.float64(ref.checksum(n, fT)),
             std=np.float64(ref.std(n, fT)), nonzero=np.int64(np.count_nonzero(fT)))


def python_reference_case() -> None:
    """The reference's Python Upwind (upwind/python/upwind.py), 12^3 x 10."""
    pydir = os.path.join(REFDIR, "upwind", "python")
    sys.path.insert(0, pydir)
    try:
        import upwind as pyup  # the reference module
    finally:
        sys.path.remove(pydir)
    n = [12, 12, 12]
    v = np.ones(3)
    L = np.ones(3)
    dt = reference_dt(n, v, L, 0.1)
    up = pyup.Upwind(v, L, n)
    for _ in range(10):
        up.advect(dt)
    save("python_12cube_10", n=np.asarray(n, np.uint64), dt=np.float64(dt), steps=np.int64(10),
         fT=up.f.copy(), checksum=np.float64(up.checksum()))


def acc_cases(port: Port) -> None:
    """The reference's OpenACC variants (upwindAcc.cxx: one advect(dt) call
    per step; upwindAcc2.cxx: advect(steps, dt)), compiled serially by
    oracle/ref_acc_harness.cpp: their drivers' own run (corner IC, v = 1,
    courant 0.1, 16^3 x 10) and a mixed-sign seeded field (7 x 5 x 6)."""
    from oracle.oracle import ReferenceAcc
    acc = ReferenceAcc()
    rng = np.random.default_rng(SEED + 7)
    for variant in (1, 2):
        n, v, L = (16, 16, 16), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)
        dt = reference_dt(n, v, L, 0.1)
        fT = acc.advect(variant, n, v, L, None, 10, dt)
        save(f"acc{variant}_16cube_10", n=np.asarray(n, np.uint64), v=np.asarray(v, np.float64),
             L=np.asarray(L, np.float64), dt=np.float64(dt), steps=np.int64(10), fT=fT,
             checksum=np.float64(port.checksum(fT)))
    n, v, L = (7, 5, 6), (0.8, -0.45, 0.3), (1.0, 2.0, 0.5)
    f0 = rng.standard_normal(int(np.prod(n)))
    dt = cfl_dt(n, v, L, 0.5)
    fT = acc.advect(2, n, v, L, f0, 12, dt)
    assert np.array_equal(fT, acc.advect(1, n, v, L, f0, 12, dt))
    save("acc2_7x5x6_mixed", n=np.asarray(n, np.uint64), v=np.asarray(v, np.float64),
         L=np.asarray(L, np.float64), dt=np.float64(dt), steps=np.int64(12), f0=f0, fT=fT,
         checksum=np.float64(port.checksum(fT)))


def filter_cases(port: Port) -> None:
    """The reference's stencil Filter (cxx/Filter.cpp, one rank on
    oracle/mpi_stub; oracle/ref_filter_harness.cpp): the laplacian driver's
    stencil (laplacian/cxx/laplacian.cxx:55-65) on sin inputs, 2-D and 3-D, on
    power-of-two and other grids (the latter exercise the `%= size_t` wrap,
    Filter.cpp:238-240); testStencil2d.cxx's stencil and input; the upwindMpi
    stencil (upwind/cxx/upwindMpi.cxx:74-92) with its corner input over 10
    steps; a seeded general stencil with repeated offsets."""
    from oracle.oracle import ReferenceFilter
    flt = ReferenceFilter()

    def lap(nd):
        st = [(tuple([0] * nd), -2.0 * nd)]
        for i in range(nd):
            for s_ in (1, -1):
                o = [0] * nd
                o[i] = s_
                st.append((tuple(o), 1.0))
        return st

    def store(name, dims, st, f0, iters):
        out, sums = flt.run(dims, st, f0, iters)
        save(name, dims=np.asarray(dims, np.uint64),
             offsets=np.array([o for o, _ in st], np.int32),
             weights=np.array([w for _, w in st], np.float64), f0=f0, iterations=np.int64(iters),
             out=out, sums=np.array(sums, np.float64))

    for dims, iters in (((16, 16), 1), ((10, 12), 1), ((6, 5, 7), 1), ((16, 16), 10)):
        nd = len(dims)
        f0 = port.filter_sin_input(dims, [0.0] * nd, [1.0] * nd)
        name = "filter_lap" + "x".join(str(d) for d in dims) + f"_it{iters}"
        store(name, dims, lap(nd), f0, iters)
    # testStencil2d.cxx: 1 on the cells with a zero index, stencil
    # {0: 0, (1, 0): 1, (0, -1): -1}
    n = 8
    i, j = np.arange(n * n) % n, np.arange(n * n) // n
    store("filter_stencil2d_8", (n, n), [((0, 0), 0.0), ((1, 0), 1.0), ((0, -1), -1.0)],
          ((i * j) == 0).astype(float), 1)
    # upwindMpi.cxx: v = 1, courant 0.1, N = 16, corner input, 10 steps
    N = 16
    dt = 0.1 * (1.0 / N)
    c = dt * 1.0 / (1.0 / N)
    diag = 1.0
    for _ in range(3):
        diag -= 1 * dt * 1.0 / (1.0 / N)
    st = [((0, 0, 0), diag), ((-1, 0, 0), c), ((0, -1, 0), c), ((0, 0, -1), c)]
    f0 = np.zeros(N ** 3)
    f0[0] = 1.0
    store("filter_upwindmpi_16_it10", (N, N, N), st, f0, 10)
    # a general stencil: offsets up to +-2, a repeated offset (first weight wins)
    rng = np.random.default_rng(SEED + 11)
    dims = (7, 5, 6)
    st = [((0, 0, 0), 0.75), ((2, 0, -1), -1.25), ((-1, 1, 0), 0.5), ((0, -2, 2), 2.0),
          ((2, 0, -1), 9.0), ((1, 1, 1), -0.375)]
    store("filter_general_7x5x6", dims, st, rng.standard_normal(int(np.prod(dims))), 2)


def filter_driver_cases() -> None:
    """The reference's Filter drivers, built unmodified for one rank on
    oracle/mpi_stub (oracle/_ref/{laplacian,testStencil2d,upwindMpiCxx}):
    their output lines (timing lines dropped; testStencil2d prints its
    outData to stderr)."""
    import subprocess
    import tempfile
    runs = {
        "laplacian_2d_16": ("laplacian", ["-numCells", "16", "-numDims", "2"]),
        "laplacian_3d_8": ("laplacian", ["-numCells", "8", "-numDims", "3"]),
        "teststencil2d_8": ("testStencil2d", ["-numCells", "8"]),
        "upwindmpi_16_5": ("upwindMpiCxx", ["-numCells", "16", "-numSteps", "5"]),
    }
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for key, (exe, args) in runs.items():
            r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", exe)] + args, cwd=d,
                               capture_output=True, text=True, check=True)
            lines = [ln for ln in (r.stdout + r.stderr).splitlines() if "times" not in ln]
            out[key] = np.array("\n".join(lines))
    save("filterdrivers_stdout", **out)


def vtk_case() -> None:
    """The reference driver binary (oracle/_ref/upwindCxx, built from the
    reference's own upwind.cxx + CmdLineArgParser.cpp) with -vtk -std: its
    stdout and up1.vtk for 6^3 x 3 steps."""
    import subprocess
    import tempfile
    exe = os.path.join(ROOT, "oracle", "_ref", "upwindCxx")
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([exe, "-numCells", "6", "-numSteps", "3", "-vtk", "-std"], cwd=d,
                           capture_output=True, text=True, check=True,
                           env=dict(os.environ, OMP_NUM_THREADS="2"))
        vtk = open(os.path.join(d, "up1.vtk")).read()
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith(("check sum", "std", "number of"))]
    save("driver_vtk_6cube_3", up1_vtk=np.array(vtk), stdout=np.array("\n".join(lines)))


def synth_case(port: Port) -> None:
    """Pins the synthetic sphere+noise generator (no reference counterpart)."""
    n = (16, 12, 10)
    L = (1.0, 1.0, 1.0)
    f = port.sphere_noise(n, L, (0.5, 0.5, 0.5), 0.2, 0.01, SEED)
    u = np.array([port.lib.fdbo_uniform(SEED, i) for i in range(8)])
    save("synth_sphere_16x12x10", n=np.asarray(n, np.uint64), f=f, uniform8=u,
         seed=np.uint64(SEED))


def main() -> None:
    build(ref=True)
    ref = Reference()
    port = Port()
    field_cases(ref, port)
    driver_cases(ref)
    python_reference_case()
    acc_cases(port)
    filter_cases(port)
    filter_driver_cases()
    vtk_case()
    synth_case(port)


if __name__ == "__main__":
    main()
