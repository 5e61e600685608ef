"""The distributed upwind form on CPU ranks (gloo, world_size 2 and 3): slab
decomposition of axis 0, the ring shift of the K upwind halo planes through
host buffers, the advance in blocks of K steps, the all-reduced checksum and
the all-gather of the field.  The per-rank compute here is the oracle on the
rank's extended slab (CPU stand-in for the GPU slab; test infrastructure),
so the gathered field must equal the oracle's whole-grid advect bit for bit:
that pins the decomposition and exchange logic that the GPU ranks run.
Also: a rank that dies before an exchange is detected, not waited on."""
from __future__ import annotations

import os
import socket
import time

import numpy as np
import pytest
import torch.multiprocessing as mp


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleSlab:
    """The slab protocol of fidibench_gb300.distributed.UpwindSlab, computed
    by the oracle on the extended slab with the global grid's spacings."""

    def __init__(self, port, v, L, n_global, layout, coeff_form=0):
        self.port, self.v, self.L = port, list(v), list(L)
        self.n_global = [int(x) for x in n_global]
        self.layout = layout
        self.plane = int(np.prod(self.n_global[1:])) if len(self.n_global) > 1 else 1
        self.n_ext = [layout.planes] + self.n_global[1:]
        self.f = np.zeros(layout.planes * self.plane)
        self.form = coeff_form

    def _rng(self, first, count):
        return slice(first * self.plane, (first + count) * self.plane)

    def get_planes(self, first, count, out):
        np.asarray(out)[:count * self.plane] = self.f[self._rng(first, count)]

    def set_planes(self, first, count, src):
        self.f[self._rng(first, count)] = np.asarray(src)[:count * self.plane]

    def advect(self, k, dt):
        self.f = self.port.advect_spacing(self.n_ext, self.v, self.L, self.n_global, self.f, k,
                                          dt, coeff_form=self.form)

    def block_begin(self, dt):
        return False  # FP64 steps: no scale to agree on

    def advect_block(self, k, dt, last):
        self.advect(k, dt)

    def checksum_own(self):
        return self.port.checksum(self.f[self._rng(*self.layout.own)])

    def set_own(self, a):
        self.f[self._rng(*self.layout.own)] = np.asarray(a).reshape(-1)

    def get_own(self):
        return self.f[self._rng(*self.layout.own)].copy()


CASES = {
    "3d_low_halo": ((11, 6, 7), (1.0, -0.7, 0.3), (1.0, 1.0, 1.0), 10, 3),
    "3d_high_halo": ((10, 5, 4), (-0.8, 0.5, 0.2), (1.0, 2.0, 0.5), 8, 2),
    "2d": ((9, 5), (0.6, -0.9), (1.0, 1.0), 7, 3),
    "1d_high": ((13,), (-1.1,), (1.0,), 9, 4),
    "zero_v0": ((8, 3, 3), (0.0, 0.4, 0.9), (1.0, 1.0, 1.0), 5, 2),
}


def _worker(rank, ws, port_no, q, case, fail_rank):
    try:
        from fidibench_gb300.distributed import DistributedUpwind
        from fidibench_gb300.sharding import init_host_group
        from oracle import Port, cfl_dt
        dist = init_host_group(rank, ws, "127.0.0.1", port_no, timeout_s=5.0)
        n, v, L, steps, halo = CASES[case]
        port = Port()
        rng = np.random.default_rng(31)
        f0 = rng.standard_normal(int(np.prod(n)))
        dt = cfl_dt(n, v, L, 0.5)
        d = DistributedUpwind(v, L, n, halo=halo,
                              slab_factory=lambda lay: OracleSlab(port, v, L, n, lay))
        d.set_global_field(f0)
        if rank == fail_rank:
            os._exit(3)  # dies between steps, before the first exchange
        d.advect(steps, dt)
        cs = d.checksum()
        full = d.gather()
        if rank == 0:
            ref = port.advect(n, v, L, f0, steps, dt)
            q.put((rank, "ok", bool(np.array_equal(full, ref)), cs, port.checksum(ref),
                   d.halo, d.bounds))
        else:
            q.put((rank, "ok", True, cs, None, d.halo, d.bounds))
        dist.destroy_process_group()
    except Exception as e:  # noqa: BLE001
        q.put((rank, "error", type(e).__name__, str(e)[:300], None, None, None))


def _run(ws, case, fail_rank=-1, wait=90.0):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port_no = free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port_no, q, case, fail_rank))
             for r in range(ws)]
    for p in procs:
        p.start()
    out = []
    deadline = time.time() + wait
    expected = ws - (1 if fail_rank >= 0 else 0)
    while len(out) < expected and time.time() < deadline:
        try:
            out.append(q.get(timeout=1.0))
        except Exception:  # noqa: BLE001
            pass
    for p in procs:
        p.join(timeout=10)
        if p.is_alive():
            p.kill()
    return out


def test_slab_bounds_cover_and_balance():
    from fidibench_gb300.distributed import halo_depth, slab_bounds
    for n0 in (1, 2, 7, 512, 1000):
        for ws in (1, 2, 3, 8):
            if ws > n0:
                with pytest.raises(ValueError):
                    slab_bounds(n0, ws)
                continue
            b = slab_bounds(n0, ws)
            assert b[0][0] == 0 and b[-1][1] == n0
            assert all(b[i][1] == b[i + 1][0] for i in range(ws - 1))
            sizes = [z1 - z0 for z0, z1 in b]
            assert max(sizes) - min(sizes) <= 1
    assert halo_depth(slab_bounds(10, 4), 3) == 2  # the thinnest slab caps the depth


def test_layout_ranges():
    from fidibench_gb300.distributed import SlabLayout
    lo = SlabLayout(4, 9, 3, 1.0, 3, 1)  # v0 >= 0: upwind neighbour below
    assert lo.planes == 8 and lo.own == (3, 5) and lo.halo_at == (0, 3)
    assert lo.send == (5, 3) and lo.upwind == 0 and lo.downwind == 2
    hi = SlabLayout(4, 9, 3, -1.0, 3, 0)  # v0 < 0: upwind neighbour above
    assert hi.own == (0, 5) and hi.halo_at == (5, 3) and hi.send == (0, 3)
    assert hi.upwind == 1 and hi.downwind == 2


@pytest.mark.parametrize("ws,case", [(2, "3d_low_halo"), (3, "3d_low_halo"),
                                     (2, "3d_high_halo"), (3, "3d_high_halo"), (2, "2d"),
                                     (3, "1d_high"), (2, "zero_v0")])
def test_distributed_matches_whole_grid_oracle(ws, case):
    out = _run(ws, case)
    assert len(out) == ws, out
    for rank, status, same, cs, ref_cs, halo, bounds in out:
        assert status == "ok", (rank, same, cs)
        if rank == 0:
            assert same, "gathered field differs from the whole-grid oracle"
            assert cs == pytest.approx(ref_cs, rel=1e-12)
    assert len({o[3] for o in out}) == 1  # every rank returns the same checksum


def test_dead_rank_is_detected_not_hung():
    t0 = time.time()
    out = _run(2, "3d_low_halo", fail_rank=1, wait=60.0)
    assert time.time() - t0 < 60.0
    assert len(out) == 1
    assert out[0][0] == 0 and out[0][1] == "error"
