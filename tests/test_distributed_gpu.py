"""The distributed form's GPU path on one GPU: every slab of a 1-4 way
decomposition as its own slab handle (fdb_upwind_create_slab), the halo
exchange done by device copies between them (SlabRing; the multi-process
form, DistributedUpwind, moves the same planes with NCCL), checked against
the oracle's whole-grid advect.  EXACT is bit-identical for every slab count
and both halo sides; the fixed-point arithmetic (one scale per slab) within
1e-13; the checksum (sum of the slabs' own-plane sums) within 1e-12.  Also
the single-rank DistributedUpwind (no process group: the halo is the slab's
own far end) and the plane-range C-ABI itself."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-13
SUM_TOL = 1e-12

CASES = [
    # n, v, L, steps, halo
    ((24, 10, 12), (1.0, -0.7, 0.3), (1.0, 1.0, 1.0), 11, 3),
    ((20, 9, 16), (-0.8, 0.5, -0.2), (1.0, 2.0, 0.5), 10, 4),
    ((17, 13), (0.6, -0.9), (1.0, 1.0), 7, 2),
    ((29,), (-1.1,), (1.0,), 9, 3),
]


@pytest.mark.parametrize("world", [1, 2, 3, 4])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_slab_ring_exact_matches_oracle(fdb, port, world, case):
    from fidibench_gb300.distributed import SlabRing
    from oracle import cfl_dt
    n, v, L, steps, halo = CASES[case]
    rng = np.random.default_rng(7 + case)
    f0 = rng.standard_normal(int(np.prod(n)))
    dt = cfl_dt(n, v, L, 0.5)
    ring = SlabRing(v, L, n, world, halo=halo, arith="exact")
    ring.set_global_field(f0)
    ring.advect(steps, dt)
    out = ring.gather()
    cs = ring.checksum()
    ring.close()
    ref = port.advect(n, v, L, f0, steps, dt)
    assert np.array_equal(out, ref), rel_maxnorm(out, ref)
    assert cs == pytest.approx(port.checksum(ref), rel=SUM_TOL, abs=1e-12)


@pytest.mark.parametrize("world", [1, 2, 4])
@pytest.mark.parametrize("v", [(1.0, -0.7, 0.3), (-0.9, 0.4, 0.6)])
def test_slab_ring_fixed_point_matches_oracle(fdb, port, world, v):
    """96 x 64 x 80 with the block-fixed-point kernel forced on every slab
    (its temporal depth = the halo depth, so one launch per exchange)."""
    from fidibench_gb300.distributed import SlabRing
    n, L = (96, 64, 80), (1.0, 1.0, 1.0)
    f0 = port.sphere_noise(n, L, (0.5, 0.5, 0.5), 0.2, 0.01, 20261203)
    dt = 0.5 / 96
    ring = SlabRing(v, L, n, world, halo=3, arith="fixed", depth=3)
    ring.set_global_field(f0)
    ring.advect(20, dt)
    out = ring.gather()
    cs = ring.checksum()
    used = {s.arith_used for s in ring.slabs}
    ring.close()
    assert used == {"fixed"}
    ref = port.advect(n, v, L, f0, 20, dt)
    assert rel_maxnorm(out, ref) <= FIELD_TOL
    assert cs == pytest.approx(port.checksum(ref), rel=SUM_TOL)


def test_single_rank_distributed_matches_plain_advect(fdb):
    """DistributedUpwind without a process group: one slab whose halo is its
    own far end (periodic); bit-identical to Upwind under EXACT."""
    import torch
    from fidibench_gb300.distributed import DistributedUpwind
    n, v, L = (40, 24, 32), (0.7, 0.2, -0.5), (1.0, 1.0, 1.0)
    dt = 0.45 / 40
    rng = np.random.default_rng(3)
    f0 = rng.random(int(np.prod(n)))
    d = DistributedUpwind(v, L, n, halo=4, arith="exact")
    d.set_global_field(f0)
    d.advect(13, dt)
    torch.cuda.synchronize()
    out = d.gather()
    cs = d.checksum()
    d.close()
    up = fdb.Upwind(v, L, n, arith="exact")
    up.f = f0
    up.advect(13, dt)
    assert np.array_equal(out, up.f)
    assert cs == pytest.approx(up.checksum(), rel=SUM_TOL)
    up.close()


def test_plane_range_capi(fdb):
    import torch
    from fidibench_gb300._capi import FDB_ERR_INVALID, FDB_OK, lib
    n = (6, 5, 4)
    up = fdb.Upwind((1.0, 1.0, 1.0), (1.0, 1.0, 1.0), n)
    f = np.arange(120, dtype=np.float64)
    up.f = f
    h = up._h
    got = np.empty(40)
    assert lib.fdb_upwind_get_planes(h, 2, 2, got.ctypes.data, 0) == FDB_OK
    assert np.array_equal(got, f[40:80])
    t = torch.full((20,), -1.0, dtype=torch.float64, device="cuda")
    assert lib.fdb_upwind_set_planes(h, 5, 1, ctypes.c_void_p(t.data_ptr()), 1) == FDB_OK
    want = f.copy()
    want[100:120] = -1.0
    assert np.array_equal(up.f, want)
    s = ctypes.c_double()
    assert lib.fdb_upwind_checksum_planes(h, 1, 3, ctypes.byref(s)) == FDB_OK
    assert s.value == pytest.approx(float(np.sum(want[20:80])), rel=1e-15)
    assert lib.fdb_upwind_get_planes(h, 5, 2, got.ctypes.data, 0) == FDB_ERR_INVALID
    assert lib.fdb_upwind_checksum_planes(h, 7, 0, ctypes.byref(s)) == FDB_ERR_INVALID
    up.close()
