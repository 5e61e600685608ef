"""The distributed form's GPU path on one GPU: every slab of a 1-4 way
decomposition as its own slab handle (fdb_upwind_create_slab), the halo
exchange done by device copies between them (SlabRing; the multi-process
form, DistributedUpwind, moves the same planes with NCCL), checked against
the oracle's whole-grid advect.  EXACT is bit-identical to the oracle for
every slab count and both halo sides; the fixed-point arithmetic (int64
blocks, int64 halo planes, one scale agreed over all slabs) is bit-identical
to the single-field advect and within 1e-13 of the oracle; the checksum (sum
of the slabs' own-plane sums) within 1e-12.  Also the single-rank
DistributedUpwind (no process group: the halo is the slab's own far end),
the block-chain guards and the plane-range C-ABI itself."""
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


@pytest.mark.parametrize("world", [1, 2, 3, 4])
@pytest.mark.parametrize("v", [(1.0, -0.7, 0.3), (-0.9, 0.4, 0.6)])
def test_slab_ring_fixed_point_bit_identical(fdb, port, world, v):
    """96 x 64 x 80 in the block-fixed-point arithmetic: the slabs keep the
    field int64 between blocks, move int64 halo planes and agree on the scale
    of the whole grid before every block, so the gathered field equals the
    single-field advect at the same depth bit for bit (two advect calls: the
    second starts from the first's scale word), and the oracle within 1e-13."""
    from fidibench_gb300.distributed import SlabRing
    n, L = (96, 64, 80), (1.0, 1.0, 1.0)
    f0 = port.sphere_noise(n, L, (0.5, 0.5, 0.5), 0.2, 0.01, 20261203)
    dt = 0.5 / 96
    ring = SlabRing(v, L, n, world, halo=3, arith="fixed")
    ring.set_global_field(f0)
    ring.advect(20, dt)
    ring.advect(7, dt)
    out = ring.gather()
    cs = ring.checksum()
    used = {s.arith_used for s in ring.slabs}
    ring.close()
    assert used == {"fixed"}
    up = fdb.Upwind(v, L, n, arith="fixed", depth=3)
    up.f = f0
    up.advect(20, dt)
    up.advect(7, dt)
    assert np.array_equal(out, up.f)
    up.close()
    ref = port.advect(n, v, L, f0, 27, dt)
    assert rel_maxnorm(out, ref) <= FIELD_TOL
    assert cs == pytest.approx(port.checksum(ref), rel=SUM_TOL)


def test_block_chain_guards_the_field(fdb):
    """While a block chain is open the field may hold int64 words: the FP64
    calls refuse, plane copies and the scale word work, and a last block
    closes the chain."""
    import ctypes
    from fidibench_gb300._capi import FDB_ERR_INVALID, FDB_OK, lib
    n = (24, 20, 32)
    up = fdb.Upwind((1.0, 0.5, -0.25), (1.0, 1.0, 1.0), n, arith="fixed", depth=3)
    up.init_sphere((0.5, 0.5, 0.5), 0.3, 0.01, 5)
    f0 = up.f
    h = up._h
    fixed = ctypes.c_int()
    dt = 0.5 / 32
    assert lib.fdb_upwind_block_begin(h, dt, ctypes.byref(fixed)) == FDB_OK and fixed.value == 1
    assert lib.fdb_upwind_advect(h, 1, dt) == FDB_ERR_INVALID
    out = np.empty(int(np.prod(n)))
    assert lib.fdb_upwind_get_field(h, out.ctypes.data, 0) == FDB_ERR_INVALID
    w = np.zeros(1, dtype=np.uint64)
    assert lib.fdb_upwind_get_scale_word(h, w.ctypes.data, 0) == FDB_OK and w[0] > 0
    assert lib.fdb_upwind_advect_block(h, 4, dt, 0) == FDB_ERR_INVALID  # deeper than 3
    for k, last in ((3, 0), (3, 0), (2, 1)):
        assert lib.fdb_upwind_advect_block(h, k, dt, last) == FDB_OK, lib.fdb_last_error()
    assert lib.fdb_upwind_advect_block(h, 1, dt, 1) == FDB_ERR_INVALID  # closed
    got = up.f
    ref = fdb.Upwind((1.0, 0.5, -0.25), (1.0, 1.0, 1.0), n, arith="fixed", depth=3)
    ref.f = f0
    ref.advect(8, dt)
    assert np.array_equal(got, ref.f)
    ref.close()
    up.close()


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
