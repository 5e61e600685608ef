"""fdb_checksum_noalloc: the checksum for callers that may not allocate GPU
memory while they run (memory pools or arenas that own all device memory,
hosts that forbid allocation after start-up).  It must give the same sum as
the handle's fdb_upwind_checksum, call after call, with its scratch in a
static device array.  Kept in its own file, named to be collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUM_TOL = 1e-12


def test_noalloc_checksum_matches_handle_checksum_twice(fdb):
    import torch
    from fidibench_gb300._capi import FDB_OK, lib

    n = (96, 80, 112)
    up = fdb.Upwind((1.0, -0.7, 0.3), (1.0, 1.0, 1.0), n)
    up.init_sphere((0.5, 0.5, 0.5), 0.2, 0.01, 7)
    ntot = int(np.prod(n))
    d_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        if call == 1:
            up.advect(10, 0.5 / 112)  # a different field for the second call
        expected = up.checksum()  # synchronises the handle's stream
        d_sum.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.fdb_checksum_noalloc(ctypes.c_void_p(up.field_ptr()), ntot,
                                      ctypes.c_void_p(d_sum.data_ptr()), ctypes.c_void_p(stream))
        assert rc == FDB_OK, lib.fdb_last_error()
        torch.cuda.synchronize()
        got = float(d_sum.item())
        assert got == pytest.approx(expected, rel=SUM_TOL), (call, got, expected)
    up.close()


def test_noalloc_checksum_rejects_bad_sizes(fdb):
    import torch
    from fidibench_gb300._capi import FDB_ERR_INVALID, lib

    x = torch.ones(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(x.data_ptr()), 0,
                                    ctypes.c_void_p(out.data_ptr()), None) == FDB_ERR_INVALID
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(x.data_ptr()), (1 << 34) + 1,
                                    ctypes.c_void_p(out.data_ptr()), None) == FDB_ERR_INVALID
    assert b"FDB_NOALLOC_MAX_VALUES" in lib.fdb_last_error()
