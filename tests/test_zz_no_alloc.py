"""fdb_checksum_noalloc: the checksum for callers that may not allocate GPU
memory while they run (memory pools or arenas that own all device memory,
hosts that forbid allocation after start-up).  It runs the same kernels with
the same chunking as the handle's fdb_upwind_checksum, so the sums must be
equal bit for bit, call after call, with its scratch in a static device array.
Kept in its own file, named to be collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_sum(lib, field_ptr: int, n: int, d_sum, stream) -> float:
    import torch
    from fidibench_gb300._capi import FDB_OK

    d_sum.fill_(float("nan"))
    torch.cuda.synchronize()
    rc = lib.fdb_checksum_noalloc(ctypes.c_void_p(field_ptr), n,
                                  ctypes.c_void_p(d_sum.data_ptr()), ctypes.c_void_p(stream))
    assert rc == FDB_OK, lib.fdb_last_error()
    torch.cuda.synchronize()
    return float(d_sum.item())


def test_noalloc_checksum_matches_handle_checksum_twice(fdb):
    import torch
    from fidibench_gb300._capi import lib

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
        got = _noalloc_sum(lib, up.field_ptr(), ntot, d_sum, stream)
        assert got == expected, (call, got, expected)
    up.close()


def test_noalloc_checksum_all_partials_and_short_last_chunk(fdb):
    """2^24 + 5 values: the reduction uses all 2048 static partial slots and
    the last CTA sums a short chunk (6150 of 8193 values)."""
    import torch
    from fidibench_gb300._capi import lib

    ntot = (1 << 24) + 5
    up = fdb.Upwind((1.0,), (1.0,), (ntot,))
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    x = torch.rand(ntot, generator=g, device="cuda", dtype=torch.float64) - 0.25
    d_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        if call == 1:
            x.mul_(-3.0)
        up.set_field(x)
        expected = up.checksum()
        got = _noalloc_sum(lib, x.data_ptr(), ntot, d_sum, stream)
        assert got == expected, (call, got, expected)
    up.close()


def test_noalloc_checksum_rejects_bad_sizes_and_pointers(fdb):
    import torch
    from fidibench_gb300._capi import FDB_ERR_INVALID, lib

    x = torch.ones(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(x.data_ptr()), 0,
                                    ctypes.c_void_p(out.data_ptr()), None) == FDB_ERR_INVALID
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(x.data_ptr()), (1 << 34) + 1,
                                    ctypes.c_void_p(out.data_ptr()), None) == FDB_ERR_INVALID
    assert b"FDB_NOALLOC_MAX_VALUES" in lib.fdb_last_error()
    # pageable host memory is rejected before any kernel is enqueued
    host = np.ones(4)
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(host.ctypes.data), 4,
                                    ctypes.c_void_p(out.data_ptr()), None) == FDB_ERR_INVALID
    assert b"d_field" in lib.fdb_last_error()
    hsum = np.zeros(1)
    assert lib.fdb_checksum_noalloc(ctypes.c_void_p(x.data_ptr()), 4,
                                    ctypes.c_void_p(hsum.ctypes.data), None) == FDB_ERR_INVALID
    assert b"d_sum" in lib.fdb_last_error()
