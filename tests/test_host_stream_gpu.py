"""fdb_upwind_advect_host_stream: the driver's cycle (initial field, advect,
checksum) over several host fields with the copies overlapping the kernels.
Every result must be bit-identical to the serial set_field / advect /
get_field / checksum sequence on the same handle kind, and that sequence is
held to the oracle by the parity tests (one case is re-checked here)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

N3 = (40, 33, 57)
V3 = (0.8, -0.45, 0.3)
L3 = (1.0, 1.2, 0.9)


def _dt(n, v, L, cfl=0.4):
    return cfl * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(L, n, v) if vj != 0.0)


def _fields(count, ntot, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(ntot) + 0.1 * k for k in range(count)]


def _serial(fdb, n, v, L, fields, steps, dt, arith="auto"):
    up = fdb.Upwind(v, L, n, arith=arith)
    outs, sums = [], []
    for f in fields:
        up.set_field(f)
        up.advect(steps, dt)
        outs.append(up.f)
        sums.append(up.checksum())
    up.close()
    return outs, np.array(sums)


@pytest.mark.parametrize("arith", ["auto", "fma", "exact"])
def test_matches_serial_cycle(fdb, arith):
    fields = _fields(4, int(np.prod(N3)), 41)
    dt = _dt(N3, V3, L3)
    ref, ref_sums = _serial(fdb, N3, V3, L3, fields, 13, dt, arith)
    up = fdb.Upwind(V3, L3, N3, arith=arith)
    out = [np.empty_like(f) for f in fields]
    sums = up.advect_host_stream(fields, 13, dt, out=out)
    for k in range(len(fields)):
        assert np.array_equal(out[k], ref[k]), k
    assert np.array_equal(sums, ref_sums)
    # the handle is left at the last result
    assert np.array_equal(up.f, ref[-1])
    up.close()


def test_oracle_parity(fdb, port):
    fields = _fields(3, int(np.prod(N3)), 42)
    dt = _dt(N3, V3, L3)
    up = fdb.Upwind(V3, L3, N3)
    out = [np.empty_like(f) for f in fields]
    sums = up.advect_host_stream(fields, 10, dt, out=out)
    up.close()
    for k, f in enumerate(fields):
        ref = port.advect(N3, V3, L3, f, 10, dt)
        assert rel_maxnorm(out[k], ref) <= 1e-13, k
        assert sums[k] == pytest.approx(port.checksum(ref), rel=1e-12), k


def test_pinned_torch_buffers_in_place(fdb):
    import torch
    fields = _fields(5, int(np.prod(N3)), 43)
    dt = _dt(N3, V3, L3)
    ref, ref_sums = _serial(fdb, N3, V3, L3, fields, 7, dt)
    host = [torch.from_numpy(f.copy()).pin_memory() for f in fields]
    up = fdb.Upwind(V3, L3, N3)
    sums = up.advect_host_stream(host, 7, dt)  # results written back in place
    for k in range(len(fields)):
        assert np.array_equal(host[k].numpy(), ref[k]), k
    assert np.array_equal(sums, ref_sums)
    up.close()


def test_shared_buffers(fdb):
    """One input buffer for every field and one output buffer for every result
    (the benchmark's form): each result is the same, the last one stays."""
    ntot = int(np.prod(N3))
    f = _fields(1, ntot, 44)[0]
    dt = _dt(N3, V3, L3)
    ref, ref_sums = _serial(fdb, N3, V3, L3, [f], 9, dt)
    out = np.empty(ntot)
    up = fdb.Upwind(V3, L3, N3)
    sums = up.advect_host_stream([f] * 6, 9, dt, out=[out] * 6)
    assert np.array_equal(out, ref[0])
    assert np.all(sums == ref_sums[0])
    up.close()


def test_repeated_calls_and_continuation(fdb):
    """The three buffers rotate across calls; advecting the handle afterwards
    continues from the last result exactly as the serial sequence does."""
    ntot = int(np.prod(N3))
    dt = _dt(N3, V3, L3)
    a = _fields(3, ntot, 45)
    b = _fields(2, ntot, 46)
    up = fdb.Upwind(V3, L3, N3)
    out_a = [np.empty(ntot) for _ in a]
    out_b = [np.empty(ntot) for _ in b]
    up.advect_host_stream(a, 11, dt, out=out_a)
    up.advect_host_stream(b, 5, dt, out=out_b)
    up.advect(4, dt)
    cont = up.f
    up.close()
    ref_a, _ = _serial(fdb, N3, V3, L3, a, 11, dt)
    ref_b, _ = _serial(fdb, N3, V3, L3, b, 5, dt)
    for k in range(len(a)):
        assert np.array_equal(out_a[k], ref_a[k]), k
    for k in range(len(b)):
        assert np.array_equal(out_b[k], ref_b[k]), k
    s = fdb.Upwind(V3, L3, N3)
    s.set_field(b[-1])
    s.advect(5, dt)
    s.advect(4, dt)
    assert np.array_equal(cont, s.f)
    s.close()


@pytest.mark.parametrize("n,v", [((300,), (-0.5,)), ((33, 90), (0.6, -0.8)),
                                 ((5, 6, 7, 8), (0.3, -0.2, 0.5, 0.1))])
def test_other_dimensions(fdb, n, v):
    L = (1.0,) * len(n)
    dt = _dt(n, v, L)
    fields = _fields(3, int(np.prod(n)), 47)
    ref, ref_sums = _serial(fdb, n, v, L, fields, 6, dt)
    up = fdb.Upwind(v, L, n)
    out = [np.empty_like(f) for f in fields]
    sums = up.advect_host_stream(fields, 6, dt, out=out)
    for k in range(len(fields)):
        assert np.array_equal(out[k], ref[k]), k
    assert np.array_equal(sums, ref_sums)
    up.close()


def test_counts(fdb):
    ntot = int(np.prod(N3))
    dt = _dt(N3, V3, L3)
    up = fdb.Upwind(V3, L3, N3)
    assert up.advect_host_stream([], 5, dt).size == 0
    f = _fields(1, ntot, 48)[0]
    out = np.empty(ntot)
    sums = up.advect_host_stream([f], 0, dt, out=[out])  # zero steps: identity
    assert np.array_equal(out, f)
    assert sums[0] == pytest.approx(float(np.sum(f)), rel=1e-12, abs=1e-9)
    up.close()


def test_errors(fdb):
    from fidibench_gb300._capi import FdbError
    ntot = int(np.prod(N3))
    dt = _dt(N3, V3, L3)
    up = fdb.Upwind(V3, L3, N3, arith="fixed")
    good = _fields(2, ntot, 49)
    with pytest.raises(ValueError):
        up.advect_host_stream([good[0], np.zeros(ntot - 1)], 3, dt)
    with pytest.raises(ValueError):
        up.advect_host_stream(good, 3, dt, out=[np.empty(ntot)])
    with pytest.raises(ValueError):
        up.advect_host_stream([good[0].astype(np.float32)], 3, dt)
    bad = good[1].copy()
    bad[17] = np.nan
    # the fixed-point path needs finite input and says so
    with pytest.raises(FdbError) as e:
        up.advect_host_stream([good[0], bad], 3, dt, out=[np.empty(ntot), np.empty(ntot)])
    assert e.value.code == 6  # FDB_ERR_NONFINITE
    # the handle is still usable and gives the serial results afterwards
    ref, ref_sums = _serial(fdb, N3, V3, L3, good, 3, dt, arith="fixed")
    out = [np.empty(ntot) for _ in good]
    sums = up.advect_host_stream(good, 3, dt, out=out)
    for k in range(len(good)):
        assert np.array_equal(out[k], ref[k]), k
    assert np.array_equal(sums, ref_sums)
    up.close()
