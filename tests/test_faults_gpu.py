"""Failure paths on the GPU without faulting it: host-side injection at the
allocation and launch sites (FDB_FAULT), non-finite input data reported by
the fixed-point kernel's error word, and a usable context afterwards."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_injected_allocation_failure(fdb, monkeypatch):
    monkeypatch.setenv("FDB_FAULT", "alloc")
    with pytest.raises(fdb.FdbError) as ei:
        fdb.Upwind((1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (8, 8, 8))
    assert ei.value.code == 7
    monkeypatch.delenv("FDB_FAULT")
    up = fdb.Upwind((1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (8, 8, 8))
    assert up.checksum() == 1.0
    up.close()


@pytest.mark.parametrize("arith", ["exact", "fixed"])
def test_injected_launch_failure(fdb, monkeypatch, arith):
    up = fdb.Upwind((1.0, -1.0, 0.5), (1.0, 1.0, 1.0), (16, 16, 16), arith=arith)
    monkeypatch.setenv("FDB_FAULT", "launch")
    with pytest.raises(fdb.FdbError) as ei:
        up.advect(5, 0.01)
    assert ei.value.code == 7
    monkeypatch.delenv("FDB_FAULT")
    up.advect(5, 0.01)
    assert np.isfinite(up.checksum())
    up.close()


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_field_is_reported_by_fixed_path(fdb, bad):
    n = (64, 64, 64)
    up = fdb.Upwind((1.0, -0.7, 0.3), (1.0, 1.0, 1.0), n, arith="fixed")
    f = np.random.default_rng(0).random(int(np.prod(n)))
    f[12345] = bad
    up.f = f
    up.advect(8, 0.5 / 64)
    with pytest.raises(fdb.FdbError) as ei:
        up.checksum()
    assert ei.value.code == 6
    up.f = np.ones(int(np.prod(n)))  # the handle stays usable
    up.advect(8, 0.5 / 64)
    assert up.checksum() == pytest.approx(float(np.prod(n)), rel=1e-12)
    up.close()


def test_nonfinite_field_propagates_in_fp64_path(fdb):
    """The FP64 arithmetics behave like the reference: NaN spreads, no error."""
    up = fdb.Upwind((1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (8, 8, 8), arith="exact")
    f = np.zeros(512)
    f[3] = np.nan
    up.f = f
    up.advect(2, 0.01)
    assert np.isnan(up.checksum())
    up.close()


def test_injected_failures_in_closed_form_adjoint(fdb, monkeypatch):
    """Allocation and launch failures inside the closed-form adjoint are
    reported, and the handle then gives the gradients of a fresh one."""
    n, L, v = (16, 18, 20), (1.0, 1.0, 1.0), (0.5, -0.4, 0.3)
    rng = np.random.default_rng(41)
    x = rng.standard_normal(int(np.prod(n)))
    lam = rng.standard_normal(x.size)
    ref = fdb.Upwind(v, L, n)
    ref.f = x
    g_ref, gv_ref = ref.adjoint(9, 0.01, lam)
    ref.close()
    up = fdb.Upwind(v, L, n)
    for kind in ("alloc", "launch"):
        up.f = x
        monkeypatch.setenv("FDB_FAULT", kind)
        with pytest.raises(fdb.FdbError) as ei:
            up.adjoint(9, 0.01, lam)
        assert ei.value.code == 7
        monkeypatch.delenv("FDB_FAULT")
    up.f = x
    g, gv = up.adjoint(9, 0.01, lam)
    assert np.array_equal(g, g_ref) and np.array_equal(gv, gv_ref)
    up.close()


def test_injected_failures_in_host_stream(fdb, monkeypatch):
    """A failed streamed cycle leaves the handle's three buffers consistent:
    the next call gives the serial results."""
    n, L, v = (16, 18, 20), (1.0, 1.0, 1.0), (0.5, -0.4, 0.3)
    rng = np.random.default_rng(42)
    fields = [rng.standard_normal(int(np.prod(n))) for _ in range(3)]
    up = fdb.Upwind(v, L, n)
    for kind in ("alloc", "launch"):
        monkeypatch.setenv("FDB_FAULT", kind)
        with pytest.raises(fdb.FdbError) as ei:
            up.advect_host_stream(fields, 5, 0.01, out=[np.empty_like(f) for f in fields])
        assert ei.value.code == 7
        monkeypatch.delenv("FDB_FAULT")
    out = [np.empty_like(f) for f in fields]
    sums = up.advect_host_stream(fields, 5, 0.01, out=out)
    for k, f in enumerate(fields):
        s = fdb.Upwind(v, L, n)
        s.f = f
        s.advect(5, 0.01)
        assert np.array_equal(out[k], s.f), k
        assert sums[k] == s.checksum(), k
        s.close()
    up.close()
