"""Adjoint (transposed step + checkpoint/recompute) through the C-ABI:
agreement with the oracle's transposed step, the dot-product identity
<A x, y> = <x, A^T y>, and central finite differences (h = 1e-6) of
L = 0.5 ||f_T - target||^2 with respect to f0 and the velocity."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

FD_TOL = 1e-6


def test_adjoint_step_matches_oracle(fdb, port):
    import torch
    n, L = (9, 10, 11), (1.0, 1.0, 1.0)
    rng = np.random.default_rng(2)
    for v in [(1.0, -0.7, 0.3), (-0.5, 0.5, -0.5), (0.2, 0.0, 1.0)]:
        dt = 0.4 / 11
        f = rng.standard_normal(990)
        lam = rng.standard_normal(990)
        ref_lam, ref_dc = port.adjoint_step(n, v, L, dt, f, lam)
        up = fdb.Upwind(v, L, n)
        fd = torch.tensor(f, device="cuda")
        ld = torch.tensor(lam, device="cuda")
        out = torch.empty_like(ld)
        dc = np.zeros(3)
        from fidibench_gb300._capi import check, lib
        check(lib.fdb_upwind_adjoint_step(up._h, dt, fd.data_ptr(), ld.data_ptr(),
                                          out.data_ptr(), dc.ctypes.data))
        assert rel_maxnorm(out.cpu().numpy(), ref_lam) <= 1e-14
        assert np.allclose(dc, ref_dc, rtol=1e-12, atol=1e-12 * np.abs(ref_dc).max())
        up.close()


@pytest.mark.parametrize("v,ckpt", [((1.0, -0.7, 0.3), 0), ((0.8, 0.5, -0.6), 7),
                                    ((-0.3, -0.9, 0.6), 1), ((0.5, 0.5, 0.5), 50)])
def test_dot_product_identity(fdb, v, ckpt):
    n, L = (24, 20, 28), (1.0, 1.0, 1.0)
    steps = 37
    dt = 0.5 / 28
    rng = np.random.default_rng(4)
    x = rng.standard_normal(int(np.prod(n)))
    y = rng.standard_normal(int(np.prod(n)))
    up = fdb.Upwind(v, L, n)
    up.f = x
    up.advect(steps, dt)
    ax = up.f
    up.f = x
    aty, _ = up.adjoint(steps, dt, y, checkpoint_every=ckpt)
    assert np.allclose(up.f, ax, rtol=0, atol=1e-13 * np.abs(ax).max())
    lhs, rhs = float(ax @ y), float(x @ aty)
    assert lhs == pytest.approx(rhs, rel=1e-11)
    up.close()


def _fd_diff(fp, fm, target, h):
    rp, rm = fp - target, fm - target
    return float(np.sum((rp - rm) * (rp + rm))) / (4.0 * h)


def _forward(fdb, v, L, n, f0, steps, dt, arith="fma"):
    up = fdb.Upwind(v, L, n, arith=arith)
    up.f = f0
    up.advect(steps, dt)
    out = up.f
    up.close()
    return out


@pytest.mark.parametrize("form", ["closed", "stepwise"])
@pytest.mark.parametrize("arith", ["fma", "fixed"])
def test_finite_differences(fdb, port, arith, form):
    """FP64 adjoint (arith fma) and the fixed-point adjoint (arith fixed, the
    default), dL/dv in closed form and step by step, against central
    differences of the same forward arithmetic."""
    n, L = (32, 24, 40), (1.0, 1.0, 1.0)
    v = np.array([0.8, 0.5, -0.6])
    steps, dt = 60, 0.5 / 40
    rng = np.random.default_rng(8)
    f0 = port.sphere_noise(n, L, (0.5, 0.5, 0.5), 0.25, 0.01, 1)
    target = rng.standard_normal(f0.size)
    up = fdb.Upwind(v, L, n, arith=arith)
    up.set_adjoint_form(form)
    up.f = f0
    up.advect(steps, dt)
    lam = up.f - target
    up.f = f0
    g0, gv = up.adjoint(steps, dt, lam, checkpoint_every=20)
    t = up.adjoint_timings()
    assert t["forward_ms"] > 0 and t["adjoint_ms"] > 0
    up.close()
    h = 1e-6
    for k in range(4):
        d = rng.standard_normal(f0.size)
        fd = _fd_diff(_forward(fdb, v, L, n, f0 + h * d, steps, dt, arith),
                      _forward(fdb, v, L, n, f0 - h * d, steps, dt, arith), target, h)
        assert float(g0 @ d) == pytest.approx(fd, rel=FD_TOL)
    for j in range(3):
        vp, vm = v.copy(), v.copy()
        vp[j] += h
        vm[j] -= h
        fd = _fd_diff(_forward(fdb, vp, L, n, f0, steps, dt, arith),
                      _forward(fdb, vm, L, n, f0, steps, dt, arith), target, h)
        assert gv[j] == pytest.approx(fd, rel=FD_TOL)


@pytest.mark.parametrize("form", ["closed", "stepwise"])
@pytest.mark.parametrize("v", [(1.0, -0.7, 0.3), (-0.3, -0.9, 0.6), (0.5, 0.0, -0.5)])
def test_fixed_adjoint_matches_fp64_adjoint(fdb, v, form):
    """The two adjoint arithmetics agree: dL/df0 to 1e-12 of max|grad|; the
    velocity gradients to 1e-8, since the fixed-point contraction reads each
    forward state in 2^29 units (2^-30 of the fixed-point range), an
    error that for random fields is below 1e-9 of the contraction."""
    n, L = (20, 28, 36), (1.0, 1.0, 1.0)
    steps, dt = 45, 0.45 / 36
    rng = np.random.default_rng(9)
    x = rng.standard_normal(int(np.prod(n)))
    lam = rng.standard_normal(x.size)
    out = {}
    for arith in ("fma", "fixed"):
        up = fdb.Upwind(v, L, n, arith=arith)
        up.set_adjoint_form(form)
        up.f = x
        out[arith] = up.adjoint(steps, dt, lam, checkpoint_every=10)
        up.close()
    g_fma, gv_fma = out["fma"]
    g_fix, gv_fix = out["fixed"]
    assert rel_maxnorm(g_fix, g_fma) <= 1e-12
    assert np.allclose(gv_fix, gv_fma, rtol=1e-8, atol=1e-8 * np.abs(gv_fma).max())


def test_adjoint_device_buffers(fdb):
    import torch
    n, L, v = (16, 16, 16), (1.0, 1.0, 1.0), (0.3, -0.6, 0.9)
    up = fdb.Upwind(v, L, n)
    x = torch.rand(4096, dtype=torch.float64, device="cuda")
    lam = torch.rand(4096, dtype=torch.float64, device="cuda")
    up.set_field(x)
    g_dev, gv_dev = up.adjoint(12, 0.02, lam)
    up.set_field(x)
    g_host, gv_host = up.adjoint(12, 0.02, lam.cpu().numpy())
    assert np.array_equal(g_dev.cpu().numpy(), g_host)
    assert np.array_equal(gv_dev, gv_host)
    up.close()


@pytest.mark.parametrize("arith", ["fixed", "fma"])
@pytest.mark.parametrize("v", [(1.0, -0.7, 0.3), (-0.3, -0.9, 0.6)])
def test_f0_only_adjoint_is_the_transposed_problem(fdb, arith, v):
    """velocity_grad=False: dL/df0 from the problem with every upwind
    direction reversed (no checkpoints) agrees with the full adjoint, leaves
    the field at f_T, and satisfies the dot-product identity."""
    n, L = (20, 28, 36), (1.0, 1.0, 1.0)
    steps, dt = 31, 0.45 / 36
    rng = np.random.default_rng(12)
    x = rng.standard_normal(int(np.prod(n)))
    y = rng.standard_normal(x.size)
    up = fdb.Upwind(v, L, n, arith=arith)
    up.f = x
    up.advect(steps, dt)
    ax = up.f  # one advect call, as the fast path runs it
    up.f = x
    g_full, _ = up.adjoint(steps, dt, y, checkpoint_every=7)
    up.f = x
    g_fast, gv = up.adjoint(steps, dt, y, velocity_grad=False)
    assert gv is None
    assert rel_maxnorm(g_fast, g_full) <= 1e-13
    assert np.array_equal(up.f, ax)
    assert float(ax @ y) == pytest.approx(float(x @ g_fast), rel=1e-11)
    up.close()


@pytest.mark.parametrize("arith", ["auto", "fma", "exact"])
def test_advect_transposed_leaves_the_field(fdb, port, arith):
    """fdb_upwind_advect_transposed: bit-identical to the grad_f0 of the
    dL/df0-only adjoint, the field and the next advect untouched, the
    oracle's transposed step applied S times, and in == out allowed."""
    n, L, v = (20, 28, 36), (1.0, 1.3, 0.8), (0.7, -0.5, 0.35)
    steps, dt = 17, 0.4 / 45
    rng = np.random.default_rng(13)
    x = rng.standard_normal(int(np.prod(n)))
    y = rng.standard_normal(x.size)
    up = fdb.Upwind(v, L, n, arith=arith)
    up.f = x
    up.advect(5, dt)
    f5 = up.f
    aty = up.advect_transposed(steps, dt, y)
    # the field is untouched and the next advect continues as without the call
    assert np.array_equal(up.f, f5)
    up.advect(6, dt)
    cont = up.f
    ref = fdb.Upwind(v, L, n, arith=arith)
    ref.f = x
    ref.advect(5, dt)
    ref.advect(6, dt)
    assert np.array_equal(cont, ref.f)
    # the same numbers as the adjoint's dL/df0-only path
    ref.f = x
    g_fast, _ = ref.adjoint(steps, dt, y, velocity_grad=False)
    assert np.array_equal(aty, g_fast)
    ref.close()
    # the oracle's transposed step, S times (FP64; the coefficient part is unused)
    lam = y.copy()
    for _ in range(steps):
        lam, _ = port.adjoint_step(n, v, L, dt, x, lam)
    assert rel_maxnorm(aty, lam) <= 1e-13
    # device buffers, in place
    import torch
    t = torch.tensor(y, device="cuda")
    up.advect_transposed(steps, dt, t, t)
    assert np.array_equal(t.cpu().numpy(), aty)
    up.close()


def test_advect_transposed_rejects_bad_input(fdb):
    from fidibench_gb300._capi import FdbError
    n, v = (12, 13, 14), (0.5, -0.4, 0.3)
    up = fdb.Upwind(v, (1.0,) * 3, n, arith="fixed")
    y = np.ones(int(np.prod(n)))
    with pytest.raises(ValueError):
        up.advect_transposed(3, 0.01, y[:-1])
    with pytest.raises(ValueError):
        up.advect_transposed(3, 0.01, y, out=np.empty(y.size, dtype=np.float32))
    bad = y.copy()
    bad[5] = np.inf
    with pytest.raises(FdbError) as e:
        up.advect_transposed(3, 0.01, bad)
    assert e.value.code == 6
    # still usable; zero steps is the identity
    assert np.array_equal(up.advect_transposed(0, 0.01, y), y)
    g4 = fdb.Upwind((0.1, 0.2, 0.3, 0.4), (1.0,) * 4, (3, 4, 5, 6))
    with pytest.raises(FdbError) as e:
        g4.advect_transposed(2, 0.01, np.ones(360))
    assert e.value.code == 4
    g4.close()
    up.close()


@pytest.mark.parametrize("arith", ["fixed", "fma"])
@pytest.mark.parametrize("n,v,cfl", [((20, 28, 36), (0.7, -0.5, 0.35), 0.4),
                                     ((24, 20, 28), (1.0, 1.0, 1.0), 0.5),  # sum a = 1.5 > 1
                                     ((18, 26, 30), (0.5, 0.0, -0.5), 0.45),
                                     ((33, 90), (0.6, -0.8), 0.4),
                                     ((300,), (-0.5,), 0.7)])
def test_closed_form_matches_stepwise(fdb, arith, n, v, cfl):
    """dL/da_j = S <lam^1, D_j f0>: the closed form against the step-by-step
    sum over every step (with checkpoints).  dL/dv to 1e-8 (the fixed-point
    step-by-step contraction reads each forward state in 2^29 units), dL/df0
    to rounding, and the field left at f_T exactly as advect() leaves it."""
    L = (1.0,) * len(n)
    dt = cfl * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(L, n, v) if vj != 0.0)
    steps = 23
    rng = np.random.default_rng(sum(n))
    x = rng.standard_normal(int(np.prod(n)))
    lam = rng.standard_normal(x.size)
    res = {}
    for form in ("closed", "stepwise"):
        up = fdb.Upwind(v, L, n, arith=arith)
        up.set_adjoint_form(form)
        up.f = x
        g0, gv = up.adjoint(steps, dt, lam, checkpoint_every=5)
        res[form] = (g0, gv, up.f)
        up.close()
    ref = fdb.Upwind(v, L, n, arith=arith)
    ref.f = x
    ref.advect(steps, dt)
    f_t = ref.f
    ref.close()
    g_c, gv_c, f_c = res["closed"]
    g_s, gv_s, _ = res["stepwise"]
    assert np.array_equal(f_c, f_t)
    assert rel_maxnorm(g_c, g_s) <= 1e-13
    tol = 1e-8 if arith == "fixed" else 1e-11
    assert np.allclose(gv_c, gv_s, rtol=tol, atol=tol * np.abs(gv_s).max())


def test_closed_form_step_counts(fdb):
    """S = 0 (identity, zero velocity gradient) and S = 1 (lam^1 = lam_T)."""
    n, L, v = (16, 18, 20), (1.0, 1.0, 1.0), (0.4, -0.3, 0.6)
    rng = np.random.default_rng(21)
    x = rng.standard_normal(int(np.prod(n)))
    lam = rng.standard_normal(x.size)
    up = fdb.Upwind(v, L, n)
    up.f = x
    g0, gv = up.adjoint(0, 0.01, lam)
    assert np.array_equal(g0, lam) and np.all(gv == 0.0)
    assert np.array_equal(up.f, x)
    g1, gv1 = up.adjoint(1, 0.01, lam)
    up.set_adjoint_form("stepwise")
    up.f = x
    g1s, gv1s = up.adjoint(1, 0.01, lam)
    assert rel_maxnorm(g1, g1s) <= 1e-13
    assert np.allclose(gv1, gv1s, rtol=1e-8, atol=1e-8 * np.abs(gv1s).max())
    from fidibench_gb300._capi import FdbError
    with pytest.raises(KeyError):
        up.set_adjoint_form("other")
    from fidibench_gb300._capi import check, lib
    with pytest.raises(FdbError):
        check(lib.fdb_upwind_set_tuning(up._h, 4, 3))
    up.close()


def test_closed_form_keeping_the_field(fdb):
    """Form "closed_keep": the closed form's gradients bit for bit, with the
    field left at f0 (single field and batch)."""
    n, L, v = (18, 22, 26), (1.0, 1.0, 1.0), (0.6, -0.4, 0.3)
    dt = 0.4 / 26
    rng = np.random.default_rng(22)
    x = rng.standard_normal(int(np.prod(n)))
    lam = rng.standard_normal(x.size)
    up = fdb.Upwind(v, L, n)
    up.f = x
    g_c, gv_c = up.adjoint(17, dt, lam)
    up.set_adjoint_form("closed_keep")
    up.f = x
    g_k, gv_k = up.adjoint(17, dt, lam)
    assert np.array_equal(g_k, g_c) and np.array_equal(gv_k, gv_c)
    assert np.array_equal(up.f, x)
    g_f, _ = up.adjoint(17, dt, lam, velocity_grad=False)
    assert np.array_equal(up.f, x)
    assert rel_maxnorm(g_f, g_c) <= 1e-13
    up.close()
    b = fdb.Batch([(v, L, n)])
    b.set_field(0, x)
    gb_c, gvb_c = b.adjoint(17, [dt], lam)
    b.set_adjoint_form("closed_keep")
    b.set_field(0, x)
    gb_k, gvb_k = b.adjoint(17, [dt], lam)
    assert np.array_equal(gb_k, gb_c) and np.array_equal(gvb_k, gvb_c)
    assert np.array_equal(b.get_field(0), x)
    b.close()

