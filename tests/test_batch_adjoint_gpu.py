"""Batched adjoint (fdb_batch_adjoint): every instance against the single-field
adjoint (fdb_upwind_adjoint), the fields left at f_T, device and host
buffers, and the dot-product identity per instance."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

# uneven instances: permuted storage (40 x 33 x 200), cubes, a 2-D and a 1-D one
SPECS = [
    {"n": (40, 33, 200), "v": (0.7, -0.4, 0.9), "L": (1.0, 2.0, 3.0)},
    {"n": (64, 64, 64), "v": (-0.3, 0.5, 0.2), "L": (1.0, 1.0, 1.0)},
    {"n": (21, 35, 48), "v": (0.2, 0.9, -0.6), "L": (1.0, 1.0, 1.0)},
    {"n": (33, 90), "v": (0.6, -0.8), "L": (1.0, 1.0)},
    {"n": (300,), "v": (-0.5,), "L": (1.0,)},
]


def _dts(specs, cfl=0.3):
    return [cfl * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(s["L"], s["n"], s["v"]))
            for s in specs]


def _batch(fdb, specs, fields):
    b = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    for k, f in enumerate(fields):
        b.set_field(k, f)
    return b


def test_batch_adjoint_matches_single_field(fdb):
    rng = np.random.default_rng(31)
    dts = _dts(SPECS)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in SPECS]
    lam = [rng.standard_normal(x.size) for x in f0]
    steps, ck = 23, 5
    b = _batch(fdb, SPECS, f0)
    b.set_tuning(depth=4)
    g0, gv = b.adjoint(steps, dts, np.concatenate(lam), checkpoint_every=ck)
    off = np.cumsum([0] + [x.size for x in f0])
    for k, s in enumerate(SPECS):
        up = fdb.Upwind(s["v"], s["L"], s["n"], depth=4)
        up.f = f0[k]
        g_ref, gv_ref = up.adjoint(steps, dts[k], lam[k], checkpoint_every=ck)
        # the transposed steps are integer arithmetic: identical whatever the
        # tiling or the stored axis order
        assert np.array_equal(g0[off[k]:off[k + 1]], g_ref), k
        # dL/dv: the same closed-form contraction, summed in the stored axis
        # order (permuted for the first instance), so equal to rounding
        nd = len(s["n"])
        assert np.allclose(gv[k, :nd], gv_ref, rtol=1e-8, atol=1e-8 * np.abs(gv_ref).max()), k
        assert np.all(gv[k, nd:] == 0.0)
        # the batch is left at f_T, as the single-field handle
        assert np.array_equal(b.get_field(k), up.f), k
        up.close()
    b.close()


def test_batch_adjoint_device_buffers(fdb):
    import torch
    specs = SPECS[1:4]
    rng = np.random.default_rng(32)
    dts = _dts(specs)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    lam = np.concatenate([rng.standard_normal(x.size) for x in f0])
    b = _batch(fdb, specs, f0)
    g_host, gv_host = b.adjoint(9, dts, lam)
    for k in range(len(specs)):
        b.set_field(k, f0[k])
    g_dev, gv_dev = b.adjoint(9, dts, torch.tensor(lam, device="cuda"))
    assert np.array_equal(g_dev.cpu().numpy(), g_host)
    assert np.array_equal(gv_dev, gv_host)
    b.close()


def test_batch_dot_product_identity(fdb):
    """<A x, y> = <x, A^T y> for every instance of one batch."""
    rng = np.random.default_rng(33)
    dts = _dts(SPECS, cfl=0.45)
    x = [rng.standard_normal(int(np.prod(s["n"]))) for s in SPECS]
    y = [rng.standard_normal(v.size) for v in x]
    b = _batch(fdb, SPECS, x)
    b.advect(17, dts)
    ax = [b.get_field(k) for k in range(len(SPECS))]
    for k in range(len(SPECS)):
        b.set_field(k, x[k])
    aty, _ = b.adjoint(17, dts, np.concatenate(y), checkpoint_every=4)
    off = np.cumsum([0] + [v.size for v in x])
    for k in range(len(SPECS)):
        lhs = float(ax[k] @ y[k])
        rhs = float(x[k] @ aty[off[k]:off[k + 1]])
        assert lhs == pytest.approx(rhs, rel=1e-11), k
    b.close()


def test_batch_adjoint_velocity_finite_differences(fdb):
    """dL/dv of L = 0.5 ||f_T - target||^2 against central differences of the
    batched forward (h = 1e-6), for every instance and axis."""
    specs = SPECS[1:]
    rng = np.random.default_rng(34)
    dts = _dts(specs)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    target = [rng.standard_normal(x.size) for x in f0]
    steps = 12

    def forward(vel):
        bb = fdb.Batch([(v, s["L"], s["n"]) for v, s in zip(vel, specs)])
        for k, f in enumerate(f0):
            bb.set_field(k, f)
        bb.advect(steps, dts)
        out = [bb.get_field(k) for k in range(len(specs))]
        bb.close()
        return out

    b = _batch(fdb, specs, f0)
    b.advect(steps, dts)
    lam = np.concatenate([b.get_field(k) - target[k] for k in range(len(specs))])
    for k, f in enumerate(f0):
        b.set_field(k, f)
    _, gv = b.adjoint(steps, dts, lam)
    b.close()
    h = 1e-6
    for k, s in enumerate(specs):
        for j in range(len(s["n"])):
            vp = [list(t["v"]) for t in specs]
            vm = [list(t["v"]) for t in specs]
            vp[k][j] += h
            vm[k][j] -= h
            fp, fm = forward(vp)[k], forward(vm)[k]
            rp, rm = fp - target[k], fm - target[k]
            fd = float(np.sum((rp - rm) * (rp + rm))) / (4.0 * h)
            assert gv[k, j] == pytest.approx(fd, rel=1e-6), (k, j)


@pytest.mark.parametrize("form", ["closed", "stepwise"])
@pytest.mark.parametrize("steps,ck", [(0, 0), (1, 0), (6, 1), (5, 9), (11, 4)])
def test_batch_adjoint_step_and_checkpoint_counts(fdb, steps, ck, form):
    """Batch against single field at equal depth (the closed form's
    transposed runs are blocked like the forward), both adjoint forms."""
    specs = SPECS[1:4]
    rng = np.random.default_rng(35)
    dts = _dts(specs)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    lam = [rng.standard_normal(x.size) for x in f0]
    b = _batch(fdb, specs, f0)
    b.set_tuning(depth=4)
    b.set_adjoint_form(form)
    g0, gv = b.adjoint(steps, dts, np.concatenate(lam), checkpoint_every=ck)
    off = np.cumsum([0] + [x.size for x in f0])
    for k, s in enumerate(specs):
        up = fdb.Upwind(s["v"], s["L"], s["n"], depth=4)
        up.set_adjoint_form(form)
        up.f = f0[k]
        g_ref, gv_ref = up.adjoint(steps, dts[k], lam[k], checkpoint_every=ck)
        assert np.array_equal(g0[off[k]:off[k + 1]], g_ref), k
        nd = len(s["n"])
        assert np.allclose(gv[k, :nd], gv_ref, rtol=1e-8,
                           atol=1e-8 * max(np.abs(gv_ref).max(), 1e-300)), k
        up.close()
    b.close()


def test_batch_adjoint_rejects_bad_input(fdb):
    from fidibench_gb300._capi import FdbError
    specs = SPECS[1:3]
    b = _batch(fdb, specs, [np.ones(int(np.prod(s["n"]))) for s in specs])
    total = sum(b.sizes)
    with pytest.raises(ValueError):
        b.adjoint(3, _dts(specs), np.zeros(total - 1))
    # a Courant number above 1 is outside the fixed kernel's domain
    bad = _dts(specs)
    bad[1] *= 10.0
    with pytest.raises(FdbError):
        b.adjoint(3, bad, np.zeros(total))
    b.close()


def test_batch_set_velocity(fdb):
    """After set_velocity the batch advects the new problem."""
    specs = SPECS[:2]
    rng = np.random.default_rng(36)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    b = _batch(fdb, specs, f0)
    v_new = (-0.6, 0.35, 0.8)
    b.set_velocity(0, v_new)
    moved = [dict(specs[0], v=v_new), specs[1]]
    dts = _dts(moved)
    b.advect(8, dts)
    for k, s in enumerate(moved):
        up = fdb.Upwind(s["v"], s["L"], s["n"])
        up.f = f0[k]
        up.advect(8, dts[k])
        assert rel_maxnorm(b.get_field(k), up.f) <= 1e-13, k
        up.close()
    b.close()


def test_batch_f0_only_adjoint(fdb):
    """velocity_grad=False on a batch: the persistent launch on the
    transposed problems agrees with the full batched adjoint and leaves the
    fields at f_T."""
    rng = np.random.default_rng(37)
    dts = _dts(SPECS)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in SPECS]
    lam = np.concatenate([rng.standard_normal(x.size) for x in f0])
    b = _batch(fdb, SPECS, f0)
    b.advect(19, dts)
    ft = [b.get_field(k) for k in range(len(SPECS))]  # one advect call, as the fast path
    for k, f in enumerate(f0):
        b.set_field(k, f)
    g_full, _ = b.adjoint(19, dts, lam, checkpoint_every=6)
    for k, f in enumerate(f0):
        b.set_field(k, f)
    g_fast, gv = b.adjoint(19, dts, lam, velocity_grad=False)
    assert gv is None
    off = np.cumsum([0] + [x.size for x in f0])
    for k in range(len(SPECS)):
        assert rel_maxnorm(g_fast[off[k]:off[k + 1]], g_full[off[k]:off[k + 1]]) <= 1e-13, k
        assert np.array_equal(b.get_field(k), ft[k]), k
    b.close()


def test_batch_advect_transposed(fdb):
    """fdb_batch_advect_transposed: the grad_f0 of the dL/df0-only batched
    adjoint bit for bit, the fields untouched, each instance within rounding
    of the single-field transposed advect, device buffers in place."""
    import torch
    rng = np.random.default_rng(38)
    dts = _dts(SPECS)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in SPECS]
    lam = np.concatenate([rng.standard_normal(x.size) for x in f0])
    b = _batch(fdb, SPECS, f0)
    aty = b.advect_transposed(19, dts, lam)
    for k in range(len(SPECS)):
        assert np.array_equal(b.get_field(k), f0[k]), k
    g_fast, _ = b.adjoint(19, dts, lam, velocity_grad=False)
    assert np.array_equal(aty, g_fast)
    off = np.cumsum([0] + [x.size for x in f0])
    for k, s in enumerate(SPECS):
        up = fdb.Upwind(s["v"], s["L"], s["n"])
        ref = up.advect_transposed(19, dts[k], lam[off[k]:off[k + 1]])
        assert rel_maxnorm(aty[off[k]:off[k + 1]], ref) <= 1e-13, k
        up.close()
    t = torch.tensor(lam, device="cuda")
    b.advect_transposed(19, dts, t, t)
    assert np.array_equal(t.cpu().numpy(), aty)
    with pytest.raises(ValueError):
        b.advect_transposed(3, dts, lam[:-1])
    b.close()


def test_batch_closed_form_matches_stepwise(fdb):
    """The batched closed form (dL/da_j = S <lam^1, D_j f0> per instance)
    against the batched step-by-step adjoint, on the uneven instances
    (permuted storage included), and the fields left at f_T either way."""
    rng = np.random.default_rng(39)
    dts = _dts(SPECS)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in SPECS]
    lam = np.concatenate([rng.standard_normal(x.size) for x in f0])
    res = {}
    for form in ("closed", "stepwise"):
        b = _batch(fdb, SPECS, f0)
        b.set_adjoint_form(form)
        g0, gv = b.adjoint(21, dts, lam, checkpoint_every=6)
        res[form] = (g0, gv, [b.get_field(k) for k in range(len(SPECS))])
        b.close()
    g_c, gv_c, f_c = res["closed"]
    g_s, gv_s, f_s = res["stepwise"]
    off = np.cumsum([0] + [x.size for x in f0])
    for k, s in enumerate(SPECS):
        assert rel_maxnorm(g_c[off[k]:off[k + 1]], g_s[off[k]:off[k + 1]]) <= 1e-13, k
        nd = len(s["n"])
        assert np.allclose(gv_c[k, :nd], gv_s[k, :nd], rtol=1e-8,
                           atol=1e-8 * np.abs(gv_s[k]).max()), k
        # the step-by-step forward runs segment by segment: f_T to rounding
        assert rel_maxnorm(f_c[k], f_s[k]) <= 1e-13, k

