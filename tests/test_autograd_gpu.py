"""The torch.autograd.Functions over advect/adjoint (single field and
batched): torch's gradcheck on tiny grids (f0 and the velocity), the batched
forward against the single-field one, and a small gradient-descent recovery
whose first gradient agrees with a central difference."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gradcheck_f0_and_velocity(fdb):
    import torch
    from fidibench_gb300.autograd import UpwindAdvect
    f0 = torch.rand((3, 4, 5), dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor([0.6, -0.4, 0.3], dtype=torch.float64, requires_grad=True)
    fn = lambda f, vel: UpwindAdvect.apply(f, vel, 3, 0.05, (1.0, 1.0, 1.0), 0)  # noqa: E731
    assert torch.autograd.gradcheck(fn, (f0, v), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_advect_fn_matches_plain_advect(fdb):
    import torch
    from fidibench_gb300.autograd import advect_fn
    n = (12, 10, 14)
    f0 = torch.rand(n, dtype=torch.float64, device="cuda")
    out = advect_fn(f0, (0.5, -0.5, 0.25), 7, 0.02)
    up = fdb.Upwind((0.5, -0.5, 0.25), (1.0, 1.0, 1.0), n)
    up.set_field(f0)
    up.advect(7, 0.02)
    assert torch.equal(out.reshape(-1).cpu(), torch.tensor(up.f))
    up.close()


def test_small_recovery_decreases_misfit(fdb):
    from fidibench_gb300.recovery import recover
    r = recover(count=3, n=16, steps=10, iters=6, seed=3)
    assert r["misfit_reduction_max"] < 0.5
    assert r["grad_fd_rel_err_max"] < 1e-6


def test_gradcheck_batched(fdb):
    """BatchAdvect (forward: the batch's advect; backward: fdb_batch_adjoint)
    on two tiny instances of different shapes, w.r.t. the concatenated f0 and
    the (count, 3) velocity rows (the padded entry of the 2-D instance has no
    effect and a zero gradient)."""
    import torch
    from fidibench_gb300.autograd import BatchAdvect
    shapes = ((3, 4, 5), (4, 3))
    lengths = ((1.0, 1.0, 1.0), (1.0, 2.0))
    f0 = torch.rand(60 + 12, dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor([[0.6, -0.4, 0.3], [-0.5, 0.7, 0.0]], dtype=torch.float64,
                     requires_grad=True)
    fn = lambda f, vel: BatchAdvect.apply(f, vel, shapes, lengths, 3, (0.05, 0.04), 0)  # noqa: E731
    assert torch.autograd.gradcheck(fn, (f0, v), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_batch_advect_fn_matches_single_field(fdb):
    import torch
    from fidibench_gb300.autograd import advect_fn, batch_advect_fn
    shapes = [(12, 10, 14), (9, 17), (30,)]
    vels = [(0.5, -0.5, 0.25), (0.3, 0.8), (-0.9,)]
    dts = [0.02, 0.015, 0.01]
    fs = [torch.rand(int(np.prod(n)), dtype=torch.float64, device="cuda") for n in shapes]
    out = batch_advect_fn(torch.cat(fs), vels, shapes, 7, dts)
    off = 0
    for f, n, v, dt in zip(fs, shapes, vels, dts):
        ref = advect_fn(f.view(n), v, 7, dt).reshape(-1)
        got = out[off:off + f.numel()]
        assert torch.max(torch.abs(got - ref)) <= 1e-13 * torch.max(torch.abs(ref))
        off += f.numel()


def test_gradcheck_f0_only(fdb):
    """With the velocity not requiring grad, both Functions take dL/df0 from
    the transposed problem alone; torch's gradcheck still holds."""
    import torch
    from fidibench_gb300.autograd import BatchAdvect, UpwindAdvect
    f0 = torch.rand((3, 4, 5), dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor([0.6, -0.4, 0.3], dtype=torch.float64)
    fn = lambda f: UpwindAdvect.apply(f, v, 3, 0.05, (1.0, 1.0, 1.0), 0)  # noqa: E731
    assert torch.autograd.gradcheck(fn, (f0,), eps=1e-6, atol=1e-8, rtol=1e-6)
    shapes = ((3, 4, 5), (4, 3))
    lengths = ((1.0, 1.0, 1.0), (1.0, 2.0))
    fb = torch.rand(72, dtype=torch.float64, device="cuda", requires_grad=True)
    vb = torch.tensor([[0.6, -0.4, 0.3], [-0.5, 0.7, 0.0]], dtype=torch.float64)
    fnb = lambda f: BatchAdvect.apply(f, vb, shapes, lengths, 3, (0.05, 0.04), 0)  # noqa: E731
    assert torch.autograd.gradcheck(fnb, (fb,), eps=1e-6, atol=1e-8, rtol=1e-6)
