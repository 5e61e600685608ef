"""The torch.autograd.Function over advect/adjoint: torch's gradcheck on a
tiny grid (f0 and the velocity), and a small gradient-descent recovery whose
first gradient agrees with a central difference."""
from __future__ import annotations

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
