"""Initial-field recovery by gradient descent through the differentiable
advect (fidibench_gb300.autograd), for many independent instances.

For each instance: f_true = a sphere indicator, data = advect(f_true); start
from f0 = 0 and take `iters` steps f0 <- f0 - lr * dL/df0 on
L = 0.5 ||advect(f0) - data||^2, the gradient coming from
torch.autograd through UpwindAdvect (forward: the fixed-point advect;
backward: the fixed-point adjoint).  With sum_j a_j <= 1 the step operator
is a contraction in the 2-norm, so lr = 1 is a safe step.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .autograd import advect_fn


def instance_specs(count: int, n: int, seed: int, courant_sum: float = 0.5):
    """Seeded velocities in [-1, 1]^3, dt = courant_sum * dx / sum_j |v_j|
    (so sum_j a_j = courant_sum), sphere centres in [0.3, 0.7]^3 and radii in
    [0.1, 0.25]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        v = rng.uniform(-1.0, 1.0, size=3)
        dt = courant_sum * (1.0 / n) / float(np.sum(np.abs(v)))
        out.append({"v": tuple(float(x) for x in v), "dt": dt,
                    "center": tuple(float(x) for x in rng.uniform(0.3, 0.7, size=3)),
                    "radius": float(rng.uniform(0.1, 0.25))})
    return out


def sphere_field(n: int, center, radius: float, device) -> torch.Tensor:
    ax = (torch.arange(n, device=device, dtype=torch.float64) + 0.5) / n
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    r2 = (z - center[0]) ** 2 + (y - center[1]) ** 2 + (x - center[2]) ** 2
    return (r2 < radius * radius).to(torch.float64)


def recover(count: int = 64, n: int = 128, steps: int = 100, iters: int = 20, seed: int = 1,
            lr: float = 1.0, fd_check: bool = True, device=None) -> dict:
    device = device or torch.device("cuda", torch.cuda.current_device())
    specs = instance_specs(count, n, seed)
    misfit0, misfit, field_err, fd_err = [], [], [], []
    t0 = time.perf_counter()
    for k, sp in enumerate(specs):
        v = torch.tensor(sp["v"], dtype=torch.float64)
        f_true = sphere_field(n, sp["center"], sp["radius"], device)
        with torch.no_grad():
            data = advect_fn(f_true, v, steps, sp["dt"])
        f0 = torch.zeros_like(f_true, requires_grad=True)
        for it in range(iters):
            out = advect_fn(f0, v, steps, sp["dt"])
            loss = 0.5 * torch.sum((out - data) ** 2)
            if it == 0:
                misfit0.append(float(loss.item()))
            f0.grad = None
            loss.backward()
            if fd_check and it == 0:
                # central difference of the (quadratic) loss along a seeded direction
                g = torch.Generator(device=device)
                g.manual_seed(seed * 1000 + k)
                dvec = torch.randn(f0.shape, generator=g, device=device, dtype=torch.float64)
                h = 1e-6
                with torch.no_grad():
                    rp = advect_fn(f0 + h * dvec, v, steps, sp["dt"]) - data
                    rm = advect_fn(f0 - h * dvec, v, steps, sp["dt"]) - data
                    fd = float(torch.sum((rp - rm) * (rp + rm)).item()) / (4 * h)
                    exact = float(torch.sum(f0.grad * dvec).item())
                fd_err.append(abs(fd - exact) / max(abs(exact), 1e-300))
            with torch.no_grad():
                f0 -= lr * f0.grad
        with torch.no_grad():
            out = advect_fn(f0, v, steps, sp["dt"])
            misfit.append(float(0.5 * torch.sum((out - data) ** 2).item()))
            field_err.append(float(torch.linalg.norm(f0 - f_true) / torch.linalg.norm(f_true)))
    el = time.perf_counter() - t0
    rel = [m / m0 for m, m0 in zip(misfit, misfit0)]
    return {"instances": count, "n": n, "time_steps": steps, "iterations": iters,
            "seconds": el, "misfit_reduction_max": max(rel), "misfit_reduction_median":
            float(np.median(rel)), "final_misfit_median": float(np.median(misfit)),
            "field_rel_err_median": float(np.median(field_err)),
            "grad_fd_rel_err_max": max(fd_err) if fd_err else None,
            "ms_per_gd_iteration": el / (count * iters) * 1e3}


__all__ = ["recover", "instance_specs", "sphere_field"]
