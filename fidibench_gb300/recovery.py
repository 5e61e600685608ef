"""Initial-field recovery by gradient descent through the differentiable
batched advect (fidibench_gb300.autograd.batch_advect_fn), for many
independent instances at once.

For each instance: f_true = a sphere indicator, data = advect(f_true); start
from f0 = 0 and take `iters` steps f0 <- f0 - lr * dL/df0 on
L = sum over instances of 0.5 ||advect(f0) - data||^2, the gradient coming
from torch.autograd through BatchAdvect (forward: the batch's persistent
advect; backward: the transposed problems, fdb_batch_advect_transposed, all
instances in every launch: the velocity is fixed, so only dL/df0 is needed).  The
loss is a sum of per-instance terms, so each instance's gradient is its own.
With sum_j a_j <= 1 the step operator is a contraction in the 2-norm, so
lr = 1 is a safe step.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .autograd import batch_advect_fn


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
    shapes = [(n, n, n)] * count
    vel = torch.tensor([sp["v"] for sp in specs], dtype=torch.float64)
    dts = [sp["dt"] for sp in specs]
    cells = n ** 3
    t0 = time.perf_counter()
    f_true = torch.cat([sphere_field(n, sp["center"], sp["radius"], device).view(-1)
                        for sp in specs])
    with torch.no_grad():
        data = batch_advect_fn(f_true, vel, shapes, steps, dts)
    f0 = torch.zeros_like(f_true, requires_grad=True)
    misfit0, fd_err = None, []
    it_s = []  # wall time of each iteration (the first carries the one-time setup)
    for it in range(iters):
        torch.cuda.synchronize(device)
        t_it = time.perf_counter()
        out = batch_advect_fn(f0, vel, shapes, steps, dts)
        per = 0.5 * ((out - data) ** 2).view(count, cells).sum(dim=1)
        if it == 0:
            misfit0 = per.detach().cpu().numpy()
        f0.grad = None
        per.sum().backward()
        if fd_check and it == 0:
            # central differences of every instance's (quadratic) loss along a
            # seeded direction: the loss is separable, so one pair of batched
            # forwards serves all instances
            g = torch.Generator(device=device)
            g.manual_seed(seed * 1000)
            dvec = torch.randn(f0.shape, generator=g, device=device, dtype=torch.float64)
            h = 1e-6
            with torch.no_grad():
                rp = batch_advect_fn(f0 + h * dvec, vel, shapes, steps, dts) - data
                rm = batch_advect_fn(f0 - h * dvec, vel, shapes, steps, dts) - data
                fd = ((rp - rm) * (rp + rm)).view(count, cells).sum(dim=1) / (4 * h)
                exact = (f0.grad * dvec).view(count, cells).sum(dim=1)
            fd_err = (torch.abs(fd - exact) / torch.clamp(torch.abs(exact), min=1e-300)).tolist()
        with torch.no_grad():
            f0 -= lr * f0.grad
        torch.cuda.synchronize(device)
        it_s.append(time.perf_counter() - t_it)
    with torch.no_grad():
        out = batch_advect_fn(f0, vel, shapes, steps, dts)
        misfit = (0.5 * ((out - data) ** 2).view(count, cells).sum(dim=1)).cpu().numpy()
        field_err = (torch.linalg.norm((f0 - f_true).view(count, cells), dim=1) /
                     torch.linalg.norm(f_true.view(count, cells), dim=1)).cpu().numpy()
    el = time.perf_counter() - t0
    rel = misfit / misfit0
    return {"instances": count, "n": n, "time_steps": steps, "iterations": iters,
            "seconds": el, "misfit_reduction_max": float(np.max(rel)), "misfit_reduction_median":
            float(np.median(rel)), "final_misfit_median": float(np.median(misfit)),
            "field_rel_err_median": float(np.median(field_err)),
            "grad_fd_rel_err_max": max(fd_err) if fd_err else None,
            "ms_per_gd_iteration": el / (count * iters) * 1e3,
            "ms_per_gd_iteration_steady": (float(np.median(it_s[1:])) if len(it_s) > 1
                                           else it_s[0]) / count * 1e3,
            "mode": "all instances per launch (batched advect, batched transposed advect)"}


__all__ = ["recover", "instance_specs", "sphere_field"]
