"""torch.autograd.Function over the upwind advection (forward: advect();
backward: the hand-written adjoint behind fdb_upwind_adjoint).

    f_T = advect_fn(f0, velocity, num_steps, dt, lengths)

f0 is a CUDA float64 tensor whose shape is the grid (row-major, last axis
fastest, as in upwind/cxx/upwind.cxx:39-44); velocity is a float64 tensor of
ndims values.  Gradients flow to both: dL/df0 from the transposed steps and
dL/dv from the per-step coefficient contractions (the upwind direction is
piecewise constant in v, so dv is the derivative within the sign pattern).
torch supplies only device memory and the autograd graph; every step runs in
libfdb_upwind.
"""
from __future__ import annotations

import threading

import numpy as np
import torch

from .upwind import Upwind

_cache_lock = threading.Lock()
_handles: dict = {}


def _handle(shape, lengths, velocity, device) -> Upwind:
    key = (tuple(shape), tuple(float(x) for x in lengths), str(device))
    with _cache_lock:
        up = _handles.get(key)
        if up is None:
            with torch.cuda.device(device):
                up = Upwind(velocity, lengths, shape)
            _handles[key] = up
    up.set_velocity(velocity)
    return up


def release_handles() -> None:
    """Free the cached per-shape handles (device memory)."""
    with _cache_lock:
        for up in _handles.values():
            up.close()
        _handles.clear()


class UpwindAdvect(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, velocity, num_steps: int, dt: float, lengths, checkpoint_every: int = 0):
        if not f0.is_cuda or f0.dtype != torch.float64:
            raise TypeError("f0 must be a CUDA float64 tensor")
        v = velocity.detach().to("cpu", torch.float64).numpy().copy()
        up = _handle(f0.shape, lengths, v, f0.device)
        torch.cuda.current_stream(f0.device).synchronize()
        up.set_field(f0.contiguous())
        up.advect(int(num_steps), float(dt))
        out = torch.empty_like(f0, memory_format=torch.contiguous_format)
        up.get_field(out)
        ctx.save_for_backward(f0.detach().contiguous(), velocity.detach())
        ctx.meta = (int(num_steps), float(dt), tuple(float(x) for x in lengths),
                    int(checkpoint_every))
        return out

    @staticmethod
    def backward(ctx, grad_out):
        f0, velocity = ctx.saved_tensors
        num_steps, dt, lengths, ck = ctx.meta
        v = velocity.to("cpu", torch.float64).numpy().copy()
        up = _handle(f0.shape, lengths, v, f0.device)
        torch.cuda.current_stream(f0.device).synchronize()
        up.set_field(f0)
        lam = grad_out.detach().to(torch.float64).contiguous().view(-1)
        g0 = torch.empty(f0.numel(), dtype=torch.float64, device=f0.device)
        g0, gv = up.adjoint(num_steps, dt, lam, g0, checkpoint_every=ck)
        grad_v = torch.as_tensor(np.asarray(gv), dtype=velocity.dtype, device=velocity.device)
        return g0.view_as(f0), grad_v, None, None, None, None


def advect_fn(f0, velocity, num_steps: int, dt: float, lengths=None, checkpoint_every: int = 0):
    """Differentiable advect: returns f after num_steps steps of size dt."""
    if lengths is None:
        lengths = (1.0,) * f0.dim()
    if not torch.is_tensor(velocity):
        velocity = torch.tensor(velocity, dtype=torch.float64)
    return UpwindAdvect.apply(f0, velocity, num_steps, dt, tuple(lengths), checkpoint_every)


__all__ = ["UpwindAdvect", "advect_fn", "release_handles"]
