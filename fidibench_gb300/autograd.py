"""torch.autograd.Function over the upwind advection (forward: advect();
backward: the hand-written adjoint behind fdb_upwind_adjoint).

    f_T = advect_fn(f0, velocity, num_steps, dt, lengths)

f0 is a CUDA float64 tensor whose shape is the grid (row-major, last axis
fastest, as in upwind/cxx/upwind.cxx:39-44); velocity is a float64 tensor of
ndims values.  Gradients flow to both: dL/df0 from the transposed steps and
dL/dv from the per-step coefficient contractions (the upwind direction is
piecewise constant in v, so dv is the derivative within the sign pattern).
When the velocity needs no gradient, the backward pass is the transposed
problem alone (fdb_upwind_advect_transposed): the forward is not re-run.
torch supplies only device memory and the autograd graph; every step runs in
libfdb_upwind.  batch_advect_fn does the same for many instances at once
(fdb_batch_advect forward, fdb_batch_adjoint backward).
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
        lam = grad_out.detach().to(torch.float64).contiguous().view(-1)
        g0 = torch.empty(f0.numel(), dtype=torch.float64, device=f0.device)
        if not ctx.needs_input_grad[1]:
            # without a velocity gradient dL/df0 = (A^T)^S lam alone: the
            # transposed problem, no re-run of the forward
            up.advect_transposed(num_steps, dt, lam, g0)
            return g0.view_as(f0), None, None, None, None, None
        up.set_field(f0)
        # the closed form with the field kept at f0: the forward already
        # produced f_T, so one transposed run and one contraction
        up.set_adjoint_form("closed_keep" if ck == 0 else "stepwise")
        g0, gv = up.adjoint(num_steps, dt, lam, g0, checkpoint_every=ck)
        grad_v = torch.as_tensor(np.asarray(gv), dtype=velocity.dtype, device=velocity.device)
        return g0.view_as(f0), grad_v, None, None, None, None


def advect_fn(f0, velocity, num_steps: int, dt: float, lengths=None, checkpoint_every: int = 0):
    """Differentiable advect: returns f after num_steps steps of size dt.
    The backward pass takes dL/dv in closed form (one transposed run and one
    contraction); checkpoint_every > 0 asks for the step-by-step adjoint with
    checkpoints at that spacing instead (the same gradient, to rounding)."""
    if lengths is None:
        lengths = (1.0,) * f0.dim()
    if not torch.is_tensor(velocity):
        velocity = torch.tensor(velocity, dtype=torch.float64)
    return UpwindAdvect.apply(f0, velocity, num_steps, dt, tuple(lengths), checkpoint_every)


# ---- many instances at once (fdb_batch_advect / fdb_batch_adjoint) -------------

_batches: dict = {}


def _batch_handle(shapes, lengths, velocity, device):
    from .batch import Batch
    key = (tuple(shapes), tuple(lengths), str(device))
    v = velocity.detach().to("cpu", torch.float64).numpy()
    with _cache_lock:
        entry = _batches.get(key)
        if entry is None:
            with torch.cuda.device(device):
                b = Batch([(v[k, :len(n)], L, n) for k, (n, L) in enumerate(zip(shapes, lengths))])
            entry = [b, v.copy()]
            _batches[key] = entry
    b, v_set = entry
    for k, n in enumerate(shapes):
        if not np.array_equal(v_set[k, :len(n)], v[k, :len(n)]):
            b.set_velocity(k, v[k, :len(n)])
            v_set[k, :len(n)] = v[k, :len(n)]
    return b


def release_batches() -> None:
    """Free the cached batches (device memory)."""
    with _cache_lock:
        for b, _ in _batches.values():
            b.close()
        _batches.clear()


class BatchAdvect(torch.autograd.Function):
    """Many independent advections in one batch: f0 is one CUDA float64
    tensor holding the instances' fields one after another (instance i starts
    at the sum of the sizes of instances 0..i-1, each row-major), velocity a
    (count, 3) float64 tensor (row i: the instance's velocity, zero-padded
    beyond its axes), dts one time step per instance.  Forward: the batch's
    persistent advect; backward: fdb_batch_adjoint, giving dL/df0 and dL/dv
    for all instances at once (fdb_batch_advect_transposed alone when the
    velocity needs no gradient)."""

    @staticmethod
    def forward(ctx, f0, velocity, shapes, lengths, num_steps: int, dts,
                checkpoint_every: int = 0):
        if not f0.is_cuda or f0.dtype != torch.float64:
            raise TypeError("f0 must be a CUDA float64 tensor")
        b = _batch_handle(shapes, lengths, velocity, f0.device)
        f0c = f0.detach().contiguous().view(-1)
        b.set_fields(f0c)
        b.advect(int(num_steps), dts)
        out = torch.empty_like(f0c)
        b.get_fields(out)
        ctx.save_for_backward(f0c, velocity.detach())
        ctx.meta = (tuple(shapes), tuple(lengths), int(num_steps), tuple(float(x) for x in dts),
                    int(checkpoint_every))
        return out.view_as(f0)

    @staticmethod
    def backward(ctx, grad_out):
        f0c, velocity = ctx.saved_tensors
        shapes, lengths, num_steps, dts, ck = ctx.meta
        b = _batch_handle(shapes, lengths, velocity, f0c.device)
        lam = grad_out.detach().to(torch.float64).contiguous().view(-1)
        if not ctx.needs_input_grad[1]:
            # dL/df0 alone: the transposed problems, no re-run of the forward
            g0 = b.advect_transposed(num_steps, dts, lam)
            return g0.view_as(grad_out), None, None, None, None, None, None
        b.set_fields(f0c)
        b.set_adjoint_form("closed_keep" if ck == 0 else "stepwise")
        g0, gv = b.adjoint(num_steps, dts, lam, checkpoint_every=ck)
        grad_v = torch.as_tensor(gv, dtype=velocity.dtype, device=velocity.device)
        return g0.view_as(grad_out), grad_v, None, None, None, None, None


def batch_advect_fn(f0, velocity, shapes, num_steps: int, dts, lengths=None,
                    checkpoint_every: int = 0):
    """Differentiable batched advect (see BatchAdvect): returns the
    concatenated fields after num_steps steps; checkpoint_every as in
    advect_fn."""
    if lengths is None:
        lengths = [(1.0,) * len(n) for n in shapes]
    shapes = [tuple(int(x) for x in n) for n in shapes]
    lengths = [tuple(float(x) for x in L) for L in lengths]
    if not torch.is_tensor(velocity):
        rows = np.zeros((len(shapes), 3))
        for k, v in enumerate(velocity):
            rows[k, :len(v)] = v
        velocity = torch.tensor(rows, dtype=torch.float64)
    return BatchAdvect.apply(f0, velocity, tuple(shapes), tuple(lengths), num_steps,
                             tuple(float(x) for x in dts), checkpoint_every)


__all__ = ["UpwindAdvect", "advect_fn", "release_handles", "BatchAdvect", "batch_advect_fn",
           "release_batches"]
