"""Batches of independent upwind problems (fdb_batch_* in include/fdb_upwind.h).

Each instance is one reference Upwind<ndims> problem (upwind/cxx/upwind.cxx:
23-49, ndims <= 3) with its own grid, velocity and time step; ``advect``
advances all of them in one persistent launch, ``advect_looped`` runs the
single-field kernel instance by instance (the comparator).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import check, lib

# how adjoint() computes dL/dv (FDB_TUNE_ADJOINT)
_ADJOINT_FORMS = {"closed": 0, "stepwise": 1, "closed_keep": 2}


class InstanceDesc(ctypes.Structure):
    _fields_ = [("ndims", ctypes.c_int), ("num_cells", ctypes.c_uint64 * 3),
                ("velocity", ctypes.c_double * 3), ("lengths", ctypes.c_double * 3)]


class Batch:
    def __init__(self, instances):
        """instances: iterable of (velocity, lengths, numCells) triples."""
        inst = list(instances)
        arr = (InstanceDesc * len(inst))()
        self.shapes = []
        for k, (v, L, n) in enumerate(inst):
            nd = len(n)
            if not (len(v) == len(L) == nd) or nd < 1 or nd > 3:
                raise ValueError("each instance needs 1..3 axes of velocity, lengths, numCells")
            arr[k].ndims = nd
            for j in range(nd):
                arr[k].num_cells[j] = int(n[j])
                arr[k].velocity[j] = float(v[j])
                arr[k].lengths[j] = float(L[j])
            self.shapes.append(tuple(int(x) for x in n))
        h = ctypes.c_void_p()
        check(lib.fdb_batch_create(len(inst), arr, ctypes.byref(h)))
        self._h = h
        self.count = len(inst)
        self.sizes = [int(np.prod(s)) for s in self.shapes]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.fdb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total_cells(self) -> int:
        c = ctypes.c_int()
        t = ctypes.c_uint64()
        check(lib.fdb_batch_count(self._h, ctypes.byref(c), ctypes.byref(t)))
        return t.value

    def storage_order(self, index: int) -> tuple:
        """Stored axis order of an instance: stored axis k is axis order[k] of
        its 3-D view (the batch marches along the axis that tiles worst)."""
        o = (ctypes.c_int * 3)()
        check(lib.fdb_batch_storage_order(self._h, int(index), o))
        return tuple(o)

    def _dts(self, dt) -> np.ndarray:
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (self.count,)))
        return d

    def advect(self, numTimeSteps: int, dt) -> None:
        d = self._dts(dt)
        check(lib.fdb_batch_advect(self._h, int(numTimeSteps), d.ctypes.data))

    def advect_looped(self, numTimeSteps: int, dt) -> None:
        d = self._dts(dt)
        check(lib.fdb_batch_advect_looped(self._h, int(numTimeSteps), d.ctypes.data))

    def adjoint(self, numTimeSteps: int, dt, lambda_T, grad_f0=None, checkpoint_every: int = 0,
                velocity_grad: bool = True):
        """Gradients of a loss L(f_T of every instance) given lambda_T =
        dL/df_T: the instances' fields one after another (instance i starts
        at sum(sizes[:i])), a numpy array or a CUDA float64 tensor.  All
        instances at once; the fields end at f_T.  Returns (grad_f0 in the
        same concatenated form and kind, grad_v of shape (count, 3): dL/dv per
        axis, 0 for missing axes).  dL/dv in closed form by default, or step
        by step (set_adjoint_form("stepwise")).  velocity_grad=False returns
        (grad_f0, None) from the transposed problems alone."""
        d = self._dts(dt)
        total = sum(self.sizes)
        is_dev = 1 if getattr(lambda_T, "is_cuda", False) else 0
        if is_dev:
            import torch
            torch.cuda.current_stream(lambda_T.device).synchronize()  # torch's writes first
            if lambda_T.numel() != total:
                raise ValueError(f"lambda_T needs {total} values, got {lambda_T.numel()}")
            if grad_f0 is None:
                grad_f0 = torch.empty(total, dtype=torch.float64, device=lambda_T.device)
            lam_p, g_p = lambda_T.data_ptr(), grad_f0.data_ptr()
        else:
            lambda_T = np.ascontiguousarray(np.asarray(lambda_T, dtype=np.float64)).reshape(-1)
            if lambda_T.size != total:
                raise ValueError(f"lambda_T needs {total} values, got {lambda_T.size}")
            if grad_f0 is None:
                grad_f0 = np.empty(total, dtype=np.float64)
            lam_p, g_p = lambda_T.ctypes.data, grad_f0.ctypes.data
        gv = np.zeros((self.count, 3), dtype=np.float64) if velocity_grad else None
        check(lib.fdb_batch_adjoint(self._h, int(numTimeSteps), d.ctypes.data, lam_p, g_p,
                                    gv.ctypes.data if velocity_grad else None,
                                    int(checkpoint_every), is_dev))
        return grad_f0, gv

    def advect_transposed(self, numTimeSteps: int, dt, values, out=None):
        """(A^T)^S applied to every instance of ``values`` (concatenated as
        in adjoint(), numpy or CUDA float64 tensor) without touching the
        fields: the grad_f0 of adjoint(velocity_grad=False), for callers that
        already hold f_T.  ``out`` may be ``values``."""
        d = self._dts(dt)
        total = sum(self.sizes)
        is_dev = 1 if getattr(values, "is_cuda", False) else 0
        if is_dev:
            import torch
            torch.cuda.current_stream(values.device).synchronize()  # torch's writes first
            if values.numel() != total:
                raise ValueError(f"values need {total} entries, got {values.numel()}")
            if out is None:
                out = torch.empty(total, dtype=torch.float64, device=values.device)
            in_p, out_p = values.data_ptr(), out.data_ptr()
        else:
            values = np.ascontiguousarray(np.asarray(values, dtype=np.float64)).reshape(-1)
            if values.size != total:
                raise ValueError(f"values need {total} entries, got {values.size}")
            if out is None:
                out = np.empty(total, dtype=np.float64)
            in_p, out_p = values.ctypes.data, out.ctypes.data
        check(lib.fdb_batch_advect_transposed(self._h, int(numTimeSteps), d.ctypes.data, in_p,
                                              out_p, is_dev))
        return out

    def checksums(self) -> np.ndarray:
        out = np.empty(self.count, dtype=np.float64)
        check(lib.fdb_batch_checksums(self._h, out.ctypes.data))
        return out

    def set_field(self, index: int, values) -> None:
        if hasattr(values, "is_cuda") and values.is_cuda:
            import torch
            torch.cuda.current_stream(values.device).synchronize()  # torch's writes first
            check(lib.fdb_batch_set_field(self._h, int(index), values.data_ptr(), 1))
            return
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float64)).reshape(-1)
        if a.size != self.sizes[index]:
            raise ValueError(f"instance {index} has {self.sizes[index]} cells, got {a.size}")
        check(lib.fdb_batch_set_field(self._h, int(index), a.ctypes.data, 0))

    def get_field(self, index: int) -> np.ndarray:
        out = np.empty(self.sizes[index], dtype=np.float64)
        check(lib.fdb_batch_get_field(self._h, int(index), out.ctypes.data, 0))
        return out

    def set_fields(self, values) -> None:
        """All fields from one concatenated array (instance i starts at
        sum(sizes[:i])): numpy or a CUDA float64 tensor."""
        total = sum(self.sizes)
        dev = bool(getattr(values, "is_cuda", False))
        if dev:
            import torch
            torch.cuda.current_stream(values.device).synchronize()  # torch's writes first
            if values.numel() != total or not values.is_contiguous():
                raise ValueError(f"need a contiguous tensor of {total} values")
            base = values.data_ptr()
        else:
            values = np.ascontiguousarray(np.asarray(values, dtype=np.float64)).reshape(-1)
            if values.size != total:
                raise ValueError(f"need {total} values, got {values.size}")
            base = values.ctypes.data
        off = 0
        for k, n in enumerate(self.sizes):
            check(lib.fdb_batch_set_field(self._h, k, base + 8 * off, 1 if dev else 0))
            off += n

    def get_fields(self, out=None):
        """All fields into one concatenated array (numpy, or `out`: a numpy
        array or a contiguous CUDA float64 tensor)."""
        total = sum(self.sizes)
        if out is None:
            out = np.empty(total, dtype=np.float64)
        dev = bool(getattr(out, "is_cuda", False))
        if dev and (out.numel() != total or not out.is_contiguous()):
            raise ValueError(f"need a contiguous tensor of {total} values")
        if not dev and out.size != total:
            raise ValueError(f"need {total} values")
        base = out.data_ptr() if dev else out.ctypes.data
        off = 0
        for k, n in enumerate(self.sizes):
            check(lib.fdb_batch_get_field(self._h, k, base + 8 * off, 1 if dev else 0))
            off += n
        return out

    def set_velocity(self, index: int, velocity) -> None:
        v = np.ascontiguousarray(np.asarray(velocity, dtype=np.float64)).reshape(-1)
        if v.size != len(self.shapes[index]):
            raise ValueError("velocity needs one value per axis of the instance")
        check(lib.fdb_batch_set_velocity(self._h, int(index), v.ctypes.data))

    def init_sphere(self, index: int, center, radius: float, noise_amp: float = 0.0,
                    seed: int = 0) -> None:
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float64))
        check(lib.fdb_batch_init_sphere(self._h, int(index), c.ctypes.data, float(radius),
                                        float(noise_amp), int(seed)))

    def set_stream(self, stream) -> None:
        raw = getattr(stream, "cuda_stream", stream)
        check(lib.fdb_batch_set_stream(self._h, raw))

    def set_tuning(self, depth: int | None = None, shape: int | None = None,
                   tile_z: int | None = None) -> None:
        """Launch-shape knobs of the persistent launch (None leaves a knob)."""
        if depth is not None:
            check(lib.fdb_batch_set_tuning(self._h, 3, int(depth)))
        if shape is not None:
            check(lib.fdb_batch_set_tuning(self._h, 2, int(shape)))
        if tile_z is not None:
            check(lib.fdb_batch_set_tuning(self._h, 1, int(tile_z)))

    def set_adjoint_form(self, form: str = "closed") -> None:
        """How adjoint() computes dL/dv: "closed" (default; S <lam^1, D_j f0>,
        one contraction), "stepwise" (checkpoints, one contraction per
        transposed step) or "closed_keep" (closed, the fields left at f0)."""
        check(lib.fdb_batch_set_tuning(self._h, 4, _ADJOINT_FORMS[form]))

    def autotune(self, numTimeSteps: int, dt, cache_path: str | None = None) -> dict:
        d = self._dts(dt)
        chosen = (ctypes.c_int * 3)()
        check(lib.fdb_batch_autotune(self._h, int(numTimeSteps), d.ctypes.data,
                                     cache_path.encode() if cache_path else None, chosen))
        return {"depth": chosen[0], "shape": chosen[1], "tile_z": chosen[2]}


def random_instances(count: int, seed: int, nmin: int = 32, nmax: int = 160, cfl: float = 0.5):
    """The uneven workload of the batched benchmark: axis lengths uniform in
    [nmin, nmax], velocities uniform in [-1, 1]^3, dt = cfl * min dx/|v|,
    sphere centres in [0.3, 0.7]^3 and radii in [0.1, 0.25] (all seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = tuple(int(x) for x in rng.integers(nmin, nmax + 1, size=3))
        v = tuple(float(x) for x in rng.uniform(-1.0, 1.0, size=3))
        L = (1.0, 1.0, 1.0)
        dt = cfl * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(L, n, v) if vj != 0.0)
        centre = tuple(float(x) for x in rng.uniform(0.3, 0.7, size=3))
        radius = float(rng.uniform(0.1, 0.25))
        out.append({"n": n, "v": v, "L": L, "dt": dt, "center": centre, "radius": radius})
    return out


__all__ = ["Batch", "InstanceDesc", "random_instances"]
_ = _capi
