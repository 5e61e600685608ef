"""Python mirror of the reference's ``Upwind`` class, backed by libfdb_upwind.

Mirrors upwind/python/upwind.py:8-86 (constructor arguments, ``advect``,
``checksum``, ``printOut``, ``saveVTK``) and adds the C++ class's members
(upwind/cxx/upwind.cxx:51-109: ``advect(numTimeSteps, deltaTime)``, ``std``,
``print``).  All state lives on the GPU; host copies are made only when the
caller asks for the field.

Differences from the Python reference, by design:
  * the field is advanced on the device by the CUDA step kernels; the
    arithmetic is selectable (``arith="exact"`` reproduces the reference's
    C++ operation order bit for bit, the default picks the fastest path that
    meets the parity bar);
  * ``f`` is a property: reading it copies the field to a numpy array,
    assigning to it uploads a new field (setInitialCondition).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import check, lib


def _as_u64(seq) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seq, dtype=np.uint64))


def _as_f64(seq) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seq, dtype=np.float64))


def _order_after_torch(t) -> None:
    """The library works on its own CUDA stream; a tensor torch has just
    written on its current stream must be complete before the library reads
    (or overwrites) it, so wait for that stream here."""
    import torch
    torch.cuda.current_stream(t.device).synchronize()


class Upwind:
    """Periodic N-D first-order upwind advection of a scalar field (FP64)."""

    def __init__(self, velocity, lengths, numCells, arith: str = "auto", depth: int = 0,
                 coeff_form: str = "cxx"):
        self.v = _as_f64(velocity)
        self.lengths = _as_f64(lengths)
        self.numCells = [int(x) for x in numCells]
        self.ndims = len(self.numCells)
        if not (len(self.v) == len(self.lengths) == self.ndims):
            raise ValueError("velocity, lengths and numCells must have the same length")
        n = _as_u64(self.numCells)
        h = ctypes.c_void_p()
        check(lib.fdb_upwind_create(self.ndims, self.v.ctypes.data, self.lengths.ctypes.data,
                                    n.ctypes.data, ctypes.byref(h)))
        self._h = h
        self.ntot = int(np.prod(self.numCells))
        # upwind/python/upwind.py:20-25
        self.upDirection = np.where(self.v < 0.0, 1, -1).astype(np.int32)
        self.deltas = self.lengths / np.asarray(self.numCells, dtype=np.float64)
        self.set_arith(arith, depth)
        if coeff_form != "cxx":
            self.set_coeff_form(coeff_form)

    # -- lifetime ---------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.fdb_upwind_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration ------------------------------------------------------------
    def set_arith(self, arith: str = "auto", depth: int = 0) -> None:
        code = _capi.ARITH_NAMES[arith] if isinstance(arith, str) else int(arith)
        check(lib.fdb_upwind_set_arith(self._h, code, int(depth)))

    def set_coeff_form(self, form: str = "cxx") -> None:
        """Rounding of the per-axis coefficient: "cxx" = ((dt*v)*up)/dx as
        upwind/cxx/upwind.cxx:72 (default); "python" (or "product") =
        dt*((v*up)/dx) as upwind/python/upwind.py:32,64 and the OpenACC
        variants.  With arith="exact" each is bit-identical to its variant."""
        check(lib.fdb_upwind_set_coeff_form(self._h, _capi.COEFF_NAMES[form]))

    def set_tile_z(self, tile_z: int) -> None:
        """Most output planes one CTA of the fixed-point kernel takes along
        the slowest axis (0 = automatic: z-slabs that shrink towards the end
        of the grid)."""
        check(lib.fdb_upwind_set_tuning(self._h, 1, int(tile_z)))

    def set_shape(self, shape: int) -> None:
        """Fixed-point kernel CTA shape: 0 = 8 rows x 8 warps, 1 = 4 x 16 (plane
        history in registers), 2 = 8 x 8, 3 = 4 x 16, 4 = 4 x 8 (history in
        shared memory), 5 = 4 x 8, 6 = 6 x 8 (history in shared memory, the
        next plane in registers, the x-1 neighbour from the history),
        -1 = automatic."""
        check(lib.fdb_upwind_set_tuning(self._h, 2, int(shape)))

    def set_adjoint_form(self, form: str = "closed") -> None:
        """How adjoint() computes dL/dv: "closed" (default: the step's
        operators commute on the periodic grid, so dL/da_j = S <lam^1, D_j f0>
        with lam^1 = (A^T)^(S-1) lam_T -- one contraction, no checkpoints) or
        "stepwise" (checkpoint/recompute and one contraction per transposed
        step; checkpoint_every applies) or "closed_keep" (the closed form
        with the field left at f0, for callers that already hold f_T)."""
        check(lib.fdb_upwind_set_tuning(self._h, 4,
                                        {"closed": 0, "stepwise": 1, "closed_keep": 2}[form]))

    def set_velocity(self, velocity) -> None:
        """New velocity for the same grid (the upwind directions follow its sign)."""
        v = _as_f64(velocity)
        if v.size != self.ndims:
            raise ValueError("velocity needs one value per axis")
        check(lib.fdb_upwind_set_velocity(self._h, v.ctypes.data))
        self.v = v
        self.upDirection = np.where(self.v < 0.0, 1, -1).astype(np.int32)

    def set_stream(self, stream) -> None:
        """Enqueue on a CUDA stream (a torch.cuda.Stream, a raw handle or None)."""
        raw = getattr(stream, "cuda_stream", stream)
        check(lib.fdb_upwind_set_stream(self._h, raw))

    @property
    def arith_used(self) -> str:
        ntot = ctypes.c_uint64()
        a = ctypes.c_int()
        check(lib.fdb_upwind_info(self._h, ctypes.byref(ntot), ctypes.byref(a)))
        return {v: k for k, v in _capi.ARITH_NAMES.items()}.get(a.value, str(a.value))

    # -- the reference API ----------------------------------------------------------
    def advect(self, *args) -> None:
        """``advect(deltaTime)`` (one step, upwind/python/upwind.py:46) or
        ``advect(numTimeSteps, deltaTime)`` (upwind/cxx/upwind.cxx:51)."""
        if len(args) == 1:
            steps, dt = 1, args[0]
        elif len(args) == 2:
            steps, dt = args
        else:
            raise TypeError("advect(deltaTime) or advect(numTimeSteps, deltaTime)")
        check(lib.fdb_upwind_advect(self._h, int(steps), float(dt)))

    def checksum(self) -> float:
        out = ctypes.c_double()
        check(lib.fdb_upwind_checksum(self._h, ctypes.byref(out)))
        return out.value

    def std(self) -> float:
        out = ctypes.c_double()
        check(lib.fdb_upwind_std(self._h, ctypes.byref(out)))
        return out.value

    def printOut(self) -> None:
        for i, x in enumerate(self.f):
            print(i, " ", x)

    def print(self) -> None:
        for i, x in enumerate(self.f):
            print(i, x)

    def saveVTK(self, fname: str) -> None:
        """ASCII rectilinear VTK file of the field (upwind/python/upwind.py:69-79)."""
        from .vtk import write_rectilinear
        write_rectilinear(fname, self.numCells, self.deltas, self.f, title="upwind")

    # -- field access ------------------------------------------------------------
    @property
    def f(self) -> np.ndarray:
        out = np.empty(self.ntot, dtype=np.float64)
        check(lib.fdb_upwind_get_field(self._h, out.ctypes.data, 0))
        return out

    @f.setter
    def f(self, values) -> None:
        self.set_field(values)

    def set_field(self, values) -> None:
        """setInitialCondition: numpy array (host) or CUDA torch tensor (device)."""
        if hasattr(values, "is_cuda") and values.is_cuda:
            t = values.detach().to(dtype=__import__("torch").float64).contiguous()
            if t.numel() != self.ntot:
                raise ValueError(f"field has {t.numel()} values, expected {self.ntot}")
            _order_after_torch(t)
            check(lib.fdb_upwind_set_field(self._h, t.data_ptr(), 1))
            return
        a = _as_f64(values).reshape(-1)
        if a.size != self.ntot:
            raise ValueError(f"field has {a.size} values, expected {self.ntot}")
        check(lib.fdb_upwind_set_field(self._h, a.ctypes.data, 0))

    def get_field(self, out=None):
        """Copy the field into ``out`` (numpy or CUDA torch tensor) or a new array."""
        if out is None:
            return self.f
        is_dev = 1 if getattr(out, "is_cuda", False) else 0
        if is_dev:
            _order_after_torch(out)
        check(lib.fdb_upwind_get_field(self._h, _capi.dptr(out), is_dev))
        return out

    def advect_host_stream(self, fields, numTimeSteps: int, deltaTime: float,
                           out=None) -> np.ndarray:
        """The driver's cycle (upwind/cxx/upwind.cxx:194-199: initial field,
        advect, checksum) over a sequence of host fields, with the upload of
        the next field and the download of the previous result overlapping
        each advect.  ``fields`` and ``out`` hold host buffers of ntot FP64
        values (numpy arrays or CPU torch tensors, pinned for the overlap);
        ``out`` defaults to writing the results back into ``fields``.
        Returns the checksum of every result; the handle is left at the last
        result."""
        fields = list(fields)
        out = fields if out is None else list(out)
        if len(out) != len(fields):
            raise ValueError("out needs one buffer per field")
        for a in fields + out:
            if getattr(a, "is_cuda", False):
                raise ValueError("advect_host_stream takes host buffers")
            ok = (a.dtype == np.float64 if isinstance(a, np.ndarray)
                  else str(a.dtype) == "torch.float64")
            contiguous = (a.flags.c_contiguous if isinstance(a, np.ndarray)
                          else a.is_contiguous())
            if not ok or not contiguous:
                raise ValueError("host fields must be contiguous float64")
            n = a.size if isinstance(a, np.ndarray) else a.numel()
            if n != self.ntot:
                raise ValueError(f"field has {n} values, expected {self.ntot}")
        for a in out:
            if isinstance(a, np.ndarray) and not a.flags.writeable:
                raise ValueError("output buffers must be writeable")
        cnt = len(fields)
        ins = (ctypes.c_void_p * max(cnt, 1))(*[_capi.dptr(a) for a in fields])
        outs = (ctypes.c_void_p * max(cnt, 1))(*[_capi.dptr(a) for a in out])
        sums = np.zeros(cnt, dtype=np.float64)
        check(lib.fdb_upwind_advect_host_stream(self._h, cnt, ins, outs, int(numTimeSteps),
                                                float(deltaTime), sums.ctypes.data))
        return sums

    def field_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(lib.fdb_upwind_field_ptr(self._h, ctypes.byref(p)))
        return p.value

    def init_sphere(self, center, radius: float, noise_amp: float = 0.0, seed: int = 0) -> None:
        c = _as_f64(center)
        if c.size != self.ndims:
            raise ValueError("centre needs one coordinate per axis")
        check(lib.fdb_upwind_init_sphere(self._h, c.ctypes.data, float(radius), float(noise_amp),
                                         int(seed)))

    # -- adjoint -------------------------------------------------------------------
    def adjoint(self, numTimeSteps: int, deltaTime: float, lambda_T, grad_f0=None,
                checkpoint_every: int = 0, velocity_grad: bool = True):
        """Gradient of a loss L(f_T) given lambda_T = dL/df_T.

        Returns (grad_f0, grad_v) and leaves the field at f_T.  dL/df0 comes
        from the transposed problem (every upwind direction reversed); dL/dv
        in closed form by default, or step by step with checkpoint/recompute
        (set_adjoint_form("stepwise"); checkpoint_every applies).
        lambda_T/grad_f0 may be numpy arrays or CUDA tensors (both of the same
        kind).  velocity_grad=False returns (grad_f0, None)."""
        is_dev = 1 if getattr(lambda_T, "is_cuda", False) else 0
        if is_dev:
            _order_after_torch(lambda_T)
        if grad_f0 is None:
            if is_dev:
                import torch
                grad_f0 = torch.empty(self.ntot, dtype=torch.float64, device=lambda_T.device)
            else:
                grad_f0 = np.empty(self.ntot, dtype=np.float64)
        if not is_dev:
            lambda_T = _as_f64(lambda_T).reshape(-1)
        gv = np.zeros(self.ndims, dtype=np.float64) if velocity_grad else None
        if not is_dev:
            grad_f0 = np.ascontiguousarray(grad_f0, dtype=np.float64)
        check(lib.fdb_upwind_adjoint(self._h, int(numTimeSteps), float(deltaTime),
                                     _capi.dptr(lambda_T), _capi.dptr(grad_f0),
                                     gv.ctypes.data if velocity_grad else None,
                                     int(checkpoint_every), is_dev))
        return grad_f0, gv

    def advect_transposed(self, numTimeSteps: int, deltaTime: float, values, out=None):
        """(A^T)^numTimeSteps applied to ``values`` (numpy array or CUDA
        float64 tensor) without touching the field: the grad_f0 of
        adjoint(velocity_grad=False), for callers that already hold f_T.
        ``out`` (same kind) may be ``values``."""
        is_dev = 1 if getattr(values, "is_cuda", False) else 0
        if is_dev:
            import torch
            if values.dtype != torch.float64 or not values.is_contiguous():
                raise ValueError("values must be a contiguous float64 tensor")
            n = values.numel()
            _order_after_torch(values)
            if out is None:
                out = torch.empty(self.ntot, dtype=torch.float64, device=values.device)
        else:
            values = _as_f64(values).reshape(-1)
            n = values.size
            if out is None:
                out = np.empty(self.ntot, dtype=np.float64)
            elif (not isinstance(out, np.ndarray) or out.dtype != np.float64
                  or not out.flags.c_contiguous or not out.flags.writeable):
                raise ValueError("out must be a writeable contiguous float64 array")
        if n != self.ntot:
            raise ValueError(f"values have {n} entries, expected {self.ntot}")
        out_n = out.numel() if is_dev else out.size
        if out_n != self.ntot or getattr(out, "is_cuda", False) != bool(is_dev):
            raise ValueError("out must match values in size and kind")
        check(lib.fdb_upwind_advect_transposed(self._h, int(numTimeSteps), float(deltaTime),
                                               _capi.dptr(values), _capi.dptr(out), is_dev))
        return out

    def adjoint_timings(self) -> dict:
        """Device milliseconds of the last adjoint call, by phase."""
        ms = np.zeros(3, dtype=np.float64)
        check(lib.fdb_upwind_adjoint_timings(self._h, ms.ctypes.data))
        return {"forward_ms": float(ms[0]), "recompute_ms": float(ms[1]),
                "adjoint_ms": float(ms[2])}


def main(argv=None) -> int:
    """Command line of the reference's Python driver (upwind/python/upwind.py:
    88-126): ``N [numTimeSteps=100] [vtk]`` on the periodic unit cube with
    N^3 cells, velocity (1, 1, 1) and courant 0.1, one advect(dt) call per
    step, then ``check sum:`` (and up.vtk with ``vtk``)."""
    import sys
    args = sys.argv[1:] if argv is None else list(argv)
    if len(args) < 1:
        print("must specify number of cells in each direction.")
        return 1
    ndims = 3
    numCells = [int(args[0])] * ndims
    print("number of cells: ", numCells)
    numTimeSteps = int(args[1]) if len(args) > 1 else 100
    print("number of time steps: ", numTimeSteps)
    doVtk = len(args) > 2 and args[2] == "vtk"
    velocity = np.ones((ndims,), np.float64)
    lengths = np.ones((ndims,), np.float64)
    courant = 0.1
    dt = float("inf")
    for j in range(ndims):
        dx = lengths[j] / float(numCells[j])
        dt = min(courant * dx / velocity[j], dt)
    # the Python class rounds its coefficients as dt * (v*up/dx) (upwind.py:32,64)
    up = Upwind(velocity, lengths, numCells, coeff_form="python")
    for _ in range(numTimeSteps):
        up.advect(dt)
    print("check sum: ", up.checksum())
    if doVtk:
        up.saveVTK("up.vtk")
    up.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
