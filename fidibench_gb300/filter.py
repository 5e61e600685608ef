"""The stencil Filter (include/fdb_filter.h) from Python.

Mirrors the public members of the reference's class Filter (cxx/Filter.h:25-
170) on one process: ``applyFilter``, ``copyOutToIn``, ``computeCheckSum``,
``setInData`` / ``setInDataByIndices``, ``getPosition``, ``saveVTK``,
``getRank`` (0), ``getNumProcs`` (1), ``isDecompValid`` (True).  Fields are
column-major (axis 0 fastest) as in the reference; ``in_data`` / ``out_data``
return them as flat numpy arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._capi import check, lib

WRAP_REFERENCE = 0
WRAP_PERIODIC = 1


def laplacian_stencil(ndims: int) -> dict:
    """The laplacian driver's stencil (laplacian/cxx/laplacian.cxx:57-66):
    -2 ndims at the centre, +1 at +-1 along each axis (insertion order kept)."""
    st = {}
    off = [0] * ndims
    st[tuple(off)] = -2.0 * ndims
    for i in range(ndims):
        off[i] = 1
        st.setdefault(tuple(off), 1.0)
        off[i] = -1
        st.setdefault(tuple(off), 1.0)
        off[i] = 0
    return st


def sin_input(pos) -> float:
    """The laplacian driver's input function: prod_i sin(2 pi x_i)."""
    res = 1.0
    for x in pos:
        res *= float(np.sin(2.0 * np.pi * x))
    return res


class Filter:
    def __init__(self, globalDims, xmins, xmaxs, stencil, wrap: int = WRAP_REFERENCE):
        """stencil: {offset tuple: weight} (or (offset, weight) pairs)."""
        items = list(stencil.items()) if hasattr(stencil, "items") else list(stencil)
        self.globalDims = [int(n) for n in globalDims]
        self.ndims = len(self.globalDims)
        self.xmins = [float(x) for x in xmins]
        self.xmaxs = [float(x) for x in xmaxs]
        if not (len(self.xmins) == len(self.xmaxs) == self.ndims):
            raise ValueError("globalDims, xmins and xmaxs must have the same length")
        offs = np.ascontiguousarray(np.array([list(o) for o, _ in items], dtype=np.int32))
        if offs.ndim != 2 or offs.shape[1] != self.ndims:
            raise ValueError("every stencil offset needs one value per axis")
        w = np.ascontiguousarray(np.array([v for _, v in items], dtype=np.float64))
        dims = np.ascontiguousarray(np.array(self.globalDims, dtype=np.uint64))
        lo = np.ascontiguousarray(np.array(self.xmins, dtype=np.float64))
        hi = np.ascontiguousarray(np.array(self.xmaxs, dtype=np.float64))
        h = ctypes.c_void_p()
        check(lib.fdb_filter_create(self.ndims, dims.ctypes.data, lo.ctypes.data, hi.ctypes.data,
                                    len(items), offs.ctypes.data, w.ctypes.data,
                                    ctypes.byref(h)))
        self._h = h
        self.ntot = int(np.prod(self.globalDims))
        self.set_wrap(wrap)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.fdb_filter_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration -----------------------------------------------------------------
    def set_wrap(self, mode: int) -> None:
        check(lib.fdb_filter_set_wrap(self._h, int(mode)))

    def set_stream(self, stream) -> None:
        raw = getattr(stream, "cuda_stream", stream)
        check(lib.fdb_filter_set_stream(self._h, raw))

    # -- the reference's members ------------------------------------------------------------
    def getRank(self) -> int:
        return 0

    def getNumProcs(self) -> int:
        return 1

    def isDecompValid(self) -> bool:
        return True

    def getPosition(self, globalInds):
        """Cell centre (Filter.cpp:104-112)."""
        return [self.xmins[i] + (globalInds[i] + 0.5) *
                ((self.xmaxs[i] - self.xmins[i]) / float(self.globalDims[i]))
                for i in range(self.ndims)]

    def _indices(self):
        n = self.globalDims
        flat = np.arange(self.ntot, dtype=np.int64)
        prod = 1
        out = []
        for d in range(self.ndims):
            out.append((flat // prod) % n[d])
            prod *= n[d]
        return out

    def setInData(self, f) -> None:
        """f(position list) -> value at every cell centre (evaluated on the
        host, as the reference does; see set_in_data for arrays)."""
        inds = self._indices()
        vals = np.array([f(self.getPosition([int(ix[i]) for ix in inds]))
                         for i in range(self.ntot)], dtype=np.float64)
        self.set_in_data(vals)

    def setInDataByIndices(self, f) -> None:
        inds = self._indices()
        vals = np.array([f([int(ix[i]) for ix in inds]) for i in range(self.ntot)],
                        dtype=np.float64)
        self.set_in_data(vals)

    def applyFilter(self) -> None:
        check(lib.fdb_filter_apply(self._h))

    def copyOutToIn(self) -> None:
        check(lib.fdb_filter_copy_out_to_in(self._h))

    def iterate(self, iterations: int) -> None:
        """iterations x (applyFilter; copyOutToIn) in one call."""
        check(lib.fdb_filter_iterate(self._h, int(iterations)))

    def computeCheckSum(self, inOrOut: str) -> float:
        out = ctypes.c_double()
        check(lib.fdb_filter_checksum(self._h, 0 if inOrOut == "input" else 1,
                                      ctypes.byref(out)))
        return out.value

    def saveVTK(self, filename: str) -> None:
        from .vtk import write_structured_filter
        write_structured_filter(filename, self.globalDims, self.xmins, self.xmaxs, self.out_data,
                                "outData")

    # -- field access -----------------------------------------------------------------------
    def set_in_data(self, values) -> None:
        if hasattr(values, "is_cuda") and values.is_cuda:
            import torch
            t = values.detach().to(dtype=torch.float64).contiguous()
            torch.cuda.current_stream(t.device).synchronize()
            check(lib.fdb_filter_set_in_data(self._h, t.data_ptr(), 1))
            return
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        if a.size != self.ntot:
            raise ValueError(f"field has {a.size} values, expected {self.ntot}")
        check(lib.fdb_filter_set_in_data(self._h, a.ctypes.data, 0))

    def _get(self, which: int) -> np.ndarray:
        out = np.empty(self.ntot, dtype=np.float64)
        check(lib.fdb_filter_get_data(self._h, which, out.ctypes.data, 0))
        return out

    @property
    def in_data(self) -> np.ndarray:
        return self._get(0)

    @property
    def out_data(self) -> np.ndarray:
        return self._get(1)


__all__ = ["Filter", "laplacian_stencil", "sin_input", "WRAP_REFERENCE", "WRAP_PERIODIC"]
