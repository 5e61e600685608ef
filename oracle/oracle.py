"""ctypes front-end of the oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/libfdb_oracle.so`` (the C restatement of
upwind/cxx/upwind.cxx:51-103, see upwind_oracle.c) and, when it was built in
this tree, ``oracle/_ref/libfdb_refupwind.so`` (the reference's own
upwind.cxx compiled by path).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference legs import this module; the product
package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libfdb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfdb_refupwind.so")
REF_EXE = os.path.join(HERE, "_ref", "upwindCxx")
REF_ACC_SO = os.path.join(HERE, "_ref", "libfdb_refacc.so")
REF_FILTER_SO = os.path.join(HERE, "_ref", "libfdb_reffilter.so")

_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def reference_dir() -> str:
    """The reference's source tree: $FDB_REFERENCE_DIR, else a folder named
    `reference` beside this repository's root (it may not exist)."""
    env = os.environ.get("FDB_REFERENCE_DIR")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def build(ref: bool | None = None) -> None:
    """Compile the restatement (always) and the reference harness (when the
    reference source tree is present) with oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    refdir = reference_dir()
    if ref is None:
        ref = os.path.isfile(os.path.join(refdir, "upwind", "cxx", "upwind.cxx"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={refdir}"], check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _u64(seq) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seq, dtype=np.uint64))


def _f64(seq) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seq, dtype=np.float64))


class Port:
    """The C restatement (upwind_oracle.c)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.isfile(path):
            build(ref=False)
        lib = ctypes.CDLL(path)
        lib.fdbo_advect.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _dp, _dp,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_int]
        lib.fdbo_advect.restype = ctypes.c_int
        lib.fdbo_advect_form.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _dp, _dp,
                                         ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int]
        lib.fdbo_advect_form.restype = ctypes.c_int
        lib.fdbo_advect_spacing.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _u64p, _dp, _dp,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                            ctypes.c_int]
        lib.fdbo_advect_spacing.restype = ctypes.c_int
        lib.fdbo_checksum.argtypes = [_dp, ctypes.c_uint64]
        lib.fdbo_checksum.restype = ctypes.c_double
        lib.fdbo_std.argtypes = [_dp, ctypes.c_uint64]
        lib.fdbo_std.restype = ctypes.c_double
        lib.fdbo_coeff.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double]
        lib.fdbo_coeff.restype = ctypes.c_double
        lib.fdbo_adjoint_step.argtypes = [ctypes.c_int, _u64p, _dp, _dp, ctypes.c_double,
                                          _dp, _dp, _dp, _dp]
        lib.fdbo_adjoint_step.restype = ctypes.c_int
        lib.fdbo_fill_sphere_noise.argtypes = [ctypes.c_int, _u64p, _dp, _dp, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_uint64, _dp]
        lib.fdbo_fill_sphere_noise.restype = ctypes.c_int
        lib.fdbo_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        lib.fdbo_uniform.restype = ctypes.c_double
        lib.fdbo_max_threads.restype = ctypes.c_int
        self.lib = lib

    def advect(self, n, v, L, f0, steps: int, dt: float, threads: int = 0,
               coeff_form: int = 0) -> np.ndarray:
        """coeff_form 0: the coefficient of upwind.cxx:72; 1: the product
        form of the OpenACC variants and the Python class."""
        return self.advect_timed(n, v, L, f0, steps, dt, threads, coeff_form)[0]

    def advect_timed(self, n, v, L, f0, steps: int, dt: float, threads: int = 0,
                     coeff_form: int = 0):
        """(final field, wall seconds of the advect call alone)."""
        import time
        n, v, L = _u64(n), _f64(v), _f64(L)
        f = np.array(f0, dtype=np.float64, copy=True).reshape(-1)
        scratch = np.empty_like(f)
        scratch.fill(0.0)  # fault the pages in outside the timed call
        t0 = time.perf_counter()
        rc = self.lib.fdbo_advect_form(len(n), n.ctypes.data_as(_u64p), _ptr(v), _ptr(L),
                                       _ptr(f), _ptr(scratch), int(steps), float(dt),
                                       int(threads), int(coeff_form))
        el = time.perf_counter() - t0
        if rc:
            raise ValueError("oracle advect rejected its arguments")
        return f, el

    def advect_spacing(self, n, v, L, n_spacing, f0, steps: int, dt: float,
                       coeff_form: int = 0) -> np.ndarray:
        """advect on the grid n with the spacings L_j / n_spacing[j] of
        another grid (a slab of planes of a larger periodic grid)."""
        n, v, L, ns = _u64(n), _f64(v), _f64(L), _u64(n_spacing)
        f = np.array(f0, dtype=np.float64, copy=True).reshape(-1)
        scratch = np.zeros_like(f)
        rc = self.lib.fdbo_advect_spacing(len(n), n.ctypes.data_as(_u64p), _ptr(v), _ptr(L),
                                          ns.ctypes.data_as(_u64p), _ptr(f), _ptr(scratch),
                                          int(steps), float(dt), 0, int(coeff_form))
        if rc:
            raise ValueError("oracle advect rejected its arguments")
        return f

    def checksum(self, f) -> float:
        f = _f64(f).reshape(-1)
        return self.lib.fdbo_checksum(_ptr(f), f.size)

    def std(self, f) -> float:
        f = _f64(f).reshape(-1)
        return self.lib.fdbo_std(_ptr(f), f.size)

    def adjoint_step(self, n, v, L, dt, f, lam_in):
        """Returns (lam_out, dcoef[ndims]) for one transposed step."""
        n, v, L = _u64(n), _f64(v), _f64(L)
        f = _f64(f).reshape(-1)
        lam_in = _f64(lam_in).reshape(-1)
        lam_out = np.empty_like(lam_in)
        dcoef = np.zeros(len(n), dtype=np.float64)
        rc = self.lib.fdbo_adjoint_step(len(n), n.ctypes.data_as(_u64p), _ptr(v), _ptr(L),
                                        float(dt), _ptr(f), _ptr(lam_in), _ptr(lam_out),
                                        _ptr(dcoef))
        if rc:
            raise ValueError("oracle adjoint rejected its arguments")
        return lam_out, dcoef

    def sphere_noise(self, n, L, center, radius, noise_amp, seed) -> np.ndarray:
        n, L, c = _u64(n), _f64(L), _f64(center)
        f = np.empty(int(np.prod(n)), dtype=np.float64)
        rc = self.lib.fdbo_fill_sphere_noise(len(n), n.ctypes.data_as(_u64p), _ptr(L), _ptr(c),
                                             float(radius), float(noise_amp), int(seed), _ptr(f))
        if rc:
            raise ValueError("oracle sphere_noise rejected its arguments")
        return f

    def max_threads(self) -> int:
        return self.lib.fdbo_max_threads()

    # -- stencil Filter (filter_oracle.c) ----------------------------------------------
    def _filter_lib(self):
        lib = self.lib
        if not getattr(self, "_filter_ready", False):
            _ip = ctypes.POINTER(ctypes.c_int)
            lib.fdbo_filter_apply.argtypes = [ctypes.c_int, _u64p, ctypes.c_int, _ip, _dp, _dp,
                                              _dp, ctypes.c_int]
            lib.fdbo_filter_apply.restype = ctypes.c_int
            lib.fdbo_filter_checksum.argtypes = [_dp, ctypes.c_uint64]
            lib.fdbo_filter_checksum.restype = ctypes.c_double
            lib.fdbo_filter_sin_input.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _dp]
            lib.fdbo_filter_sin_input.restype = ctypes.c_int
            lib.fdbo_stencil_order.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _ip, _ip]
            lib.fdbo_stencil_order.restype = ctypes.c_int
            self._filter_ready = True
        return lib

    def filter_apply(self, dims, stencil, f_in, periodic: bool = False) -> np.ndarray:
        """One applyFilter of `stencil` ({offset tuple: weight} or a list of
        (offset, weight) pairs, insertion order kept) on the column-major
        field f_in; periodic=False reproduces the reference's index wrap."""
        lib = self._filter_lib()
        items = list(stencil.items()) if hasattr(stencil, "items") else list(stencil)
        dims = _u64(dims)
        offs = np.ascontiguousarray(np.array([o for o, _ in items], dtype=np.int32).reshape(-1))
        w = _f64([x for _, x in items])
        fi = _f64(f_in).reshape(-1)
        out = np.empty_like(fi)
        rc = lib.fdbo_filter_apply(len(dims), dims.ctypes.data_as(_u64p), len(items),
                                   offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(w),
                                   _ptr(fi), _ptr(out), 1 if periodic else 0)
        if rc:
            raise ValueError("oracle filter rejected its arguments")
        return out

    def filter_checksum(self, f) -> float:
        f = _f64(f).reshape(-1)
        return self._filter_lib().fdbo_filter_checksum(_ptr(f), f.size)

    def filter_sin_input(self, dims, xmins, xmaxs) -> np.ndarray:
        lib = self._filter_lib()
        dims, lo, hi = _u64(dims), _f64(xmins), _f64(xmaxs)
        f = np.empty(int(np.prod(dims)), dtype=np.float64)
        lib.fdbo_filter_sin_input(len(dims), dims.ctypes.data_as(_u64p), _ptr(lo), _ptr(hi),
                                  _ptr(f))
        return f

    def stencil_order(self, offsets) -> list[int]:
        """Term indices in the reference's std::map order (first insertion of
        a repeated offset wins)."""
        lib = self._filter_lib()
        o = np.ascontiguousarray(np.array(offsets, dtype=np.int32))
        nd = o.shape[1]
        order = np.zeros(len(o), dtype=np.int32)
        nu = ctypes.c_int()
        ip = ctypes.POINTER(ctypes.c_int)
        lib.fdbo_stencil_order(nd, len(o), o.ctypes.data_as(ip), order.ctypes.data_as(ip),
                               ctypes.byref(nu))
        return [int(x) for x in order[:nu.value]]


class Reference:
    """The reference's own Upwind<NDIMS> (ref_harness.cpp), when built here."""

    def __init__(self, path: str = REF_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.fdbr_advect.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _dp, _dp,
                                    ctypes.c_int, ctypes.c_double, _dp]
        lib.fdbr_advect.restype = ctypes.c_int
        lib.fdbr_default_field.argtypes = [ctypes.c_int, _u64p, _dp]
        lib.fdbr_default_field.restype = ctypes.c_int
        lib.fdbr_checksum.argtypes = [ctypes.c_int, _u64p, _dp]
        lib.fdbr_checksum.restype = ctypes.c_double
        lib.fdbr_std.argtypes = [ctypes.c_int, _u64p, _dp]
        lib.fdbr_std.restype = ctypes.c_double
        self.lib = lib

    @staticmethod
    def available() -> bool:
        return os.path.isfile(REF_SO)

    def advect(self, n, v, L, f0, steps: int, dt: float) -> np.ndarray:
        return self.advect_timed(n, v, L, f0, steps, dt)[0]

    def advect_timed(self, n, v, L, f0, steps: int, dt: float):
        """(final field, wall seconds of the reference's advect() call alone)."""
        n, v, L = _u64(n), _f64(v), _f64(L)
        out = np.empty(int(np.prod(n)), dtype=np.float64)
        fin = None if f0 is None else _f64(f0).reshape(-1)
        sec = ctypes.c_double(0.0)
        rc = self.lib.fdbr_advect(len(n), n.ctypes.data_as(_u64p), _ptr(v), _ptr(L),
                                  None if fin is None else _ptr(fin), _ptr(out),
                                  int(steps), float(dt), ctypes.byref(sec))
        if rc:
            raise ValueError("reference harness rejected its arguments")
        return out, sec.value

    def default_field(self, n) -> np.ndarray:
        n = _u64(n)
        out = np.empty(int(np.prod(n)), dtype=np.float64)
        self.lib.fdbr_default_field(len(n), n.ctypes.data_as(_u64p), _ptr(out))
        return out

    def checksum(self, n, f) -> float:
        n = _u64(n)
        f = _f64(f).reshape(-1)
        return self.lib.fdbr_checksum(len(n), n.ctypes.data_as(_u64p), _ptr(f))

    def std(self, n, f) -> float:
        n = _u64(n)
        f = _f64(f).reshape(-1)
        return self.lib.fdbr_std(len(n), n.ctypes.data_as(_u64p), _ptr(f))


class ReferenceAcc:
    """The reference's OpenACC variants upwindAcc.cxx (variant 1: one-step
    advect(double)) and upwindAcc2.cxx (variant 2: advect(int, double)),
    compiled serially by ref_acc_harness.cpp, when built here.  3-D only."""

    def __init__(self, path: str = REF_ACC_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.fdbr_acc_advect.argtypes = [ctypes.c_int, _u64p, _dp, _dp, _dp, _dp, ctypes.c_int,
                                        ctypes.c_double]
        lib.fdbr_acc_advect.restype = ctypes.c_int
        self.lib = lib

    @staticmethod
    def available() -> bool:
        return os.path.isfile(REF_ACC_SO)

    def advect(self, variant: int, n, v, L, f0, steps: int, dt: float) -> np.ndarray:
        n, v, L = _u64(n), _f64(v), _f64(L)
        if len(n) != 3:
            raise ValueError("the OpenACC variants are 3-D")
        out = np.empty(int(np.prod(n)), dtype=np.float64)
        fin = None if f0 is None else _f64(f0).reshape(-1)
        rc = self.lib.fdbr_acc_advect(int(variant), n.ctypes.data_as(_u64p), _ptr(v), _ptr(L),
                                      None if fin is None else _ptr(fin), _ptr(out), int(steps),
                                      float(dt))
        if rc:
            raise ValueError("reference OpenACC harness rejected its arguments")
        return out


class ReferenceFilter:
    """The reference's stencil Filter (cxx/Filter.cpp and its CubeDecomp,
    MultiArrayIter, writeVTK) for one rank on oracle/mpi_stub, compiled by
    ref_filter_harness.cpp, when built here."""

    def __init__(self, path: str = REF_FILTER_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        _ip = ctypes.POINTER(ctypes.c_int)
        lib.fdbr_filter_run.argtypes = [ctypes.c_int, _u64p, ctypes.c_int, _ip, _dp, _dp, _dp,
                                        ctypes.c_int, _dp]
        lib.fdbr_filter_run.restype = ctypes.c_int
        self.lib = lib

    @staticmethod
    def available() -> bool:
        return os.path.isfile(REF_FILTER_SO)

    def run(self, dims, stencil, f_in, iterations: int = 1):
        """(outData, (input checksum, output checksum)) after `iterations`
        applyFilter calls with copyOutToIn between them; `stencil` is a dict
        or a list of (offset, weight) pairs inserted in order."""
        items = list(stencil.items()) if hasattr(stencil, "items") else list(stencil)
        dims = _u64(dims)
        offs = np.ascontiguousarray(np.array([o for o, _ in items], dtype=np.int32).reshape(-1))
        w = _f64([x for _, x in items])
        fi = _f64(f_in).reshape(-1)
        out = np.empty_like(fi)
        sums = np.zeros(2)
        rc = self.lib.fdbr_filter_run(len(dims), dims.ctypes.data_as(_u64p), len(items),
                                      offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      _ptr(w), _ptr(fi), _ptr(out), int(iterations), _ptr(sums))
        if rc:
            raise ValueError(f"reference Filter harness rejected its arguments ({rc})")
        return out, (float(sums[0]), float(sums[1]))


def reference_dt(n, v, L, courant: float) -> float:
    """dt = min_j courant * dx_j / v_j as the reference driver computes it
    (upwind/cxx/upwind.cxx:186-192, which assumes v_j > 0)."""
    dt = np.finfo(np.float64).max
    for nj, vj, Lj in zip(n, v, L):
        dx = float(Lj) / float(nj)
        val = courant * dx / float(vj)
        dt = val if val < dt else dt
    return dt


def cfl_dt(n, v, L, cfl: float) -> float:
    """dt = cfl * min_j dx_j / |v_j| (axes with v_j = 0 are skipped), the rule
    the synthetic workloads use for signed velocities."""
    dt = np.inf
    for nj, vj, Lj in zip(n, v, L):
        if vj != 0.0:
            dt = min(dt, cfl * (float(Lj) / float(nj)) / abs(float(vj)))
    return float(dt if np.isfinite(dt) else cfl)
