"""ctypes binding of libfdb_upwind.so (the C-ABI in include/fdb_upwind.h and
include/fdb_filter.h).

The library is loaded from the package's in-tree ``_lib/`` directory.  There
is no fallback: if the shared library is missing or was built for another
host, importing this module raises, so no caller can silently end up on a CPU
path.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfdb_upwind.so")

FDB_OK = 0
FDB_ERR_INVALID = 1
FDB_ERR_CUDA = 2
FDB_ERR_ALLOC = 3
FDB_ERR_UNSUPPORTED = 4
FDB_ERR_TIMEOUT = 5
FDB_ERR_NONFINITE = 6
FDB_ERR_INJECTED = 7
FDB_MAX_DIMS = 8

ARITH_AUTO = 0
ARITH_EXACT = 1
ARITH_FMA = 2
ARITH_FIXED = 3
ARITH_NAMES = {"auto": ARITH_AUTO, "exact": ARITH_EXACT, "fma": ARITH_FMA, "fixed": ARITH_FIXED}

COEFF_CXX = 0
COEFF_PRODUCT = 1
# "python": the reference's Python class rounds its coefficients as the
# OpenACC/OpenMP-offload variants do
COEFF_NAMES = {"cxx": COEFF_CXX, "product": COEFF_PRODUCT, "python": COEFF_PRODUCT}

_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p
_int = ctypes.c_int

# name -> (restype, argtypes); every symbol declared in include/*.h
SIGNATURES: dict[str, tuple] = {
    "fdb_last_error": (ctypes.c_char_p, []),
    "fdb_version": (ctypes.c_char_p, []),
    "fdb_launch_count": (ctypes.c_uint64, []),
    "fdb_upwind_create": (_int, [_int, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "fdb_upwind_destroy": (_int, [_vp]),
    "fdb_upwind_set_field": (_int, [_vp, _vp, _int]),
    "fdb_upwind_get_field": (_int, [_vp, _vp, _int]),
    "fdb_upwind_field_ptr": (_int, [_vp, ctypes.POINTER(_vp)]),
    "fdb_upwind_advect": (_int, [_vp, _int, ctypes.c_double]),
    "fdb_upwind_checksum": (_int, [_vp, _dp]),
    "fdb_upwind_advect_host_stream": (_int, [_vp, _int, _vp, _vp, _int, ctypes.c_double, _vp]),
    "fdb_upwind_advect_transposed": (_int, [_vp, _int, ctypes.c_double, _vp, _vp, _int]),
    "fdb_upwind_std": (_int, [_vp, _dp]),
    "fdb_upwind_set_stream": (_int, [_vp, _vp]),
    "fdb_upwind_set_velocity": (_int, [_vp, _vp]),
    "fdb_upwind_set_arith": (_int, [_vp, _int, _int]),
    "fdb_upwind_set_coeff_form": (_int, [_vp, _int]),
    "fdb_upwind_create_slab": (_int, [_int, _vp, _vp, _vp, ctypes.c_uint64,
                                      ctypes.POINTER(_vp)]),
    "fdb_upwind_get_planes": (_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, _vp, _int]),
    "fdb_upwind_set_planes": (_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, _vp, _int]),
    "fdb_upwind_checksum_planes": (_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, _dp]),
    "fdb_upwind_set_own_planes": (_int, [_vp, ctypes.c_uint64, ctypes.c_uint64]),
    "fdb_upwind_block_begin": (_int, [_vp, ctypes.c_double, ctypes.POINTER(_int)]),
    "fdb_upwind_advect_block": (_int, [_vp, _int, ctypes.c_double, _int]),
    "fdb_upwind_get_scale_word": (_int, [_vp, _vp, _int]),
    "fdb_upwind_set_scale_word": (_int, [_vp, _vp, _int]),
    "fdb_upwind_info": (_int, [_vp, _u64p, ctypes.POINTER(_int)]),
    "fdb_upwind_set_tuning": (_int, [_vp, _int, _int]),
    "fdb_checksum_noalloc": (_int, [_vp, ctypes.c_uint64, _vp, _vp]),
    "fdb_batch_create": (_int, [_int, _vp, ctypes.POINTER(_vp)]),
    "fdb_batch_destroy": (_int, [_vp]),
    "fdb_batch_count": (_int, [_vp, ctypes.POINTER(_int), _u64p]),
    "fdb_batch_storage_order": (_int, [_vp, _int, ctypes.POINTER(_int)]),
    "fdb_batch_adjoint": (_int, [_vp, _int, _vp, _vp, _vp, _vp, _int, _int]),
    "fdb_batch_advect_transposed": (_int, [_vp, _int, _vp, _vp, _vp, _int]),
    "fdb_batch_set_velocity": (_int, [_vp, _int, _vp]),
    "fdb_batch_set_field": (_int, [_vp, _int, _vp, _int]),
    "fdb_batch_get_field": (_int, [_vp, _int, _vp, _int]),
    "fdb_batch_init_sphere": (_int, [_vp, _int, _vp, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_uint64]),
    "fdb_batch_set_stream": (_int, [_vp, _vp]),
    "fdb_batch_set_tuning": (_int, [_vp, _int, _int]),
    "fdb_batch_advect": (_int, [_vp, _int, _vp]),
    "fdb_batch_advect_looped": (_int, [_vp, _int, _vp]),
    "fdb_batch_checksums": (_int, [_vp, _vp]),
    "fdb_batch_autotune": (_int, [_vp, _int, _vp, ctypes.c_char_p, _vp]),
    "fdb_upwind_init_sphere": (_int, [_vp, _vp, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_uint64]),
    "fdb_upwind_adjoint": (_int, [_vp, _int, ctypes.c_double, _vp, _vp, _vp, _int, _int]),
    "fdb_upwind_adjoint_step": (_int, [_vp, ctypes.c_double, _vp, _vp, _vp, _vp]),
    "fdb_upwind_adjoint_timings": (_int, [_vp, _vp]),
    # include/fdb_filter.h
    "fdb_filter_create": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, ctypes.POINTER(_vp)]),
    "fdb_filter_destroy": (_int, [_vp]),
    "fdb_filter_set_in_data": (_int, [_vp, _vp, _int]),
    "fdb_filter_get_data": (_int, [_vp, _int, _vp, _int]),
    "fdb_filter_apply": (_int, [_vp]),
    "fdb_filter_copy_out_to_in": (_int, [_vp]),
    "fdb_filter_iterate": (_int, [_vp, _int]),
    "fdb_filter_checksum": (_int, [_vp, _int, _dp]),
    "fdb_filter_set_wrap": (_int, [_vp, _int]),
    "fdb_filter_set_stream": (_int, [_vp, _vp]),
    "fdb_filter_info": (_int, [_vp, _u64p, ctypes.POINTER(_int)]),
    "fdb_filter_synchronize": (_int, [_vp]),
}


class FdbError(RuntimeError):
    """A non-zero status from libfdb_upwind, with fdb_last_error()'s text."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"fdb error {code}: {msg}")
        self.code = code


def _load() -> ctypes.CDLL:
    if not os.path.isfile(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python fidibench_gb300/build.py` "
            "(the CUDA library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(rc: int) -> None:
    if rc != FDB_OK:
        raise FdbError(rc, lib.fdb_last_error().decode(errors="replace"))


def dptr(a) -> int | None:
    """Address of a contiguous numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
