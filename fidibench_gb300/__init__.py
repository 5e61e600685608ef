"""fidibench_gb300 -- GB300-native (sm_103a) upwind advection.

The hot path of FiDiBench (Upwind<NDIMS>::advect, upwind/cxx/upwind.cxx:51-86)
as hand-written CUDA behind a plain C-ABI (include/fdb_upwind.h), with the
reference's C++ class rebuilt on top (include/fidibench_gb/Upwind.h) and the
Python class mirrored here (upwind.Upwind).  Importing the package loads the
CUDA library and raises if it is missing: there is no CPU fallback.
"""
from ._capi import FdbError, lib  # noqa: F401  (loads libfdb_upwind.so or raises)
from .upwind import Upwind  # noqa: F401

__all__ = ["Upwind", "FdbError"]
from .batch import Batch  # noqa: F401,E402

__all__.append("Batch")
