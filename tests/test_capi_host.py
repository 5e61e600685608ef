"""The C-ABI library on a host without a GPU: it loads, exports every symbol
that include/*.h declares, and rejects bad arguments before touching CUDA."""
from __future__ import annotations

import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols() -> set[str]:
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fdb_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def capi():
    from fidibench_gb300 import _capi
    return _capi


def test_library_exports_every_declared_symbol(capi):
    names = declared_symbols()
    assert "fdb_upwind_advect" in names and "fdb_upwind_create" in names
    missing = [n for n in sorted(names) if not hasattr(capi.lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(capi):
    assert declared_symbols() <= set(capi.SIGNATURES), \
        declared_symbols() - set(capi.SIGNATURES)


def test_version_and_error_text(capi):
    assert b"sm_103a" in capi.lib.fdb_version()
    assert isinstance(capi.lib.fdb_last_error(), bytes)


@pytest.mark.parametrize("ndims,n,L,v", [
    (0, [4], [1.0], [1.0]),
    (9, [2] * 9, [1.0] * 9, [1.0] * 9),
    (3, [4, 0, 4], [1.0] * 3, [1.0] * 3),
    (3, [4, 4, 4], [1.0, -1.0, 1.0], [1.0] * 3),
    (2, [4, 4], [1.0, 1.0], [float("nan"), 1.0]),
])
def test_create_rejects_invalid_geometry(capi, ndims, n, L, v):
    h = ctypes.c_void_p()
    nn = np.asarray(n + [1] * 9, dtype=np.uint64)
    vv = np.asarray(v + [0.0] * 9, dtype=np.float64)
    ll = np.asarray(L + [1.0] * 9, dtype=np.float64)
    rc = capi.lib.fdb_upwind_create(ndims, vv.ctypes.data, ll.ctypes.data, nn.ctypes.data,
                                    ctypes.byref(h))
    assert rc == capi.FDB_ERR_INVALID
    assert h.value is None
    assert capi.lib.fdb_last_error()


def test_null_handle_is_rejected(capi):
    out = ctypes.c_double()
    assert capi.lib.fdb_upwind_checksum(None, ctypes.byref(out)) == capi.FDB_ERR_INVALID
    assert capi.lib.fdb_upwind_advect(None, 1, 0.1) == capi.FDB_ERR_INVALID
    assert capi.lib.fdb_upwind_destroy(None) == capi.FDB_OK


def test_upwind_class_rejects_mismatched_lengths():
    from fidibench_gb300 import Upwind
    with pytest.raises(ValueError):
        Upwind([1.0, 1.0], [1.0], [4, 4])


def test_cpp_facade_check_compiles(tmp_path):
    """The C++ facade test program builds against the headers and the library
    (it runs in the GPU suite)."""
    import subprocess
    src = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")
    lib_dir = os.path.join(ROOT, "fidibench_gb300", "_lib")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                        src, "-o", str(tmp_path / "facade_check"), "-L", lib_dir,
                        "-lfdb_upwind", "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr
