"""In-tree build of libfdb_upwind.so and the upwindCxx driver.

    python fidibench_gb300/build.py          # or __graft_entry__.build()

Every CUDA translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into
``fidibench_gb300/_lib/libfdb_upwind.so`` (static CUDA runtime, plain C ABI).
The C++ driver ``drivers/upwindCxx.cpp`` (the reference's CLI on top of the
C++ facade ``include/fidibench_gb/Upwind.h``) is linked against it.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_lib", "obj")
LIB = os.path.join(PKG, "_lib", "libfdb_upwind.so")
DRIVER = os.path.join(PKG, "_lib", "upwindCxx")
DRIVERS = ("upwindCxx", "upwindAccCxx", "upwindAcc2Cxx", "upwindMpiCxx", "laplacian", "testStencil2d")  # drivers/<name>.cpp -> _lib/<name>
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfdb_upwind")
    return cand


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _run(cmd) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if os.environ.get("FDB_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)


def cuda_flags(extra=()) -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + INCLUDE, "-I" + CSRC] + list(extra)


def build(force: bool = False, verbose: bool = False) -> str:
    if verbose:
        os.environ["FDB_BUILD_VERBOSE"] = "1"
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    hdr_time = _newest(headers)
    extra = ["-Xptxas", "-v"] if os.environ.get("FDB_PTXAS_VERBOSE") else []

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
                os.path.getmtime(src), hdr_time):
            _run([nvcc] + cuda_flags(extra) + ["-c", src, "-o", obj])
        return obj

    workers = min(len(sources), os.cpu_count() or 4) or 1
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, sources))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)

    for name in DRIVERS:
        drv_src = os.path.join(PKG, "drivers", name + ".cpp")
        exe = os.path.join(PKG, "_lib", name)
        deps = [drv_src, LIB] + glob.glob(os.path.join(INCLUDE, "fidibench_gb", "*.h")) + \
            glob.glob(os.path.join(INCLUDE, "*.h")) + \
            glob.glob(os.path.join(PKG, "drivers", "*.h"))
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < _newest(deps):
            _run(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, drv_src, "-o", exe,
                  "-L" + os.path.dirname(LIB), "-lfdb_upwind", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
