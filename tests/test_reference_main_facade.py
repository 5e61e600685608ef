"""Drop-in check of the C++ facade: the reference's own driver `main()`
functions, taken from the reference source tree at test time (never copied
into this repository), compile and link unchanged against
include/fidibench_gb/Upwind.h and libfdb_upwind.so, with the reference's
cxx/CmdLineArgParser.cpp.  That is the integration a maintainer performs:
keep the driver, drop the in-file class, include the facade.

  upwind/cxx/upwind.cxx      main() (:139-217): std::vector<size_t> ctor,
                             advect(int, double), checksum(), std(), saveVTK()
  upwind/cxx/upwindAcc.cxx   main() (:117-172): std::vector<int> ctor,
                             advect(double) per step, checksum(), saveVTK()
  upwind/cxx/upwindAcc2.cxx  main() (:137-193): std::vector<int> ctor,
                             advect(int, double), std()

The same for the Filter facade (include/fidibench_gb/Filter.h): the
reference's Filter drivers laplacian/cxx/laplacian.cxx, testStencil2d.cxx and
upwind/cxx/upwindMpi.cxx, whole and unchanged, with the single-rank MPI
stand-in oracle/mpi_stub providing MPI_Init, MPI_Wtime, MPI_Reduce and the
other calls they make outside the Filter.

The built programs run `-h` here (no GPU needed: help only); their numerical
twins, this repository's drivers, run the ctest cases in the GPU suite.  CPU
only; skipped where the reference tree is absent."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT

PRELUDE = """\
#include <vector>
#include <array>
#include <functional>
#include <algorithm>
#include <numeric>
#include <string>
#include <fstream>
#include <limits>
#include <iostream>
#include <sstream>
#include <cstring>
#include <cmath>
#include "CmdLineArgParser.h"
#include "fidibench_gb/Upwind.h"
"""


def _refdir() -> str:
    from oracle.oracle import reference_dir
    return reference_dir()


def _main_of(path: str) -> str:
    """The text of the file from its `int main(` line to the end."""
    lines = open(path).read().splitlines(keepends=True)
    for k, ln in enumerate(lines):
        if ln.startswith("int main("):
            return "".join(lines[k:])
    raise AssertionError(f"no `int main(` in {path}")


@pytest.fixture(scope="module")
def lib_dir():
    from fidibench_gb300 import build
    build.build()
    return os.path.join(ROOT, "fidibench_gb300", "_lib")


@pytest.mark.parametrize("src", ["upwind.cxx", "upwindAcc.cxx", "upwindAcc2.cxx"])
def test_reference_main_builds_against_facade(src, lib_dir, tmp_path):
    refdir = _refdir()
    path = os.path.join(refdir, "upwind", "cxx", src)
    if not os.path.isfile(path):
        pytest.skip("the reference source tree is not present")
    tu = tmp_path / ("main_" + src.replace(".cxx", ".cpp"))
    tu.write_text(PRELUDE + "\n" + _main_of(path))
    exe = tmp_path / src.replace(".cxx", "")
    r = subprocess.run(
        ["g++", "-std=c++17", "-O1", "-w", "-I", os.path.join(ROOT, "include"),
         "-I", os.path.join(refdir, "cxx"), str(tu),
         os.path.join(refdir, "cxx", "CmdLineArgParser.cpp"), "-o", str(exe),
         "-L", lib_dir, "-lfdb_upwind", "-Wl,-rpath," + lib_dir],
        capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
    h = subprocess.run([str(exe), "-h"], capture_output=True, text=True, timeout=60)
    assert h.returncode == 0, h.stderr
    assert "-numCells" in h.stdout


@pytest.mark.parametrize("src", ["laplacian/cxx/laplacian.cxx", "laplacian/cxx/testStencil2d.cxx",
                                 "upwind/cxx/upwindMpi.cxx"])
def test_reference_filter_driver_builds_against_facade(src, lib_dir, tmp_path):
    refdir = _refdir()
    path = os.path.join(refdir, src)
    if not os.path.isfile(path):
        pytest.skip("the reference source tree is not present")
    stub = os.path.join(ROOT, "oracle", "mpi_stub")
    obj = tmp_path / "mpi_stub.o"
    r = subprocess.run(["gcc", "-std=c11", "-O1", "-D_POSIX_C_SOURCE=199309L", "-I", stub, "-c",
                        os.path.join(stub, "mpi_stub.c"), "-o", str(obj)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / os.path.basename(src).replace(".cxx", "")
    # include/fidibench_gb first: the driver's "Filter.h" is the facade
    r = subprocess.run(
        ["g++", "-std=c++17", "-O1", "-w", "-I", os.path.join(ROOT, "include", "fidibench_gb"),
         "-I", os.path.join(ROOT, "include"), "-I", stub, "-I", os.path.join(refdir, "cxx"),
         path, os.path.join(refdir, "cxx", "CmdLineArgParser.cpp"), str(obj), "-o", str(exe),
         "-L", lib_dir, "-lfdb_upwind", "-Wl,-rpath," + lib_dir],
        capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
    h = subprocess.run([str(exe), "-h"], capture_output=True, text=True, timeout=60)
    assert h.returncode == 0, h.stderr
    assert "-numCells" in h.stdout
