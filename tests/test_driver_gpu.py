"""The reference's ctest cases and CLI contract, run against the upwindCxx
driver built on the C++ facade (include/fidibench_gb/Upwind.h).

upwind/cxx/CMakeLists.txt:54-91 registers `upwindCxx 32 10` under
OMP_NUM_THREADS = 1, 2, 4, 8 and unset, passing when stdout matches
"[Cc]heck sum:[ ]*[1|0\\.999]" (the positional 32 10 are ignored by the
reference's parser, so every case runs the default 128^3 x 10)."""
from __future__ import annotations

import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "fidibench_gb300", "_lib", "upwindCxx")
CTEST_REGEX = re.compile(r"[Cc]heck sum:[ ]*[1|0\.999]")


def run(args, cwd=None, env=None):
    return subprocess.run([EXE] + list(args), capture_output=True, text=True, cwd=cwd,
                          env=dict(os.environ, **(env or {})), timeout=300)


@pytest.mark.parametrize("threads", [None, "1", "2", "4", "8"])
def test_ctest_upwindCxx_cases(threads):
    r = run(["32", "10"], env={} if threads is None else {"OMP_NUM_THREADS": threads})
    assert r.returncode == 0, r.stderr
    assert CTEST_REGEX.search(r.stdout), r.stdout
    assert "number of cells:  128 128 128" in r.stdout
    assert "number of time steps: 10" in r.stdout


def test_std_line_matches_reference_driver():
    g = load_golden("driver_128cube_10")
    r = run(["-std", "-arith", "exact"])
    assert r.returncode == 0, r.stderr
    assert "check sum: 1\n" in r.stdout
    assert f"std      : {float(g['std']):g}" in r.stdout


@pytest.mark.parametrize("arith", ["exact", "auto"])
def test_vtk_output_matches_reference_writer(tmp_path, arith):
    g = load_golden("driver_vtk_6cube_3")
    r = run(["-numCells", "6", "-numSteps", "3", "-vtk", "-std", "-arith", arith],
            cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    ours = (tmp_path / "up1.vtk").read_text()
    if arith == "exact":
        assert ours == str(g["up1_vtk"])
    else:
        assert ours.splitlines()[:13] == str(g["up1_vtk"]).splitlines()[:13]
    ref_lines = [ln for ln in str(g["stdout"]).splitlines() if ln.startswith(("check", "std"))]
    for ln in ref_lines:
        assert ln in r.stdout
    assert (tmp_path / "up0.vtk").exists()


def test_invalid_option_prints_help():
    r = run(["-bogus"])
    assert "-bogus is not a valid option." in r.stdout
    assert "ERROR when parsing command line arguments" in r.stderr


def test_python_mirror_vtk_matches(tmp_path, fdb):
    g = load_golden("driver_vtk_6cube_3")
    from oracle import reference_dt
    up = fdb.Upwind([1.0] * 3, [1.0] * 3, [6] * 3, arith="exact")
    up.advect(3, reference_dt([6] * 3, [1.0] * 3, [1.0] * 3, 0.1))
    up.saveVTK(str(tmp_path / "py.vtk"))
    ours = (tmp_path / "py.vtk").read_text()
    ref = str(g["up1_vtk"])
    # same layout and values; the Python writer titles the file "upwind"
    assert ours.splitlines()[2:] == ref.splitlines()[2:]
    up.close()
    assert np.isfinite(up.ntot)


def test_python_cli_matches_reference_contract(tmp_path):
    """`python -m fidibench_gb300.upwind N S [vtk]`: the reference Python
    driver's command line and output lines (upwind/python/upwind.py:88-126;
    ctest upwindPython regex `[Cc]heck sum:[ ]*[1\\.0|0\\.999]`)."""
    import sys
    r = subprocess.run([sys.executable, "-m", "fidibench_gb300.upwind", "32", "10", "vtk"],
                       cwd=tmp_path, env={**os.environ, "PYTHONPATH": ROOT},
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "number of cells:  [32, 32, 32]"
    assert lines[1] == "number of time steps:  10"
    assert re.search(r"[Cc]heck sum:[ ]*[1\.0|0\.999]", lines[2])
    assert abs(float(lines[2].split()[-1]) - 1.0) < 1e-12
    assert (tmp_path / "up.vtk").exists()
    r = subprocess.run([sys.executable, "-m", "fidibench_gb300.upwind"], cwd=tmp_path,
                       env={**os.environ, "PYTHONPATH": ROOT}, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 1
    assert "must specify number of cells" in r.stdout


def test_driver_adjoint_matches_python(fdb):
    """`upwindCxx -velocity ... -adjoint` (the C++ facade's adjoint) against
    the Python mirror's adjoint on the same problem: the reference driver's
    32^3 grid, f0 = corner mass, L = 0.5 sum f_T^2."""
    r = run(["-numCells", "32", "-numSteps", "12", "-velocity", "0.8,0.5,-0.6", "-adjoint"])
    assert r.returncode == 0, r.stderr
    out = r.stdout
    gv_line = next(line for line in out.splitlines() if line.startswith("dL/dv:"))
    gv = np.array([float(x) for x in gv_line.split()[1:]])
    g_line = next(line for line in out.splitlines() if line.startswith("|dL/df0|:"))
    g_norm = float(g_line.split()[-1])
    v, n = (0.8, 0.5, -0.6), (32, 32, 32)
    dt = min(0.1 * (1.0 / 32) / abs(x) for x in v)
    up = fdb.Upwind(v, (1.0, 1.0, 1.0), n)
    f0 = up.f
    up.advect(12, dt)
    lam = up.f
    up.f = f0
    g0, gv_ref = up.adjoint(12, dt, lam)
    up.close()
    assert np.allclose(gv, gv_ref, rtol=1e-12, atol=0.0)
    assert g_norm == pytest.approx(float(np.linalg.norm(g0)), rel=1e-12)


def test_cpp_facade_additions(tmp_path):
    """tests/cpp/facade_check.cpp: advectHostStream against the serial cycle
    and advectTransposed against the dL/df0-only adjoint, bit for bit."""
    src = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")
    lib_dir = os.path.join(ROOT, "fidibench_gb300", "_lib")
    exe = str(tmp_path / "facade_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o",
                    exe, "-L", lib_dir, "-lfdb_upwind", "-Wl,-rpath," + lib_dir], check=True,
                   timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok" in r.stdout


ACC_EXE = {name: os.path.join(ROOT, "fidibench_gb300", "_lib", name)
           for name in ("upwindAccCxx", "upwindAcc2Cxx")}


@pytest.mark.parametrize("name", ["upwindAccCxx", "upwindAcc2Cxx"])
def test_ctest_acc_cases(name):
    """upwind/cxx/CMakeLists.txt:93-107: `upwindAccCxx 32 10` and
    `upwindAcc2Cxx 32 10`, same regex; the positional tokens are ignored, so
    both run the default 128^3 x 10 (one advect(dt) call per step for Acc)."""
    r = subprocess.run([ACC_EXE[name], "32", "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert CTEST_REGEX.search(r.stdout), r.stdout
    assert "number of cells:  128 128 128" in r.stdout
    assert "number of time steps: 10" in r.stdout


@pytest.mark.parametrize("name,golden", [("upwindAccCxx", "acc1_16cube_10"),
                                         ("upwindAcc2Cxx", "acc2_16cube_10")])
def test_acc_driver_vtk_matches_reference_variant(tmp_path, fdb, name, golden):
    """The driver's up.vtk under EXACT holds the reference variant's field
    (the golden fixture, written with the same ASCII layout by the Python
    mirror's writer for comparison)."""
    g = load_golden(golden)
    args = [ACC_EXE[name], "-numCells", "16", "-numSteps", "10", "-vtk", "-arith", "exact"]
    if name == "upwindAcc2Cxx":
        args.append("-std")
    r = subprocess.run(args, capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "check sum: 1\n" in r.stdout
    if name == "upwindAcc2Cxx":
        assert "std      : " in r.stdout
    from fidibench_gb300.vtk import write_rectilinear
    n = [int(x) for x in g["n"]]
    write_rectilinear(str(tmp_path / "ref.vtk"), n, [1.0 / x for x in n], g["fT"],
                      title="upwind.cxx")
    assert (tmp_path / "up.vtk").read_text() == (tmp_path / "ref.vtk").read_text()


def test_acc_driver_rejects_bad_option():
    r = subprocess.run([ACC_EXE["upwindAccCxx"], "-std"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1
    assert "-std is not a valid option." in r.stdout
    assert "ERROR: wrong command line arguments" in r.stderr
