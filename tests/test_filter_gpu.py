"""Parity of the GPU stencil Filter (include/fdb_filter.h, csrc/filter.cu) with
the CPU restatement of the reference's Filter (oracle/filter_oracle.c): the
output must be bit-identical (same terms in std::map order, every product and
sum separately rounded), in both wrap modes, on the 3-axis fast path and the
generic kernel; plus the laplacian driver's command-line contract."""
from __future__ import annotations

import math
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

LAPLACIAN = os.path.join(ROOT, "fidibench_gb300", "_lib", "laplacian")


def run_filter(dims, stencil, f0, periodic=False, applies=1):
    from fidibench_gb300.filter import Filter, WRAP_PERIODIC, WRAP_REFERENCE
    nd = len(dims)
    flt = Filter(dims, [0.0] * nd, [1.0] * nd, stencil,
                 wrap=WRAP_PERIODIC if periodic else WRAP_REFERENCE)
    flt.set_in_data(f0)
    for k in range(applies):
        flt.applyFilter()
        if k + 1 < applies:
            flt.copyOutToIn()
    out = flt.out_data
    cs = flt.computeCheckSum("output")
    flt.close()
    return out, cs


def oracle_applies(port, dims, stencil, f0, periodic=False, applies=1):
    f = np.array(f0, dtype=float)
    for _ in range(applies):
        f = port.filter_apply(dims, stencil, f, periodic=periodic)
    return f


def laplacian(nd):
    from fidibench_gb300.filter import laplacian_stencil
    return laplacian_stencil(nd)


@pytest.mark.parametrize("name", ["filter_lap16x16_it1", "filter_lap10x12_it1",
                                  "filter_lap6x5x7_it1", "filter_lap16x16_it10",
                                  "filter_stencil2d_8", "filter_upwindmpi_16_it10",
                                  "filter_general_7x5x6"])
def test_matches_reference_filter_golden(name):
    """The reference's own Filter (one rank), bit for bit."""
    from conftest import load_golden
    g = load_golden(name)
    dims = [int(x) for x in g["dims"]]
    nd = len(dims)
    st = list(zip([tuple(int(x) for x in o) for o in g["offsets"].reshape(-1, nd)],
                  [float(w) for w in g["weights"]]))
    out, cs = run_filter(dims, st, g["f0"], applies=int(g["iterations"]))
    assert np.array_equal(out, g["out"])
    assert np.array_equal(np.signbit(out), np.signbit(g["out"]))
    assert cs == pytest.approx(float(g["sums"][1]), rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("dims", [(64, 64), (100, 37), (16, 24, 40), (33, 7, 5), (1000,),
                                  (8, 8, 8)])
def test_laplacian_bit_identical(port, dims, periodic):
    nd = len(dims)
    f0 = port.filter_sin_input(dims, [0.0] * nd, [1.0] * nd)
    out, cs = run_filter(dims, laplacian(nd), f0, periodic, applies=3)
    ref = oracle_applies(port, dims, laplacian(nd), f0, periodic, applies=3)
    assert np.array_equal(out, ref)
    assert np.array_equal(np.signbit(out), np.signbit(ref))
    assert cs == pytest.approx(port.filter_checksum(ref), abs=1e-12 * np.sum(np.abs(ref)) + 1e-300)


@pytest.mark.parametrize("seed", range(6))
def test_random_stencils_bit_identical(port, seed):
    rng = np.random.default_rng(seed)
    nd = int(rng.integers(1, 4))
    dims = tuple(int(x) for x in rng.integers(3, 40, size=nd))
    nterms = int(rng.integers(1, 12))
    st = []
    for _ in range(nterms):
        off = tuple(int(x) for x in rng.integers(-5, 6, size=nd))
        w = float(rng.choice([1.0, -1.0, 0.0, rng.standard_normal(), 2.5, -6.0]))
        st.append((off, w))
    f0 = rng.standard_normal(int(np.prod(dims)))
    f0[rng.integers(0, f0.size, size=3)] = -0.0
    for periodic in (False, True):
        out, _ = run_filter(dims, st, f0, periodic)
        ref = port.filter_apply(dims, st, f0, periodic=periodic)
        assert np.array_equal(out, ref)
        assert np.array_equal(np.signbit(out), np.signbit(ref))


@pytest.mark.parametrize("dims", [(4, 3, 5, 2), (3, 2, 2, 3, 2)])
def test_generic_kernel_more_axes(port, dims):
    nd = len(dims)
    rng = np.random.default_rng(nd)
    f0 = rng.standard_normal(int(np.prod(dims)))
    for periodic in (False, True):
        out, _ = run_filter(dims, laplacian(nd), f0, periodic)
        assert np.array_equal(out, port.filter_apply(dims, laplacian(nd), f0, periodic=periodic))


def test_many_terms_generic_path(port):
    """More terms than the fast path's table: the generic kernel."""
    dims = (20, 12)
    st = [((i, j), 0.01 * (i + 3 * j)) for i in range(-3, 4) for j in range(-3, 3)]
    assert len(st) > 32
    f0 = np.random.default_rng(3).standard_normal(240)
    out, _ = run_filter(dims, st, f0)
    assert np.array_equal(out, port.filter_apply(dims, st, f0))


def test_iterate_equals_apply_copy_loop(port):
    from fidibench_gb300.filter import Filter
    dims = (48, 40)
    f0 = port.filter_sin_input(dims, [0, 0], [1, 1])
    a = Filter(dims, [0, 0], [1, 1], laplacian(2))
    a.set_in_data(f0)
    a.iterate(5)
    b = Filter(dims, [0, 0], [1, 1], laplacian(2))
    b.set_in_data(f0)
    for _ in range(5):
        b.applyFilter()
        b.copyOutToIn()
    for x, y in ((a.in_data, b.in_data), (a.out_data, b.out_data), (a.in_data, a.out_data)):
        assert np.array_equal(x, y)
    assert np.array_equal(a.out_data, oracle_applies(port, dims, laplacian(2), f0, applies=5))
    a.close()
    b.close()


def test_set_in_data_by_function_matches_reference_positions(port):
    from fidibench_gb300.filter import Filter, sin_input
    dims = (6, 5)
    flt = Filter(dims, [0, 0], [1, 1], laplacian(2))
    flt.setInData(sin_input)
    assert np.allclose(flt.in_data, port.filter_sin_input(dims, [0, 0], [1, 1]), rtol=0,
                       atol=1e-15)
    assert flt.getPosition([0, 4]) == [0.5 / 6, 4.5 / 5]
    flt.close()


def test_known_answer_laplacian_of_sines():
    from fidibench_gb300.filter import Filter, WRAP_PERIODIC
    dims = (64, 32, 16)
    flt = Filter(dims, [0] * 3, [1] * 3, laplacian(3), wrap=WRAP_PERIODIC)
    x = [(np.arange(n) + 0.5) / n for n in dims]
    f = (np.sin(2 * np.pi * x[0])[None, None, :] * np.sin(2 * np.pi * x[1])[None, :, None] *
         np.sin(2 * np.pi * x[2])[:, None, None]).reshape(-1)
    flt.set_in_data(f)
    flt.applyFilter()
    lam = sum(2.0 * (math.cos(2.0 * math.pi / n) - 1.0) for n in dims)
    assert np.max(np.abs(flt.out_data - lam * f)) < 1e-14
    flt.close()


def test_errors_are_reported():
    from fidibench_gb300 import FdbError
    from fidibench_gb300.filter import Filter
    with pytest.raises(FdbError):
        Filter((0, 4), [0, 0], [1, 1], {(0, 0): 1.0})
    with pytest.raises(ValueError):
        Filter((4, 4), [0, 0], [1, 1], {(0,): 1.0})
    flt = Filter((4, 4), [0, 0], [1, 1], {(0, 0): 1.0})
    with pytest.raises(FdbError):
        flt.set_wrap(7)
    flt.close()


@pytest.mark.parametrize("nd,n", [(2, 64), (3, 24)])
def test_laplacian_driver_ctest_contract(port, nd, n):
    """laplacian/cxx/CMakeLists.txt: `laplacian -numDims 2|3 -numCells N`,
    PASS_REGULAR_EXPRESSION "[Cc]heck sums:[ ]*"."""
    r = subprocess.run([LAPLACIAN, "-numDims", str(nd), "-numCells", str(n)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "Number of procs: 1"
    assert lines[1] == "global dimensions: " + " ".join([str(n)] * nd) + " "
    assert lines[2] == "Domain decomp " + "1 " * nd
    assert re.match(r"Laplace times min/max/avg: \S+/\S+/\S+ \[seconds\]", lines[3])
    assert re.search(r"[Cc]heck sums:[ ]*", lines[4])
    m = re.match(r"Check sums: input = (\S+) output = (\S+)", lines[4])
    dims = (n,) * nd
    f = oracle_applies(port, dims, laplacian(nd),
                       port.filter_sin_input(dims, [0] * nd, [1] * nd), applies=10)
    # the driver prints 6 significant digits (C++ stream defaults)
    want = port.filter_checksum(f)
    tol = 1e-12 * np.sum(np.abs(f)) + 5e-6 * abs(want)
    assert abs(float(m.group(1)) - want) <= tol
    assert abs(float(m.group(2)) - want) <= tol


def test_laplacian_driver_vtk_matches_python_writer(tmp_path, port):
    r = subprocess.run([LAPLACIAN, "-numDims", "2", "-numCells", "6", "-vtk"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Data will be written to file laplacian.vtk" in r.stdout
    from fidibench_gb300.vtk import write_structured_filter
    f = oracle_applies(port, (6, 6), laplacian(2),
                       port.filter_sin_input((6, 6), [0, 0], [1, 1]), applies=10)
    write_structured_filter(str(tmp_path / "py.vtk"), (6, 6), [0, 0], [1, 1], f, "outData")
    assert (tmp_path / "laplacian.vtk").read_text() == (tmp_path / "py.vtk").read_text()


def _driver(name, args, cwd=None):
    exe = os.path.join(ROOT, "fidibench_gb300", "_lib", name)
    return subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=300,
                          cwd=cwd)


def _golden_lines(key):
    from conftest import load_golden
    return str(load_golden("filterdrivers_stdout")[key]).splitlines()


@pytest.mark.parametrize("key,args", [("laplacian_2d_16", ["-numCells", "16", "-numDims", "2"]),
                                      ("laplacian_3d_8", ["-numCells", "8", "-numDims", "3"])])
def test_laplacian_driver_matches_reference_output(key, args):
    """The reference laplacian driver's output (built unmodified for one rank
    on the MPI stand-in): the same lines; the check sums of this sine field
    cancel to ~1e-13, so they agree to that absolute level (the reference
    sums sequentially, the library by a fixed tree)."""
    r = _driver("laplacian", args)
    assert r.returncode == 0, r.stderr
    ours = [ln for ln in r.stdout.splitlines() if "times" not in ln]
    ref = _golden_lines(key)
    assert ours[:-1] == ref[:-1]
    a = [float(x) for x in re.findall(r"= ([-+0-9.e]+)", ours[-1])]
    b = [float(x) for x in re.findall(r"= ([-+0-9.e]+)", ref[-1])]
    assert len(a) == len(b) == 2
    assert all(abs(x - y) <= 1e-12 for x, y in zip(a, b)), (ours[-1], ref[-1])


def test_teststencil2d_driver_matches_reference_output():
    r = _driver("testStencil2d", ["-numCells", "8"])
    assert r.returncode == 0, r.stderr
    assert (r.stdout + r.stderr).splitlines() == _golden_lines("teststencil2d_8")


def test_upwindmpi_driver_matches_reference_output(tmp_path):
    """upwindMpiCxx -numCells 16 -numSteps 5: every line of the reference's
    one-rank run (the step as a Filter stencil, per-step check sums)."""
    r = _driver("upwindMpiCxx", ["-numCells", "16", "-numSteps", "5", "-vtk"],
                cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    ours = [ln for ln in r.stdout.splitlines() if "times" not in ln and "Data will" not in ln]
    assert ours == _golden_lines("upwindmpi_16_5")
    assert (tmp_path / "upMpi.vtk").exists()
