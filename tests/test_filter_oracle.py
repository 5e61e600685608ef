"""The stencil Filter's CPU restatement (oracle/filter_oracle.c), pinned bit
for bit to the reference's own Filter (cxx/Filter.cpp with CubeDecomp,
MultiArrayIter and writeVTK), which oracle/Makefile compiles for one rank
against the single-rank MPI stand-in oracle/mpi_stub: through the golden
fixtures tests/golden/filter_*.npz that tests/golden/make_golden.py made from
it, and (where it was built here) against the compiled reference directly on
seeded random stencils.  Also known answers read from the reference's sources:

  * the discrete Laplacian of prod_j sin(2 pi x_j) on a periodic power-of-two
    grid is sum_j 2 (cos(2 pi / N_j) - 1) times the input (to rounding);
  * testStencil2d.cxx's case: stencil {(0,0): 0, (1,0): 1, (0,-1): -1} on
    8 x 8 with input 1 on the cells that have a zero index;
  * the terms run in std::map order and a repeated offset keeps its first
    weight;
  * Filter.cpp:238-240 reduces a negative index -m with `%= size_t(N)`,
    giving (2^64 - m) mod N (periodic only for powers of two)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import golden_files, load_golden

FILTER_GOLDEN = golden_files("filter_*.npz")


def golden_stencil(g):
    nd = len(g["dims"])
    offs = [tuple(int(x) for x in o) for o in g["offsets"].reshape(-1, nd)]
    return list(zip(offs, [float(w) for w in g["weights"]]))


@pytest.mark.parametrize("path", FILTER_GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
def test_port_matches_reference_filter_golden(port, path):
    g = load_golden(path)
    dims = [int(x) for x in g["dims"]]
    st = golden_stencil(g)
    f = g["f0"]
    for _ in range(int(g["iterations"])):
        f = port.filter_apply(dims, st, f)
    assert np.array_equal(f, g["out"])
    assert np.array_equal(np.signbit(f), np.signbit(g["out"]))
    assert port.filter_checksum(f) == float(g["sums"][1])


def test_port_matches_compiled_reference_filter(port):
    from oracle.oracle import ReferenceFilter
    if not ReferenceFilter.available():
        pytest.skip("reference Filter not built in this tree")
    ref = ReferenceFilter()
    rng = np.random.default_rng(41)
    for _ in range(10):
        nd = int(rng.integers(1, 4))
        dims = [int(x) for x in rng.integers(2, 9, size=nd)]
        nt = int(rng.integers(1, 6))
        st = [(tuple(int(x) for x in rng.integers(-2, 3, size=nd)), float(rng.normal()))
              for _ in range(nt)]
        f0 = rng.standard_normal(int(np.prod(dims)))
        iters = int(rng.integers(1, 4))
        out, sums = ref.run(dims, st, f0, iters)
        f = f0
        for _ in range(iters):
            f = port.filter_apply(dims, st, f)
        assert np.array_equal(f, out), (dims, st)
        assert port.filter_checksum(f) == sums[1]


def laplacian_stencil(nd):
    """laplacian/cxx/laplacian.cxx:57-66"""
    st = {tuple([0] * nd): -2.0 * nd}
    for i in range(nd):
        o = [0] * nd
        o[i] = 1
        st.setdefault(tuple(o), 1.0)
        o[i] = -1
        st.setdefault(tuple(o), 1.0)
    return st


@pytest.mark.parametrize("dims", [(16,), (32, 16), (8, 16, 32), (4, 4, 4, 4)])
def test_laplacian_of_sines_known_answer(port, dims):
    nd = len(dims)
    f = port.filter_sin_input(dims, [0.0] * nd, [1.0] * nd)
    out = port.filter_apply(dims, laplacian_stencil(nd), f)
    lam = sum(2.0 * (math.cos(2.0 * math.pi / n) - 1.0) for n in dims)
    assert np.max(np.abs(out - lam * f)) <= 8 * nd * np.finfo(float).eps * np.max(np.abs(f))


def test_stencil2d_known_answer(port):
    n = 8
    st = {(0, 0): 0.0, (1, 0): 1.0, (0, -1): -1.0}
    i = np.arange(n * n) % n          # axis 0 (fastest)
    j = np.arange(n * n) // n         # axis 1
    f = ((i * j) == 0).astype(float)
    out = port.filter_apply((n, n), st, f)
    F = f.reshape(n, n)               # F[j, i]
    expect = np.roll(F, -1, axis=1) - np.roll(F, 1, axis=0)
    assert np.array_equal(out.reshape(n, n), expect + 0.0 * F)


def test_map_order_and_first_weight_wins(port):
    offs = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
            (1, 0, 0)]
    assert port.stencil_order(offs) == [2, 4, 6, 0, 5, 3, 1]
    st = [((1,), 2.0), ((0,), 1.0), ((1,), 100.0)]
    x = np.arange(5, dtype=float)
    out = port.filter_apply((5,), st, x, periodic=True)
    assert np.array_equal(out, x + 2.0 * np.roll(x, -1))


@pytest.mark.parametrize("n", [6, 7, 10, 100, 8000])
def test_reference_wrap_of_negative_indices(port, n):
    x = np.arange(n, dtype=float)
    ref = port.filter_apply((n,), {(-1,): 1.0}, x)
    per = port.filter_apply((n,), {(-1,): 1.0}, x, periodic=True)
    assert ref[0] == float((2 ** 64 - 1) % n)
    assert per[0] == float(n - 1)
    assert np.array_equal(ref[1:], per[1:])
    ref2 = port.filter_apply((n,), {(-2,): 1.0}, x)
    assert ref2[0] == float((2 ** 64 - 2) % n) and ref2[1] == float((2 ** 64 - 1) % n)


def test_power_of_two_wrap_is_periodic(port):
    rng = np.random.default_rng(1)
    dims = (16, 8, 4)
    st = {(-1, 0, 0): 0.5, (0, -3, 1): -1.25, (2, 0, -1): 3.0, (0, 0, 0): 1.0}
    f = rng.standard_normal(int(np.prod(dims)))
    assert np.array_equal(port.filter_apply(dims, st, f),
                          port.filter_apply(dims, st, f, periodic=True))


def test_checksum_is_sequential(port):
    f = np.array([1e16, 1.0, -1e16, 1.0])
    assert port.filter_checksum(f) == ((1e16 + 1.0) - 1e16) + 1.0
