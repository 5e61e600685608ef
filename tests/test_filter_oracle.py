"""The stencil Filter's CPU restatement (oracle/filter_oracle.c) against known
answers read from the reference's sources (cxx/Filter.cpp, laplacian/cxx/):
the reference's Filter needs MPI, which this image lacks, so it is not run.

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
