"""Host check of the block-fixed-point helpers (fidibench_gb300/csrc/
fixed_point.cuh, shared by host and device code): the IEEE bit-pattern
conversions against exact rational arithmetic, and the Q1.62 product's
error bound.  Compiled with g++ into a throwaway library; CPU only."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

from conftest import ROOT

SRC = r"""
#include <stdint.h>
#include "fixed_point.cuh"
extern "C" {
int64_t t_to_fixed(double f, int s) { return fdb::to_fixed(f, s); }
double t_to_double(int64_t F, int s) { return fdb::to_double(F, s); }
void t_qcoeff(double a, int32_t* a1, int32_t* a0) {
  fdb::QCoeff q = fdb::make_qcoeff(a); *a1 = q.a1; *a0 = q.a0;
}
// the kernels' cell update (the same source, compiled for the host)
int64_t t_update(int64_t c, int64_t zb, int64_t up, int64_t left, const double* a) {
  return fdb::fixed_update(c, zb, up, left, fdb::make_qcoeff(a[0]), fdb::make_qcoeff(a[1]),
                           fdb::make_qcoeff(a[2]));
}
}
"""


@pytest.fixture(scope="module")
def fx():
    d = tempfile.mkdtemp()
    src = os.path.join(d, "t.cpp")
    so = os.path.join(d, "t.so")
    with open(src, "w") as fh:
        fh.write(SRC)
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "fidibench_gb300", "csrc"), src, "-o", so], check=True)
    lib = ctypes.CDLL(so)
    lib.t_to_fixed.argtypes = [ctypes.c_double, ctypes.c_int]
    lib.t_to_fixed.restype = ctypes.c_int64
    lib.t_to_double.argtypes = [ctypes.c_int64, ctypes.c_int]
    lib.t_to_double.restype = ctypes.c_double
    lib.t_qcoeff.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_int32),
                             ctypes.POINTER(ctypes.c_int32)]
    lib.t_update.argtypes = [ctypes.c_int64] * 4 + [ctypes.POINTER(ctypes.c_double)]
    lib.t_update.restype = ctypes.c_int64
    return lib


def test_to_fixed_matches_exact_rounding(fx):
    rng = np.random.default_rng(1)
    vals = list(rng.standard_normal(300)) + list(rng.random(300) * 1e-12) + \
        [0.0, -0.0, 1.0, -1.0, 0.5, 1e-300, 5e-324, 0.99999999999999989]
    for s in (58, 60, 40, 70):
        for f in vals:
            F = fx.t_to_fixed(float(f), s)
            exact = Fraction(float(f)) * (Fraction(2) ** s)
            if float(f) != 0.0 and abs(float(f)) < 2.0 ** -1022:
                assert F == 0  # subnormals flush
                continue
            if abs(exact) >= 2 ** 60:
                continue  # outside the kernel's range (the scale keeps |F| < 2^60)
            assert abs(Fraction(F) - exact) <= Fraction(1, 2), (f, s, F)


def test_to_double_is_correctly_rounded(fx):
    rng = np.random.default_rng(2)
    Fs = [int(x) for x in rng.integers(-(1 << 62), 1 << 62, size=400)] + \
        [1, -1, 3, (1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6, (1 << 62) - 1, 0]
    for s in (60, 58, 0, -5, 1000):
        for F in Fs:
            d = fx.t_to_double(F, s)
            want = float(Fraction(F) / (Fraction(2) ** s)) if F else 0.0
            assert d == want, (F, s, d, want)


def test_round_trip_exact_for_53_bit_values(fx):
    rng = np.random.default_rng(3)
    for f in rng.uniform(-1, 1, size=500):
        F = fx.t_to_fixed(float(f), 60)
        assert fx.t_to_double(F, 60) == float(f)


@pytest.mark.parametrize("a", [0.0, 0.5, 0.35, 0.15, 1.0, 0.8 * 0.5, 1e-7, 0.999999999])
def test_qcoeff_halves(fx, a):
    a1 = ctypes.c_int32()
    a0 = ctypes.c_int32()
    fx.t_qcoeff(a, ctypes.byref(a1), ctypes.byref(a0))
    A = (a1.value << 32) + a0.value
    assert abs(Fraction(A) - Fraction(a) * 2 ** 62) < 1
    assert 0 <= a1.value <= 1 << 30 and -(1 << 31) <= a0.value < 1 << 31


@pytest.mark.parametrize("a", [(0.5, 0.35, 0.15), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0),
                               (1e-7, 0.999999999, 0.4), (0.3, 0.0, 1.0)])
def test_update_error_bound(fx, a):
    """F' within 8 units of F + sum_j a_j D_j (the Q1.62 coefficients), also at
    the range limits |F| < 2^59, and exactly F when every difference is 0."""
    q = []
    for aj in a:
        a1 = ctypes.c_int32()
        a0 = ctypes.c_int32()
        fx.t_qcoeff(aj, ctypes.byref(a1), ctypes.byref(a0))
        q.append((a1.value << 32) + a0.value)
    av = (ctypes.c_double * 3)(*a)
    lim = (1 << 59) - 1
    rng = np.random.default_rng(5)
    cases = [tuple(int(x) for x in rng.integers(-lim, lim, size=4, endpoint=True))
             for _ in range(400)]
    cases += [(lim, -lim, -lim, -lim), (-lim, lim, lim, lim), (0, lim, -lim, lim),
              (lim, lim, lim, lim), (-lim, -lim, -lim, -lim), (12345, 12345, 12345, 12345)]
    for c, zb, up, left in cases:
        got = fx.t_update(c, zb, up, left, av)
        exact = c + Fraction(4 * sum(A * (u - c) for A, u in zip(q, (zb, up, left))), 1 << 64)
        assert abs(Fraction(got) - exact) <= 8, (a, c, zb, up, left)
        if zb == up == left == c:
            assert got == c
