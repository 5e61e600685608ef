"""The oracle itself: pinned against the reference's golden vectors, the
reference harness (when built here), and analytic known answers.  CPU only."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_maxnorm

FIELD_CASES = [p for p in golden_files("g*.npz")]


@pytest.mark.parametrize("path", FIELD_CASES, ids=lambda p: p.split("/")[-1][:-4])
def test_port_matches_golden_bit_exact(port, path):
    g = load_golden(path)
    out = port.advect(g["n"], g["v"], g["L"], g["f0"], int(g["steps"]), float(g["dt"]))
    assert np.array_equal(out, g["fT"]), rel_maxnorm(out, g["fT"])
    assert port.checksum(out) == float(g["checksum"])
    assert port.std(out) == float(g["std"])


@pytest.mark.parametrize("threads", [1, 2, 4])
def test_port_thread_count_independent(port, threads):
    g = load_golden("g3_7x5x6_mixed")
    out = port.advect(g["n"], g["v"], g["L"], g["f0"], int(g["steps"]), float(g["dt"]),
                      threads=threads)
    assert np.array_equal(out, g["fT"])


def test_driver_golden_32(port):
    """The reference driver's own run: corner IC, courant 0.1 (upwind.cxx:174-199)."""
    g = load_golden("driver_32cube_10")
    n = [int(x) for x in g["n"]]
    f0 = np.zeros(int(np.prod(n)))
    f0[0] = 1.0
    out = port.advect(n, [1.0] * 3, [1.0] * 3, f0, int(g["steps"]), float(g["dt"]))
    assert np.array_equal(out[g["idx"]], g["values"])
    assert port.checksum(out) == float(g["checksum"])
    assert port.std(out) == float(g["std"])
    assert np.count_nonzero(out) == int(g["nonzero"])


def multinomial(a, b, c, n, cz, cy, cx):
    k = n - a - b - c
    if k < 0:
        return 0.0
    coef = math.factorial(n) // (math.factorial(a) * math.factorial(b) * math.factorial(c)
                                 * math.factorial(k))
    return coef * cz ** a * cy ** b * cx ** c * (1 - cz - cy - cx) ** k


def test_known_answer_point_mass(port):
    """Before the mass wraps around, the corner point mass spreads as a
    multinomial: f(a,b,c) = n!/(a!b!c!k!) c0^a c1^b c2^c (1-sum c)^k."""
    N, steps = 24, 10
    n = (N, N, N)
    dt = 0.1 / N
    f0 = np.zeros(N ** 3)
    f0[0] = 1.0
    out = port.advect(n, [1.0] * 3, [1.0] * 3, f0, steps, dt).reshape(n)
    for (a, b, c) in [(0, 0, 0), (0, 0, 1), (1, 2, 3), (10, 0, 0), (3, 3, 4), (2, 5, 1)]:
        assert out[a, b, c] == pytest.approx(multinomial(a, b, c, steps, 0.1, 0.1, 0.1),
                                             rel=1e-12, abs=1e-300)
    assert out[0, 0, 0] == pytest.approx(0.7 ** 10, rel=1e-14)
    assert float(np.sum(out)) == pytest.approx(1.0, rel=1e-14)


def test_reference_ctest_known_values():
    g = load_golden("driver_128cube_10")
    # f[0] = 0.7^10 and f[(0,0,1)] = 10 * 0.1 * 0.7^9 at 128^3 x 10 (courant 0.1)
    assert g["values"][0] == pytest.approx(0.0282475249, rel=1e-14)
    assert g["values"][1] == pytest.approx(0.040353607, rel=1e-14)
    assert float(g["checksum"]) == pytest.approx(1.0, rel=1e-14)
    assert float(g["std"]) == pytest.approx(0.00011898287050402086, rel=1e-14)


def test_port_matches_reference_harness_random(port, reference):
    rng = np.random.default_rng(7)
    for _ in range(6):
        nd = int(rng.integers(1, 4))
        n = tuple(int(x) for x in rng.integers(1, 9, size=nd))
        v = tuple(float(x) for x in rng.uniform(-1, 1, size=nd))
        L = tuple(float(x) for x in rng.uniform(0.5, 2, size=nd))
        f0 = rng.standard_normal(int(np.prod(n)))
        steps = int(rng.integers(0, 12))
        dt = 0.3 * min(Lj / nj for Lj, nj in zip(L, n))
        a = port.advect(n, v, L, f0, steps, dt)
        b = reference.advect(n, v, L, f0, steps, dt)
        assert np.array_equal(a, b)
        assert port.checksum(a) == reference.checksum(n, a)


@pytest.mark.parametrize("name", ["acc1_16cube_10", "acc2_16cube_10", "acc2_7x5x6_mixed"])
def test_port_product_form_matches_acc_golden_bit_exact(port, name):
    """The product coefficient form (dt * (v*up/dx)) restates the OpenACC
    variants upwindAcc.cxx / upwindAcc2.cxx bit for bit."""
    g = load_golden(name)
    n = [int(x) for x in g["n"]]
    if "f0" in g:
        f0 = g["f0"]
    else:
        f0 = np.zeros(int(np.prod(n)))
        f0[0] = 1.0
    out = port.advect(n, g["v"], g["L"], f0, int(g["steps"]), float(g["dt"]), coeff_form=1)
    assert np.array_equal(out, g["fT"]), rel_maxnorm(out, g["fT"])
    assert port.checksum(out) == float(g["checksum"])


def test_port_product_form_matches_python_reference_bit_exact(port):
    """The reference's Python class (upwind.py:32,64) rounds its coefficient
    the same way: bit-identical under the product form."""
    g = load_golden("python_12cube_10")
    n = [int(x) for x in g["n"]]
    f0 = np.zeros(int(np.prod(n)))
    f0[0] = 1.0
    out = port.advect(n, [1.0] * 3, [1.0] * 3, f0, int(g["steps"]), float(g["dt"]),
                      coeff_form=1)
    assert np.array_equal(out, g["fT"])


def test_port_product_form_matches_acc_harness(port):
    """Random 3-D cases against the reference's OpenACC variants compiled
    here (skipped where they were not built)."""
    from oracle.oracle import ReferenceAcc
    if not ReferenceAcc.available():
        pytest.skip("reference OpenACC harness not built in this tree")
    acc = ReferenceAcc()
    rng = np.random.default_rng(29)
    for _ in range(12):
        n = tuple(int(x) for x in rng.integers(1, 9, size=3))
        v = tuple(float(x) for x in rng.uniform(-1.5, 1.5, size=3))
        L = tuple(float(x) for x in rng.uniform(0.5, 2, size=3))
        f0 = rng.standard_normal(int(np.prod(n)))
        steps = int(rng.integers(0, 9))
        dt = 0.3 * min(Lj / nj for Lj, nj in zip(L, n))
        a = port.advect(n, v, L, f0, steps, dt, coeff_form=1)
        for variant in (1, 2):
            assert np.array_equal(a, acc.advect(variant, n, v, L, f0, steps, dt)), variant


def test_python_reference_close_to_cxx_order(port):
    """The reference's Python class multiplies (dt*coeff)*(...) (upwind.py:64);
    the C++ order differs by rounding only."""
    g = load_golden("python_12cube_10")
    n = [int(x) for x in g["n"]]
    f0 = np.zeros(int(np.prod(n)))
    f0[0] = 1.0
    out = port.advect(n, [1.0] * 3, [1.0] * 3, f0, int(g["steps"]), float(g["dt"]))
    assert rel_maxnorm(out, g["fT"]) < 1e-14


def test_sphere_generator_pinned(port):
    g = load_golden("synth_sphere_16x12x10")
    f = port.sphere_noise(g["n"], (1.0, 1.0, 1.0), (0.5, 0.5, 0.5), 0.2, 0.01, int(g["seed"]))
    assert np.array_equal(f, g["f"])
    u = np.array([port.lib.fdbo_uniform(int(g["seed"]), i) for i in range(8)])
    assert np.array_equal(u, g["uniform8"])


def test_adjoint_oracle_dot_product(port):
    """<A x, y> = <x, A^T y> for the oracle's transposed step, every sign mix."""
    rng = np.random.default_rng(3)
    for v in [(1.0, -0.7, 0.3), (-1.0, -0.5, -0.2), (0.4, 0.8, -1.0)]:
        n = (5, 6, 7)
        L = (1.0, 1.0, 1.0)
        dt = 0.5 / 7
        x = rng.standard_normal(210)
        y = rng.standard_normal(210)
        ax = port.advect(n, v, L, x, 1, dt)
        aty, _ = port.adjoint_step(n, v, L, dt, np.zeros(210), y)
        assert float(ax @ y) == pytest.approx(float(x @ aty), rel=1e-13)


def test_adjoint_oracle_velocity_gradient_fd(port):
    """dcoef from the oracle adjoint matches a central difference in c_j."""
    rng = np.random.default_rng(5)
    n, L = (4, 5, 6), (1.0, 1.0, 1.0)
    v = np.array([0.6, -0.4, 0.3])
    dt = 0.1
    f = rng.standard_normal(120)
    lam = rng.standard_normal(120)
    _, dcoef = port.adjoint_step(n, v, L, dt, f, lam)
    for j in range(3):
        h = 1e-6
        vp, vm = v.copy(), v.copy()
        vp[j] += h
        vm[j] -= h
        jp = float(lam @ port.advect(n, vp, L, f, 1, dt))
        jm = float(lam @ port.advect(n, vm, L, f, 1, dt))
        dcdv = dt * (1.0 if v[j] < 0 else -1.0) * n[j] / L[j]
        assert dcoef[j] * dcdv == pytest.approx((jp - jm) / (2 * h), rel=1e-6)


@pytest.mark.parametrize("n,v,cfl", [((6, 7, 8), (0.7, -0.5, 0.35), 0.4),
                                     ((5, 6, 7), (1.0, 1.0, 1.0), 0.5),  # sum a = 1.5 > 1
                                     ((6, 5, 9), (0.5, 0.0, -0.5), 0.45),
                                     ((9, 11), (0.6, -0.8), 0.4),
                                     ((17,), (-0.5,), 0.7)])
def test_closed_form_velocity_gradient_identity(port, n, v, cfl):
    """On the periodic grid with constant coefficients the step's operators
    commute, so the per-step velocity contractions of the reverse sweep sum to
    S <lam^1, D_j f0> with lam^1 = (A^T)^(S-1) lam_T.  Checked on the oracle's
    own FP64 step and transposed step (no GPU)."""
    L = (1.0,) * len(n)
    dt = cfl * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(L, n, v) if vj != 0.0)
    S = 9
    rng = np.random.default_rng(sum(n) + S)
    f0 = rng.standard_normal(int(np.prod(n)))
    lam_t = rng.standard_normal(f0.size)
    states = [f0]
    for _ in range(S - 1):
        states.append(port.advect(n, v, L, states[-1], 1, dt))
    lam = lam_t.copy()
    dcoef = np.zeros(len(n))
    for k in range(S - 1, -1, -1):
        lam, dc = port.adjoint_step(n, v, L, dt, states[k], lam)
        dcoef += dc
        if k == 1:
            lam1 = lam.copy()
    if S == 1:
        lam1 = lam_t
    f = f0.reshape(n)
    closed = np.empty(len(n))
    for j in range(len(n)):
        up = 1 if v[j] < 0 else -1
        dj = (np.roll(f, -up, axis=j) - f).reshape(-1)  # f[i + up_j e_j] - f[i]
        closed[j] = -S * float(lam1 @ dj)
    assert np.allclose(closed, dcoef, rtol=1e-12, atol=1e-12 * np.abs(dcoef).max())
