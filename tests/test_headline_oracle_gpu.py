"""The benchmark workloads themselves against the oracle (no GPU-vs-GPU
transitivity): the 512^3 x 100 roofline workload, a seeded sample of the
uneven 256-instance batch through the persistent launch, and a field of wide
dynamic range that shows where the block-fixed-point arithmetic's per-cell
values differ from the reference's FP64 ones.

Bars: EXACT bit-identical to the oracle (which is pinned bit for bit to the
reference's upwind.cxx); FMA and fixed point within 1e-13 relative max-norm;
checksums within 1e-12 relative.  The oracle runs on all host cores
(OpenMP); the 512^3 x 100 reference run takes ~16 s on 16 cores and holds
three 1 GiB host fields."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-13
SUM_TOL = 1e-12

C2_N = (512, 512, 512)
C2_V = (1.0, -0.7, 0.3)
C2_L = (1.0, 1.0, 1.0)
C2_DT = 0.5 / 512
C2_STEPS = 100
C2_SEED = 20261203


@pytest.fixture(scope="module")
def c2_oracle(port):
    """(f0, f_T, checksum) of the 512^3 x 100 workload on the oracle."""
    f0 = port.sphere_noise(C2_N, C2_L, (0.5, 0.5, 0.5), 0.2, 0.01, C2_SEED)
    fT = port.advect(C2_N, C2_V, C2_L, f0, C2_STEPS, C2_DT)
    return f0, fT, port.checksum(fT)


@pytest.mark.parametrize("arith", ["exact", "fma", "auto"])
def test_c2_literal_matches_oracle(fdb, c2_oracle, arith):
    f0, ref, ref_sum = c2_oracle
    up = fdb.Upwind(C2_V, C2_L, C2_N, arith=arith)
    up.init_sphere((0.5, 0.5, 0.5), 0.2, 0.01, C2_SEED)
    assert np.array_equal(up.f, f0)  # the device generator is the oracle's
    up.advect(C2_STEPS, C2_DT)
    out = up.f
    cs = up.checksum()
    used = up.arith_used
    up.close()
    if arith == "auto":
        assert used == "fixed"  # the benchmarked arithmetic
    err = rel_maxnorm(out, ref)
    if used == "exact":
        assert np.array_equal(out, ref), err
    assert err <= FIELD_TOL, (used, err)
    assert cs == pytest.approx(ref_sum, rel=SUM_TOL), (used, cs, ref_sum)


def test_c3_sample_matches_oracle(fdb, port):
    """The benchmark's batch (256 instances, axes uniform in [32, 160],
    velocities in [-1, 1]^3, CFL 0.5, sphere fields), all instances in one
    persistent launch at the tuning the autotuner picks for it and at the
    default tuning, 50 steps; 8 seeded instances checked against the
    oracle."""
    from fidibench_gb300.batch import random_instances

    specs = random_instances(256, 20261203)
    rng = np.random.default_rng(20261203)
    sample = sorted(int(k) for k in rng.choice(256, size=8, replace=False))
    b = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])

    def reset():
        for k, s in enumerate(specs):
            b.init_sphere(k, s["center"], s["radius"], 0.0, 20261203 + k)

    reset()
    f0 = {k: b.get_field(k) for k in sample}
    refs = {k: port.advect(specs[k]["n"], specs[k]["v"], specs[k]["L"], f0[k], 50,
                           specs[k]["dt"]) for k in sample}
    dts = [s["dt"] for s in specs]
    for tuning in ({"depth": 3, "shape": 4, "tile_z": 0}, None):
        if tuning is not None:
            b.set_tuning(**tuning)
        else:
            b.set_tuning(depth=0, shape=-1, tile_z=0)
        reset()
        b.advect(50, dts)
        sums = b.checksums()
        for k in sample:
            err = rel_maxnorm(b.get_field(k), refs[k])
            assert err <= FIELD_TOL, (tuning, k, err)
            assert sums[k] == pytest.approx(port.checksum(refs[k]), rel=SUM_TOL), (tuning, k)
    b.close()


def test_wide_dynamic_range_point_mass(fdb, port):
    """The reference driver's field (f = 0, f[0] = 1; upwind.cxx:45-48) at 64^3
    with its dt (v = 1, CFL 0.1) for 200 steps: the mass spreads into tails
    that fall to ~1e-200 of the peak.  EXACT keeps them bit for bit.  The
    block-fixed-point arithmetic holds one scale per launch, so cells below
    one unit (2^-57 of max|f|) become 0: it meets the max-norm bar, and the
    cells it flushes are exactly tails far below that bar."""
    from oracle import reference_dt

    n = (64, 64, 64)
    v = (1.0, 1.0, 1.0)
    L = (1.0, 1.0, 1.0)
    dt = reference_dt(n, v, L, 0.1)
    steps = 200
    f0 = np.zeros(64 ** 3)
    f0[0] = 1.0
    ref = port.advect(n, v, L, f0, steps, dt)
    peak = float(np.max(np.abs(ref)))
    tiny = np.abs(ref) < 1e-30 * peak
    assert np.count_nonzero(tiny & (ref != 0.0)) > 1000  # the range this test is about

    results = {}
    for arith in ("exact", "fixed"):
        up = fdb.Upwind(v, L, n, arith=arith)
        up.advect(steps, dt)
        results[arith] = (up.f, up.checksum(), up.arith_used)
        up.close()
    ex, ex_sum, used = results["exact"]
    assert used == "exact"
    assert np.array_equal(ex, ref)
    assert np.count_nonzero(ex) == np.count_nonzero(ref)

    fx, fx_sum, used = results["fixed"]
    assert used == "fixed"
    assert rel_maxnorm(fx, ref) <= FIELD_TOL
    assert fx_sum == pytest.approx(port.checksum(ref), rel=SUM_TOL)
    flushed = (fx == 0.0) & (ref != 0.0)
    # recorded, not hidden: the fixed path holds fewer non-zero cells ...
    nz_ref, nz_fx = int(np.count_nonzero(ref)), int(np.count_nonzero(fx))
    print(f"non-zero cells: reference {nz_ref}, fixed point {nz_fx}, flushed {int(flushed.sum())}")
    assert nz_fx < nz_ref
    # ... and every flushed cell is a tail below the max-norm bar
    assert float(np.max(np.abs(ref[flushed]))) <= FIELD_TOL * peak
    # relative precision per cell holds only well above the unit
    big = np.abs(ref) >= 1e-6 * peak
    assert float(np.max(np.abs(fx[big] - ref[big]) / np.abs(ref[big]))) <= 1e-7
