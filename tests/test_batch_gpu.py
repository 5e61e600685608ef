"""Batched form through the C-ABI: every instance against the oracle, the
persistent launch bit-identical to the single-field kernel looped over the
instances, graph replay, tuning choices, and the bounded-wait error path."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-13
SUM_TOL = 1e-12


def make_batch(fdb, specs, seed=3):
    b = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    for k, s in enumerate(specs):
        b.init_sphere(k, s["center"], s["radius"], 0.01, seed + k)
    return b


def small_specs(count=9, seed=5, nmin=5, nmax=40):
    from fidibench_gb300.batch import random_instances
    return random_instances(count, seed, nmin, nmax)


def test_batched_matches_oracle(fdb, port):
    specs = small_specs()
    b = make_batch(fdb, specs)
    f0 = [b.get_field(k) for k in range(b.count)]
    dts = [s["dt"] for s in specs]
    steps = 11
    b.advect(steps, dts)
    sums = b.checksums()
    for k, s in enumerate(specs):
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], steps, s["dt"])
        assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL, k
        assert sums[k] == pytest.approx(port.checksum(ref), rel=SUM_TOL)
    b.close()


@pytest.mark.parametrize("depth,shape,tile_z", [(4, -1, 0), (2, 3, 0), (3, 2, 8), (4, 4, 5)])
def test_batched_bit_identical_to_looped(fdb, depth, shape, tile_z):
    specs = small_specs(count=7, seed=11, nmin=20, nmax=70)
    dts = [s["dt"] for s in specs]
    a = make_batch(fdb, specs)
    c = make_batch(fdb, specs)
    a.set_tuning(depth=depth, shape=shape, tile_z=tile_z)
    c.set_tuning(depth=depth)  # the looped comparator takes the same time blocks
    for _ in range(2):  # the second call replays the captured graph
        a.advect(21, dts)
        c.advect_looped(21, dts)
    # integer arithmetic: any tiling gives the same field, so equal time
    # blocks are bit-equal
    for k in range(a.count):
        assert np.array_equal(a.get_field(k), c.get_field(k)), k
    a.close()
    c.close()


def test_looped_default_depth_matches_oracle(fdb, port):
    """Without a depth the looped comparator runs every instance as
    fdb_upwind_advect does (fixed point at its default depth, or FP64 below
    2^18 cells): bit-identical to Upwind.advect, and within the parity
    tolerance of the oracle."""
    specs = small_specs(count=6, seed=17, nmin=30, nmax=110)
    dts = [s["dt"] for s in specs]
    b = make_batch(fdb, specs)
    f0 = [b.get_field(k) for k in range(b.count)]
    b.advect_looped(13, dts)
    for k, s in enumerate(specs):
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], 13, s["dt"])
        assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL, k
        up = fdb.Upwind(s["v"], s["L"], s["n"])
        up.f = f0[k]
        up.advect(13, s["dt"])
        assert np.array_equal(b.get_field(k), up.f), k
        up.close()
    b.close()


def test_batched_any_depth_matches_oracle(fdb, port):
    specs = small_specs(count=5, seed=13, nmin=8, nmax=33)
    dts = [s["dt"] for s in specs]
    for depth in (2, 3, 4):
        b = make_batch(fdb, specs)
        f0 = [b.get_field(k) for k in range(b.count)]
        b.set_tuning(depth=depth)
        b.advect(10, dts)
        for k, s in enumerate(specs):
            ref = port.advect(s["n"], s["v"], s["L"], f0[k], 10, s["dt"])
            assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL, (depth, k)
        b.close()


def test_autotune_keeps_results_and_caches(fdb, tmp_path, port):
    specs = small_specs(count=6, seed=17, nmin=16, nmax=48)
    dts = [s["dt"] for s in specs]
    b = make_batch(fdb, specs)
    f0 = [b.get_field(k) for k in range(b.count)]
    cache = str(tmp_path / "tune.txt")
    chosen = b.autotune(8, dts, cache)
    assert chosen["depth"] in (2, 3, 4)
    for k in range(b.count):  # the autotuner restores the fields
        assert np.array_equal(b.get_field(k), f0[k])
    again = b.autotune(8, dts, cache)  # from the cache
    assert again == chosen
    b.advect(8, dts)
    for k, s in enumerate(specs):
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], 8, s["dt"])
        assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL
    b.close()


def test_bounded_wait_expires_with_error_and_context_survives(fdb, monkeypatch):
    """FDB_FAULT=timeout makes every dependency unsatisfiable with a ~1 ms
    wait budget: the kernel must give up, report FDB_ERR_TIMEOUT, and leave
    the context usable."""
    specs = small_specs(count=3, seed=19, nmin=30, nmax=40)
    dts = [s["dt"] for s in specs]
    b = make_batch(fdb, specs)
    monkeypatch.setenv("FDB_FAULT", "timeout")
    b.advect(12, dts)
    with pytest.raises(fdb.FdbError) as ei:
        b.checksums()
    assert ei.value.code == 5
    monkeypatch.delenv("FDB_FAULT")
    for k, s in enumerate(specs):
        b.init_sphere(k, s["center"], s["radius"], 0.0, 1)
    b.advect(12, dts)
    assert np.all(np.isfinite(b.checksums()))
    b.close()


def test_unsupported_instance_falls_back(fdb, port):
    # a Courant number above 1 on one instance: the batch loops the FP64 path
    specs = small_specs(count=3, seed=23, nmin=10, nmax=20)
    specs[1] = dict(specs[1], dt=specs[1]["dt"] * 3.0)
    dts = [s["dt"] for s in specs]
    b = make_batch(fdb, specs)
    f0 = [b.get_field(k) for k in range(b.count)]
    b.advect(5, dts)
    for k, s in enumerate(specs):
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], 5, s["dt"])
        assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL
    b.close()


def test_permuted_storage_is_invisible(fdb, port):
    """An instance stored with its axes permuted (marched along the axis
    that tiles worst): fields go in and out in the caller's order, the sphere
    generator gives the single-field values, and the advected field is
    bit-identical to Upwind.advect where that runs fixed point too (the
    fixed-point update does not depend on the order of the axes) and within
    the parity tolerance of the oracle."""
    specs = [
        {"n": (40, 33, 200), "v": (0.7, -0.4, 0.9), "L": (1.0, 2.0, 3.0)},
        {"n": (64, 64, 64), "v": (-0.3, 0.5, 0.2), "L": (1.0, 1.0, 1.0)},
        {"n": (33, 90), "v": (0.6, -0.8), "L": (1.0, 1.0)},
    ]
    for s in specs:
        s["dt"] = 0.3 * min(Lj / nj / abs(vj) for Lj, nj, vj in zip(s["L"], s["n"], s["v"]))
    b = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    assert sorted(b.storage_order(0)) == [0, 1, 2]
    assert b.storage_order(0) != (0, 1, 2)  # 200 planes of 40 x 33 tile worst as x or y
    assert b.storage_order(1) == (0, 1, 2)  # ties keep the caller's order
    rng = np.random.default_rng(21)
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    for k in range(len(specs)):
        b.set_field(k, f0[k])
        assert np.array_equal(b.get_field(k), f0[k]), k
    dts = [s["dt"] for s in specs]
    b.set_tuning(depth=4)
    b.advect(13, dts)
    sums = b.checksums()
    for k, s in enumerate(specs):
        up = fdb.Upwind(s["v"], s["L"], s["n"], depth=4)  # the same time blocks
        up.f = f0[k]
        up.advect(13, s["dt"])
        if np.prod(s["n"]) >= 1 << 18:  # Upwind.advect runs it in fixed point too
            assert np.array_equal(b.get_field(k), up.f), k
        else:
            assert rel_maxnorm(b.get_field(k), up.f) <= FIELD_TOL, k
        assert sums[k] == pytest.approx(up.checksum(), rel=SUM_TOL)
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], 13, s["dt"])
        assert rel_maxnorm(b.get_field(k), ref) <= FIELD_TOL, k
        up.init_sphere((0.4, 0.5, 0.6)[:len(s["n"])], 0.3, 0.01, 77 + k)
        b.init_sphere(k, (0.4, 0.5, 0.6)[:len(s["n"])], 0.3, 0.01, 77 + k)
        assert np.array_equal(b.get_field(k), up.f), k
        up.close()
    b.close()


@pytest.mark.parametrize("depth,tile_z", [(2, 0), (3, 0), (4, 0), (3, 7)])
def test_packed_tiles_edge_shapes(fdb, port, depth, tile_z):
    """Packed tiles on the shapes that stress them: 1-D and 2-D instances
    (axes of one cell), axes shorter than the depth (more halo than output),
    remainders that put up to 8 x 8 rectangles in one tile, and z ranges
    (tile_z caps them) whose last one overlaps the one before.  Every
    instance is bit-identical to the single-field kernel looped at the same
    depth and within the parity tolerance of the oracle."""
    rng = np.random.default_rng(29)
    shapes = [(3,), (2, 5), (1, 7, 4), (7, 3, 2), (31, 1, 40), (29, 58, 3), (5, 200),
              (61, 2, 33), (90, 31, 1), (1, 1, 64)]
    specs = []
    for n in shapes:
        v = tuple(float(x) for x in rng.uniform(-1.0, 1.0, len(n)))
        L = tuple(float(x) for x in rng.uniform(0.5, 2.0, len(n)))
        dt = 0.3 / sum(abs(vj) * nj / Lj for Lj, nj, vj in zip(L, n, v))  # Courant sum 0.3
        specs.append({"n": n, "v": v, "L": L, "dt": dt})
    dts = [s["dt"] for s in specs]
    a = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    c = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    f0 = [rng.standard_normal(int(np.prod(s["n"]))) for s in specs]
    for k in range(len(specs)):
        a.set_field(k, f0[k])
        c.set_field(k, f0[k])
    a.set_tuning(depth=depth, shape=4, tile_z=tile_z)
    c.set_tuning(depth=depth)
    a.advect(17, dts)
    c.advect_looped(17, dts)
    for k, s in enumerate(specs):
        assert np.array_equal(a.get_field(k), c.get_field(k)), k
        ref = port.advect(s["n"], s["v"], s["L"], f0[k], 17, s["dt"])
        assert rel_maxnorm(a.get_field(k), ref) <= FIELD_TOL, k
    a.close()
    c.close()


@pytest.mark.parametrize("depth", [2, 3])
def test_packed_tiles_larger_instances_bit_identical(fdb, depth):
    """A few instances with axes above one tile width on every axis (full
    tiles, remainders in x and y, z ranges split to fill the remainder
    tiles), mixed with small ones: the persistent launch at the default
    shape equals the single-field kernel looped at the same depth."""
    from fidibench_gb300.batch import random_instances
    specs = random_instances(4, 31, 90, 200) + random_instances(5, 37, 8, 40)
    dts = [s["dt"] for s in specs]
    a = make_batch(fdb, specs)
    c = make_batch(fdb, specs)
    a.set_tuning(depth=depth, shape=4, tile_z=0)
    c.set_tuning(depth=depth)
    a.advect(2 * depth + 1, dts)  # a last time block shorter than the depth
    c.advect_looped(2 * depth + 1, dts)
    for k in range(a.count):
        assert np.array_equal(a.get_field(k), c.get_field(k)), k
    a.close()
    c.close()
