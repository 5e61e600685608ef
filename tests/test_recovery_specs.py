"""The recovery workload's seeded instances (host logic, no GPU): the time
step rules.  "sum" keeps every instance at a Courant sum of 0.5 (stable);
"per_axis" reads CFL 0.5 per axis, so the sum reaches up to 1.5 and the
instances above 1 amplify their checkerboard mode."""
from __future__ import annotations

import pytest

from fidibench_gb300.recovery import instance_specs


def courant(sp, n):
    a = [sp["dt"] * n * abs(v) for v in sp["v"]]
    return sum(a), max(a)


def test_sum_rule_is_stable():
    n = 128
    for sp in instance_specs(64, n, 20261203):
        s, _ = courant(sp, n)
        assert s == pytest.approx(0.5, rel=1e-12)


def test_per_axis_rule_reads_each_axis():
    n = 128
    specs = instance_specs(64, n, 20261203, cfl_rule="per_axis")
    sums = []
    for sp in specs:
        s, m = courant(sp, n)
        assert m == pytest.approx(0.5, rel=1e-12)
        sums.append(s)
    assert max(sums) <= 1.5 + 1e-12
    assert any(s > 1.0 for s in sums)  # the literal rule leaves the stable range


def test_same_seed_same_instances_and_rule_check():
    a = instance_specs(8, 64, 7)
    b = instance_specs(8, 64, 7, cfl_rule="per_axis")
    assert [x["v"] for x in a] == [x["v"] for x in b]
    assert [x["center"] for x in a] == [x["center"] for x in b]
    with pytest.raises(ValueError):
        instance_specs(2, 8, 1, cfl_rule="cfl")
