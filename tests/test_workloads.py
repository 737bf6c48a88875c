"""The synthetic workloads (CPU): the center half-width calibrated to ~30%
intersecting six-type pairs, the literal [-1,1]^3 centers at ~3%, and the
hull sizes of the bench distributions."""
import numpy as np

from distance3d_gb300 import workloads
from distance3d_gb300.collider_set import HULL
from oracle import oracle


def intersecting_fraction(half_width, n=40000, seed=0):
    cs, i1, i2 = workloads.pairs_mixed_six(n, seed=seed, center_half_width=half_width)
    g = oracle.gjk_distance(cs, i1, i2)
    return float(np.mean(g["dist"] == 0.0)), cs


def test_calibrated_half_width_gives_thirty_percent():
    f, cs = intersecting_fraction(workloads.INTERSECT30_HALF_WIDTH)
    assert 0.27 <= f <= 0.33, f
    hull = cs.types == HULL
    counts = cs.hull_count[hull]
    assert counts.min() >= 8 and counts.max() <= 256
    assert 0.12 <= hull.mean() <= 0.21  # one of six types


def test_literal_unit_box_gives_few_intersections():
    f, _ = intersecting_fraction(1.0)
    assert 0.015 <= f <= 0.05, f
