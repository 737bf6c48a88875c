"""MPR on the GPU (through the C ABI) against the reference's golden vectors
and the oracle, bit for bit: flags, depths, directions, contact positions,
status."""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.mpr import mpr_batch
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu


def host(r):
    return {k: v.cpu().numpy() for k, v in r.items()}


def assert_same(r, ref):
    assert np.array_equal(r["hit"], ref["hit"])
    assert np.array_equal(r["status"], ref["status"])
    for k in ("depth", "dir", "pos"):
        if k in r:
            assert np.array_equal(r[k], ref[k], equal_nan=True), k


@pytest.mark.parametrize("fx", ["all9", "mesh10"])
def test_mpr_matches_reference_golden(golden, fx):
    g, cs = golden("gjk_" + fx)
    m, _ = golden("mpr_" + fx)
    st = ColliderStore(cs)
    r = host(mpr_batch(st, m["i1"], m["i2"]))
    assert np.all(r["status"] == 0)
    assert np.array_equal(r["hit"], m["hit"])
    for k in ("depth", "dir", "pos"):
        assert np.array_equal(r[k], m[k], equal_nan=True), k
    ri = host(mpr_batch(st, m["i1"], m["i2"], penetration=False))
    assert np.array_equal(ri["hit"], m["hit_intersection"])
    assert set(ri) == {"hit", "status"}


@pytest.mark.parametrize("maker,kw", [
    (workloads.pairs_all_types, dict(margin_fraction=0.5)),
    (workloads.pairs_all_types, dict(types=workloads.ALL_TYPES_MESH)),
    (workloads.pairs_mixed_six, dict(center_half_width=workloads.INTERSECT30_HALF_WIDTH)),
    (workloads.pairs_sphere_capsule_box, {}),
])
def test_mpr_matches_oracle(maker, kw):
    cs, i1, i2 = maker(20000, seed=51, **kw)
    st = ColliderStore(cs)
    r = host(mpr_batch(st, i1, i2))
    assert_same(r, oracle.mpr(cs, i1, i2))
    assert r["hit"].sum() > 500


def test_mpr_edge_cases():
    cs, i1, i2 = workloads.pairs_all_types(256, seed=52)
    st = ColliderStore(cs)
    assert mpr_batch(st, [], [])["hit"].numel() == 0
    # every collider against itself (centers coincide: the reference nudges v0)
    same = np.arange(len(cs), dtype=np.int32)
    assert_same(host(mpr_batch(st, same, same)), oracle.mpr(cs, same, same))
    # the refinement bound: zero expansions allowed
    r = host(mpr_batch(st, i1, i2, refine_limit=0))
    ref = oracle.mpr(cs, i1, i2, refine_limit=0)
    assert_same(r, ref)
    assert (ref["status"] == 3).any()
    # tolerance and iteration options
    for kw in (dict(mpr_tolerance=1e-2), dict(max_iterations=1), dict(max_iterations=0)):
        assert_same(host(mpr_batch(st, i1, i2, **kw)),
                    oracle.mpr(cs, i1, i2, tolerance=kw.get("mpr_tolerance", 1e-4),
                               max_iterations=kw.get("max_iterations", 100)))


def test_drop_in_mpr():
    from distance3d_gb300 import colliders, mpr
    s1 = colliders.Sphere(np.zeros(3), 1.0)
    s2 = colliders.Sphere(np.array([0.0, 0.0, 1.0]), 0.5)
    hit, depth, pdir, pos = mpr.mpr_penetration(s1, s2)
    assert hit and depth == 0.5
    np.testing.assert_array_almost_equal(pdir, [0, 0, 1])
    assert mpr.mpr_intersection(s1, s2)
    far = colliders.Sphere(np.array([5.0, 0.0, 0.0]), 0.5)
    assert mpr.mpr_penetration(s1, far) == (False, None, None, None)
    assert not mpr.mpr_intersection(s1, far)
