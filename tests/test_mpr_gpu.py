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


# MPR decides a pair whose origin lies just outside its portal by whether
# the portal can still expand by more than its tolerance (1e-4, mpr.py:290-
# 299), so its flag is defined only up to that tolerance: the two forms may
# differ within it
FLAG_MARGIN = 1e-4


def rel_depth_err(a, b):
    both = a["hit"] & b["hit"]
    return np.abs(a["depth"][both] - b["depth"][both]) / np.maximum(1.0, b["depth"][both]), both


@pytest.mark.parametrize("types", [workloads.ALL_TYPES, workloads.ALL_TYPES_MESH])
def test_mixed_mpr_against_fp64(types):
    """Mixed MPR against the plain FP64 MPR.

    Flags: identical wherever the pair is more than the MPR tolerance (1e-4)
    from touching (FP64 GJK distance, FP64 EPA depth).  Depths: MPR's depth is the distance to
    the final portal face, and which face the search ends on is sensitive to
    its inputs -- moving every collider by 1e-9 changes the FP64 depth by
    more than 1e-5 (relative to max(1, depth)) on about 2% of the pairs, by
    up to 1e-2.  The mixed depths must stay within a few times that spread
    (quantiles of the relative error against those of the moved FP64 run).
    Directions are unit or zero vectors; the intersection-only flags equal
    the penetration form's."""
    from distance3d_gb300.collider_set import ColliderSet
    from distance3d_gb300.epa import epa_batch
    from distance3d_gb300.gjk import gjk_distance_batch
    cs, i1, i2 = workloads.pairs_all_types(40000, seed=53, types=types)
    st = ColliderStore(cs)
    f = host(mpr_batch(st, i1, i2))
    m = host(mpr_batch(st, i1, i2, precision="mixed"))
    g = host(gjk_distance_batch(st, i1, i2))
    assert np.all(m["status"] == 0)
    # flags: wherever FP64 GJK separates the pair by more than the tolerance,
    # or FP64 EPA finds it deeper than that, both forms decide alike (the
    # reference's MPR itself misses a few pairs that EPA finds deep)
    sep = g["dist"] > FLAG_MARGIN
    full = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    e = host(epa_batch(st, i1[full], i2[full], g["simplex"][full], max_faces=256, max_loose_edges=128))
    deep = np.zeros(len(i1), bool)
    deep[full] = (e["status"] == 0) & (np.linalg.norm(e["mtv"], axis=1) > FLAG_MARGIN)
    assert np.array_equal(m["hit"][sep | deep], f["hit"][sep | deep])
    assert not np.any(m["hit"][sep])
    poses = cs.poses.copy()
    poses[:, 9:] += 1e-9
    verts = cs.vertices.copy()
    verts[:, :3] += 1e-9
    moved = ColliderSet(cs.types, poses, cs.params, cs.hull_offset, cs.hull_count, verts, cs.links)
    q = host(mpr_batch(ColliderStore(moved), i1, i2))
    err_m, both = rel_depth_err(m, f)
    err_q, _ = rel_depth_err(q, f)
    assert np.quantile(err_q, 0.999) > 1e-4  # the FP64 form's own sensitivity
    for p, floor in ((0.99, 1e-3), (0.999, 1e-2)):
        assert np.quantile(err_m, p) <= max(floor, 5 * np.quantile(err_q, p)), (p, np.quantile(err_m, p))
    nd = np.linalg.norm(m["dir"][both], axis=1)
    assert np.all((np.abs(nd - 1.0) < 1e-12) | (nd == 0.0))
    mi = host(mpr_batch(st, i1, i2, precision="mixed", penetration=False))
    assert np.array_equal(mi["hit"], m["hit"])
