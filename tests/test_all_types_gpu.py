"""Disk, Ellipse, Cone, MeshGraph and the Margin wrapper on the GPU, next to
the six original types: supports, AABBs, pose updates, GJK and EPA in both
forms, against the reference's golden vectors and the oracle.

FP64 results are compared bit for bit.  The mixed form keeps the tolerances
of the six-type tests (1e-5 relative distance error, identical intersection
flags beyond 1e-6, certified EPA depths).
"""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.collider_set import ColliderSet, HULL, MARGIN
from distance3d_gb300.epa import epa_batch
from distance3d_gb300.gjk import gjk_distance_batch, gjk_intersection_batch
from distance3d_gb300.store import ColliderStore
from oracle import oracle
from tests.test_epa_gpu import check_mixed_depths
from tests.test_gjk_gpu import assert_bit_exact, host, mixed_check

pytestmark = pytest.mark.gpu


FIXTURES = ["all9", "mesh10"]


@pytest.mark.parametrize("fx", FIXTURES)
def test_supports_and_aabbs_match_reference(golden, fx):
    g, cs = golden("gjk_" + fx)
    st = ColliderStore(cs)
    n = len(cs)
    idx = np.repeat(np.arange(n), 6).astype(np.int32)
    got = st.support(idx, g["support_dirs"].reshape(-1, 3)).cpu().numpy().reshape(n, 6, 3)
    assert np.array_equal(got, g["supports"])
    assert np.array_equal(st.aabbs().cpu().numpy(), g["aabbs"])


@pytest.mark.parametrize("fx", FIXTURES)
def test_fp64_gjk_matches_reference_golden(golden, fx):
    g, cs = golden("gjk_" + fx)
    st = ColliderStore(cs)
    r = host(gjk_distance_batch(st, g["i1"], g["i2"]))
    assert np.all(r["status"] == 0)
    assert_bit_exact(r, g, written=~np.isnan(g["simplex"]))
    h = gjk_intersection_batch(st, g["i1"], g["i2"])
    assert np.array_equal(h["hit"].cpu().numpy(), g["intersect"])


@pytest.mark.parametrize("fx", FIXTURES)
@pytest.mark.parametrize("tag,kw", [("default", {}), ("large", dict(max_faces=256, max_loose_edges=128)),
                                    ("tight", dict(max_iter=20, max_faces=24, max_loose_edges=6)),
                                    ("short", dict(max_iter=6, max_faces=256, max_loose_edges=128)),
                                    ("edges", dict(max_faces=256, max_loose_edges=4)),
                                    ("eps", dict(max_faces=256, max_loose_edges=128, epsilon=1e-4))])
def test_fp64_epa_matches_reference_golden(golden, fx, tag, kw):
    g, cs = golden("gjk_" + fx)
    e, _ = golden("epa_" + fx)
    p = e["pair"]
    r = host(epa_batch(ColliderStore(cs), g["i1"][p], g["i2"][p], g["simplex"][p], **kw))
    st = e[f"status_{tag}"]
    assert np.array_equal(r["status"], st)
    ok = (st == 0) | (st == 4)  # converged, or the closest face's MTV at the iteration bound
    assert np.array_equal(r["mtv"][ok], e[f"mtv_{tag}"][ok])
    assert np.array_equal(r["n_faces"][ok], e[f"n_faces_{tag}"][ok])


@pytest.mark.parametrize("margin_fraction,types", [(0.0, workloads.ALL_TYPES), (0.5, workloads.ALL_TYPES),
                                                   (0.25, workloads.ALL_TYPES_MESH)])
def test_fp64_matches_oracle(margin_fraction, types):
    cs, i1, i2 = workloads.pairs_all_types(20000, seed=41, margin_fraction=margin_fraction, types=types)
    st = ColliderStore(cs)
    r = host(gjk_distance_batch(st, i1, i2))
    ref = oracle.gjk_distance(cs, i1, i2)
    assert_bit_exact(r, ref)
    assert np.array_equal(r["status"], ref["status"])
    h = gjk_intersection_batch(st, i1, i2)["hit"].cpu().numpy()
    assert np.array_equal(h, oracle.gjk_intersection(cs, i1, i2)["hit"])
    hit = np.flatnonzero(r["dist"] == 0.0)
    kw = dict(max_faces=256, max_loose_edges=128)
    e = host(epa_batch(st, i1[hit], i2[hit], r["simplex"][hit], **kw))
    eref = oracle.epa(cs, i1[hit], i2[hit], r["simplex"][hit], **kw)
    assert np.array_equal(e["status"], eref["status"])
    assert np.array_equal(e["mtv"], eref["mtv"], equal_nan=True)
    assert np.array_equal(e["n_faces"], eref["n_faces"])


@pytest.mark.parametrize("fx,types", [("all9", workloads.ALL_TYPES), ("mesh10", workloads.ALL_TYPES_MESH)])
def test_mixed_gjk_within_tolerance(golden, fx, types):
    cs, i1, i2 = workloads.pairs_all_types(30000, seed=42, types=types)
    st = ColliderStore(cs)
    r = host(gjk_distance_batch(st, i1, i2, precision="mixed"))
    assert np.all(r["status"] == 0)
    mixed_check(r, oracle.gjk_distance(cs, i1, i2), cs, np.asarray(i1), np.asarray(i2))
    g, cs = golden("gjk_" + fx)
    r = host(gjk_distance_batch(ColliderStore(cs), g["i1"], g["i2"], precision="mixed"))
    mixed_check(r, g, cs, g["i1"], g["i2"])


@pytest.mark.parametrize("types", [workloads.ALL_TYPES, workloads.ALL_TYPES_MESH])
def test_mixed_epa_within_tolerance(types):
    cs, i1, i2 = workloads.pairs_all_types(30000, seed=43, types=types)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero(g["dist"] == 0.0)
    kw = dict(max_faces=256, max_loose_edges=128)
    m = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], precision="mixed", **kw))
    ref = oracle.epa(cs, i1[hit], i2[hit], g["simplex"][hit], **kw)
    assert (m["status"] == 0).sum() >= 0.99 * (ref["status"] == 0).sum()
    both, _ = check_mixed_depths(cs, i1[hit], i2[hit], m, ref)
    dm = np.linalg.norm(m["mtv"][both], axis=1)
    dr = np.linalg.norm(ref["mtv"][both], axis=1)
    n = m["mtv"][both] / np.maximum(dm, 1e-300)[:, None]
    h = oracle.depth_upper_bound(cs, i1[hit][both], i2[hit][both], n)
    pos = dm > 0
    assert np.all(np.abs(h[pos] - dm[pos]) <= 1e-7 * np.maximum(1.0, dm[pos]))
    assert np.all(h <= dr + 1e-5 * np.maximum(1.0, dr))


def test_set_poses_new_types():
    """update_pose of disks (normal = R column 2, basis re-derived), ellipses,
    cones and wrapped colliders: AABBs and supports as the oracle computes
    them from the new poses."""
    cs, _, _ = workloads.pairs_all_types(2000, seed=44, margin_fraction=0.5, types=workloads.ALL_TYPES_MESH)
    st = ColliderStore(cs)
    movable = np.flatnonzero(cs.base_types != HULL).astype(np.int32)
    new = workloads.random_colliders(np.random.default_rng(5), len(movable), [1], 1.0).poses
    st.set_poses(movable, new)
    moved = ColliderSet(cs.types, cs.poses.copy(), cs.params, cs.hull_offset, cs.hull_count, cs.vertices,
                        cs.links)
    moved.poses[movable] = new
    assert np.array_equal(st.aabbs().cpu().numpy(), oracle.aabbs(moved))
    idx = np.repeat(np.arange(len(cs)), 4).astype(np.int32)
    dirs = np.random.default_rng(6).normal(size=(len(idx), 3))
    assert np.array_equal(st.support(idx, dirs).cpu().numpy(), oracle.support_batch(moved, idx, dirs))
    with pytest.raises(NotImplementedError):
        st.set_poses(np.flatnonzero((cs.types & ~MARGIN) == HULL)[:1], np.eye(4)[None])


def test_collider_objects(golden):
    """This package's Disk / Ellipse / Cone / MeshGraph / Margin objects,
    packed by from_colliders, give the reference's supports and boxes."""
    from scipy.spatial import ConvexHull
    from distance3d_gb300 import colliders
    g, cs = golden("gjk_mesh10")
    objs = []
    for i in range(80):
        t = int(cs.types[i]) & ~MARGIN
        pose = np.eye(4)
        pose[:3, :3] = cs.poses[i, :9].reshape(3, 3)
        pose[:3, 3] = cs.poses[i, 9:]
        p = cs.params[i]
        if t == 6:
            c = colliders.Disk(pose[:3, 3].copy(), float(p[0]), pose[:3, 2].copy())
        elif t == 7:
            c = colliders.Ellipse(pose[:3, 3].copy(), np.ascontiguousarray(pose[:3, :2].T), p[:2].copy())
        elif t == 8:
            c = colliders.Cone(pose, float(p[0]), float(p[1]))
        elif t == 9:
            o, n = int(cs.hull_offset[i]), int(cs.hull_count[i])
            v = np.ascontiguousarray(cs.vertices[o:o + n, :3])
            c = colliders.MeshGraph(pose, v, ConvexHull(v).simplices)
        else:
            continue
        if int(cs.types[i]) & MARGIN:
            c = colliders.Margin(c, float(p[3]))
        objs.append((i, c))
    assert len(objs) > 10
    for i, c in objs:
        assert np.array_equal(c.aabb(), g["aabbs"][i])
        for k in range(6):
            assert np.array_equal(c.support_function(g["support_dirs"][i, k]), g["supports"][i, k])


def test_collide_all_types_equals_separate_calls():
    """d3d_collide (GJK, then EPA on the intersecting pairs) on the nine-type
    workload gives what the separate entry points give."""
    from distance3d_gb300.serve import CollisionBatch
    from tests.test_serve_gpu import EPA_KW, separate_calls
    cs, i1, i2 = workloads.pairs_all_types(8000, seed=45)
    st = ColliderStore(cs)
    for precision in ("fp64", "mixed"):
        r = CollisionBatch(st, 8192, precision=precision, epa_kw=EPA_KW, graphs=True).run(i1, i2)
        g, hit, e = separate_calls(st, np.asarray(i1), np.asarray(i2), precision)
        for k in ("dist", "cp1", "cp2", "simplex", "n_simplex", "status", "iterations"):
            assert np.array_equal(r[k], g[k], equal_nan=True), k
        assert np.array_equal(r["epa_status"][hit], e["status"])
        assert np.array_equal(r["mtv"][hit], e["mtv"], equal_nan=True)


def test_edge_colliders_match_reference(golden):
    """Degenerate and boundary colliders on the GPU, FP64 form: supports,
    AABBs, GJK, intersection, EPA and MPR equal the reference's."""
    from distance3d_gb300.mpr import mpr_batch
    g, cs = golden("edge")
    st = ColliderStore(cs)
    n, k = len(cs), len(g["support_dirs"])
    idx = np.repeat(np.arange(n), k).astype(np.int32)
    got = st.support(idx, np.tile(g["support_dirs"], (n, 1))).cpu().numpy().reshape(n, k, 3)
    assert np.array_equal(got, g["supports"], equal_nan=True)
    assert np.array_equal(st.aabbs().cpu().numpy(), g["aabbs"], equal_nan=True)
    r = host(gjk_distance_batch(st, g["i1"], g["i2"]))
    ok = ~g["sanity"]
    assert np.all(r["status"][ok] == 0)
    for key in ("dist", "n_simplex", "iterations"):
        assert np.array_equal(r[key][ok], g[key][ok]), key
    assert np.array_equal(r["cp1"][ok], g["cp1"][ok], equal_nan=True)
    assert np.array_equal(r["cp2"][ok], g["cp2"][ok], equal_nan=True)
    h = gjk_intersection_batch(st, g["i1"], g["i2"])["hit"].cpu().numpy()
    assert np.array_equal(h, g["intersect"])
    m = host(mpr_batch(st, g["i1"], g["i2"]))
    assert np.array_equal(m["hit"], g["mpr_hit"])
    for key in ("depth", "dir", "pos"):
        assert np.array_equal(m[key], g["mpr_" + key], equal_nan=True), key
    p = g["epa_pair"]
    for tag, kw in (("default", {}), ("large", dict(max_faces=256, max_loose_edges=128))):
        e = host(epa_batch(st, g["i1"][p], g["i2"][p], g["simplex"][p], **kw))
        s = g[f"epa_status_{tag}"]
        assert np.array_equal(e["status"], s)
        assert np.array_equal(e["mtv"][s == 0], g[f"epa_mtv_{tag}"][s == 0])
    # the mixed forms on the same pairs: GJK within tolerance, MPR flags
    mg = host(gjk_distance_batch(st, g["i1"], g["i2"], precision="mixed"))
    mixed_check(mg, g, cs, g["i1"], g["i2"])


@pytest.mark.parametrize("fx", ["scb", "mixed6", "all9", "mesh10"])
@pytest.mark.parametrize("tag,kw", [("clip", dict(max_distance_squared=0.01)), ("coarse", dict(tolerance=1e-3))])
def test_fp64_gjk_options_match_reference_golden(golden, fx, tag, kw):
    """The FP64 GJK with a clipping distance many pairs exceed and with a
    coarse tolerance under which the reference's sanity assertion fails on
    some pairs: statuses, distances and points of the reference."""
    g, cs = golden("gjk_" + fx)
    r = host(gjk_distance_batch(ColliderStore(cs), g["i1"], g["i2"], **kw))
    st = g[f"status_{tag}"]
    assert np.array_equal(r["status"], st)
    ok = st != 2
    assert np.array_equal(r["dist"][ok], g[f"dist_{tag}"][ok])
    assert np.array_equal(r["cp1"][ok], g[f"cp1_{tag}"][ok], equal_nan=True)
