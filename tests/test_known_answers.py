"""Known answers from the distance3d reference's own tests, on the GPU path
and on the oracle.

Inputs and expected values are the reference's (test_gjk.py, test_gjk_jolt.py,
test_epa.py), cited per test.  Each case runs on two backends: the C oracle
(CPU, always) and the CUDA library through the C ABI (marked gpu).
"""
import itertools

import numpy as np
import pytest
from numpy.testing import assert_array_almost_equal
from pytest import approx

from distance3d_gb300 import colliders
from distance3d_gb300.collider_set import ColliderSet

BACKENDS = ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)]
MAX_FLOAT = np.finfo(float).max


def distance_batch(backend, pairs, **kw):
    """GJK distance for a list of (collider1, collider2): dict of numpy arrays."""
    cols = [c for p in pairs for c in p]
    cs = ColliderSet.from_colliders(cols)
    i1 = np.arange(0, 2 * len(pairs), 2, dtype=np.int32)
    i2 = i1 + 1
    if backend == "oracle":
        from oracle import oracle
        r = oracle.gjk_distance(cs, i1, i2, **kw)
        h = oracle.gjk_intersection(cs, i1, i2)
        r["hit"] = h["hit"]
        return r
    from distance3d_gb300.store import ColliderStore
    from distance3d_gb300.gjk import gjk_distance_batch, gjk_intersection_batch
    st = ColliderStore(cs)
    r = {k: v.cpu().numpy() for k, v in gjk_distance_batch(st, i1, i2, **kw).items()}
    r["hit"] = gjk_intersection_batch(st, i1, i2)["hit"].cpu().numpy()
    return r


def hull(v):
    return colliders.ConvexHullVertices(np.array(v, dtype=float))


@pytest.mark.parametrize("backend", BACKENDS)
def test_points_and_segments(backend):
    """test_gjk.py:7-53: exact 0 / 1 distances and flags."""
    p1, p2 = hull([[0.0, 0.0, 0.0]]), hull([[1.0, 0.0, 0.0]])
    s1 = hull([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    s2 = hull([[0.0, 1.0, 0.0], [1.0, 1.0, 0.0]])
    s3 = hull([[0.5, -1.0, 0.0], [0.5, 1.0, 0.0]])
    cases = [(p1, p1, 0.0, True), (p1, p2, 1.0, False), (s1, s1, 0.0, True), (s1, p1, 0.0, True),
             (s1, p2, 0.0, True), (s1, s2, 1.0, False), (s1, s3, 0.0, True)]
    r = distance_batch(backend, [(a, b) for a, b, _, _ in cases])
    for k, (_, _, d, hit) in enumerate(cases):
        assert r["dist"][k] == d
        assert bool(r["hit"][k]) == hit


@pytest.mark.parametrize("backend", BACKENDS)
def test_boxes(backend):
    """test_gjk.py:56-129: touching unit boxes and the rotated-box golden."""
    b1 = colliders.Box(np.eye(4), np.ones(3))
    pairs = []
    for dim1, dim2, dim3 in itertools.product(range(3), repeat=3):
        for s1, s2, s3 in itertools.product([-1, 1], repeat=3):
            pose = np.eye(4)
            pose[dim1, 3] = s1
            pose[dim2, 3] = s2
            pose[dim3, 3] = s3
            pairs.append((b1, colliders.Box(pose, np.ones(3))))
    R = np.array([[-0.29265666, -0.76990535, 0.56709596], [0.93923897, -0.12018753, 0.32153556],
                  [-0.17939408, 0.62673815, 0.75829879]])
    pa, pb = np.eye(4), np.eye(4)
    pa[:3, :3] = pb[:3, :3] = R
    pa[:3, 3] = [0.1867558, -0.09772779, 0.09500884]
    pb[:3, 3] = [3.73511598, -1.95455576, 1.90017684]
    pairs.append((colliders.Box(pa, np.array([2.89098828, 1.15032456, 2.37517511])),
                  colliders.Box(pb, np.array([0.96366276, 0.38344152, 0.79172504]))))
    r = distance_batch(backend, pairs)
    for k in range(len(pairs) - 1):
        assert approx(r["dist"][k]) == 0.0
    assert approx(r["dist"][-1]) == 1.7900192730149391


@pytest.mark.parametrize("backend", BACKENDS)
def test_spheres_cylinders_capsules(backend):
    """test_gjk.py:132-309."""
    s1 = colliders.Sphere(np.zeros(3), 1.0)
    s2 = colliders.Sphere(np.array([1.0, 1.0, 1.0]), 1.0)
    s3 = colliders.Sphere(np.array([0.0, 0.0, 3.0]), 1.0)
    cy1 = colliders.Cylinder(np.eye(4), 1, 1)
    t = np.eye(4)
    t[:3, 3] = [3, 0, 0]
    cy2 = colliders.Cylinder(t, 1, 1)
    cap2 = colliders.Capsule(t, 1, 1)
    t2 = np.eye(4)
    t2[:3, 3] = [0, 0, 4]
    cy3 = colliders.Cylinder(t2, 1, 1)
    cap3 = colliders.Capsule(t2, 1, 1)
    cap1 = colliders.Capsule(np.eye(4), 1, 1)
    pairs = [(s1, s1), (s1, s2), (s1, s3), (cy1, cy1), (cy1, cy2), (cy1, cy3), (cap1, cap1), (cap1, cap2),
             (cap1, cap3)]
    r = distance_batch(backend, pairs)
    expected = [0, 0, 1, 0, 1, 3, 0, 1, 1]
    for k, d in enumerate(expected):
        assert approx(r["dist"][k]) == d
    assert_array_almost_equal(r["cp1"][6], r["cp2"][6])
    assert_array_almost_equal(r["cp1"][7], [1, 0, -0.5])
    assert_array_almost_equal(r["cp2"][7], [2, 0, -0.5])
    assert_array_almost_equal(r["cp1"][8], [0, 0, 1.5])
    assert_array_almost_equal(r["cp2"][8], [0, 0, 2.5])


@pytest.mark.parametrize("backend", BACKENDS)
def test_random_point_clouds(backend):
    """test_gjk.py:373-408 (RandomState(23)): closest points inside the
    clouds' boxes and |cp2 - cp1| == dist."""
    rs = np.random.RandomState(23)
    pairs, neg = [], []
    for sign in (1, -1):
        for _ in range(50):
            v1 = rs.rand(6, 3) * np.array([[2, 5, 1]])
            v2 = rs.rand(6, 3) * (np.array([[1, 3, 1]]) if sign > 0 else np.array([[-2, -3, 1]]))
            pairs.append((hull(v1), hull(v2)))
            neg.append(sign < 0)
    r = distance_batch(backend, pairs)
    for k in range(len(pairs)):
        c1, c2 = r["cp1"][k], r["cp2"][k]
        assert 0 <= c1[0] < 2 and 0 <= c1[1] < 5 and 0 <= c1[2] < 1
        if not neg[k]:
            assert 0 <= c2[0] < 1 and 0 <= c2[1] < 3 and 0 <= c2[2] < 1
        else:
            assert -2 < c2[0] <= 2 and -3 < c2[1] <= 5 and 0 <= c2[2] < 1
        assert approx(r["dist"][k]) == np.linalg.norm(c2 - c1)


@pytest.mark.parametrize("backend", BACKENDS)
def test_too_far_away(backend):
    """test_gjk_jolt.py:88-95: clipping."""
    r = distance_batch(backend, [(hull([[0.0, 0.0, 0.0]]), hull([[100000000.0, 0.0, 0.0]]))])
    assert r["dist"][0] == MAX_FLOAT
    assert r["status"][0] == 1
    assert np.all(np.isnan(r["cp1"][0]))


EPA_V1 = np.array([[1.76405235, 0.40015721, 0.97873798], [2.2408932, 1.86755799, -0.97727788],
                   [0.4105985, 0.14404357, 1.45427351], [0.33367433, 1.49407907, -0.20515826],
                   [0.3130677, -0.85409574, -2.55298982], [2.26975462, -1.45436567, 0.04575852],
                   [-0.18718385, 1.53277921, 1.46935877]])
EPA_V2 = np.array([[-2.32605299, -0.31242692, 0.07599278], [0.88503416, 1.23786508, -0.467683],
                   [-0.64755927, -1.01306774, -1.50037412], [-2.05152671, 1.98626062, -0.59000837],
                   [-0.78333082, -1.21731013, 0.69713417], [-1.95915437, -0.17725505, -0.97582275],
                   [0.04164598, -0.47531991, -1.26098837], [-0.37343875, 0.4638171, -0.01383896],
                   [-0.04278462, -0.59883687, -0.44309735]])


def epa_run(backend, cs, i1, i2, simplex, **kw):
    if backend == "oracle":
        from oracle import oracle
        return oracle.epa(cs, i1, i2, simplex, **kw)
    from distance3d_gb300.store import ColliderStore
    from distance3d_gb300.epa import epa_batch
    return {k: v.cpu().numpy() for k, v in epa_batch(ColliderStore(cs), i1, i2, simplex, **kw).items()}


@pytest.mark.parametrize("backend", BACKENDS)
def test_epa_golden(backend):
    """test_epa.py:7-34."""
    r = distance_batch(backend, [(hull(EPA_V1), hull(EPA_V2))])
    assert_array_almost_equal(r["cp1"][0], r["cp2"][0])
    cs = ColliderSet.from_colliders([hull(EPA_V1), hull(EPA_V2)])
    e = epa_run(backend, cs, [0], [1], r["simplex"])
    assert e["status"][0] == 0
    assert_array_almost_equal(e["mtv"][0], np.array([-0.387287, 0.179576, -0.176204]))


@pytest.mark.parametrize("backend", BACKENDS)
def test_epa_separation(backend):
    """test_epa.py:37-60 (RandomState(25)): moving convex2 by (1 + depth)
    along the MTV direction gives GJK distance 1."""
    rs = np.random.RandomState(25)
    sets = []
    for _ in range(50):
        sets.append((rs.rand(6, 3) * np.array([[2, 2, 2]]), rs.rand(6, 3) * np.array([[1, 1, 1]])))
    r = distance_batch(backend, [(hull(a), hull(b)) for a, b in sets])
    hit = np.flatnonzero(r["dist"] <= 0.0)
    assert len(hit) > 10
    cs = ColliderSet.from_colliders([c for k in hit for c in (hull(sets[k][0]), hull(sets[k][1]))])
    i1 = np.arange(0, 2 * len(hit), 2)
    e = epa_run(backend, cs, i1, i1 + 1, r["simplex"][hit])
    assert np.all(e["status"] == 0)
    moved = []
    for j, k in enumerate(hit):
        depth = np.linalg.norm(e["mtv"][j])
        pdir = e["mtv"][j] / depth
        moved.append((hull(sets[k][0]), hull(sets[k][1] + (1.0 + depth) * pdir[np.newaxis])))
    r2 = distance_batch(backend, moved)
    for d in r2["dist"]:
        assert approx(d) == 1.0


def aabbs_of(backend, cols, poses=None):
    """(n,3,2) boxes of collider objects; ``poses`` (index -> 4x4) are set
    through the store's pose update (update_pose on the GPU path)."""
    cs = ColliderSet.from_colliders(cols)
    if backend == "oracle":
        from oracle import oracle
        if poses:
            cs = ColliderSet(cs.types, cs.poses.copy(), cs.params, cs.hull_offset, cs.hull_count, cs.vertices)
            for i, p in poses.items():
                cs.poses[i, :9] = p[:3, :3].reshape(-1)
                cs.poses[i, 9:] = p[:3, 3]
        return oracle.aabbs(cs)
    from distance3d_gb300.store import ColliderStore
    st = ColliderStore(cs)
    if poses:
        st.set_poses(list(poses), np.stack(list(poses.values())))
    return st.aabbs().cpu().numpy()


@pytest.mark.parametrize("backend", BACKENDS)
def test_cone_disk_margin_aabbs(backend):
    """test_colliders.py:47-97: cone, disk and Margin(box) boxes, before and
    after update_pose."""
    cone = colliders.Cone(np.eye(4), 0.5, 1.0)
    disk = colliders.Disk(np.zeros(3), 0.5, np.array([0.0, 0.0, 1.0]))
    boxm = colliders.Margin(colliders.Box(np.eye(4), np.array([1.0, 1.0, 1.0])), 0.1)
    a = aabbs_of(backend, [cone, disk, boxm])
    assert_array_almost_equal(a[0], [[-0.5, 0.5], [-0.5, 0.5], [0.0, 1.0]])
    assert_array_almost_equal(a[1], [[-0.5, 0.5], [-0.5, 0.5], [0.0, 0.0]])
    assert_array_almost_equal(a[2], [[-0.6, 0.6], [-0.6, 0.6], [-0.6, 0.6]])
    p0, p1 = np.eye(4), np.eye(4)
    p0[:3, 3] = 0.1, 0.2, 0.3
    p1[:3, 3] = -0.1, -0.2, -0.3
    a = aabbs_of(backend, [cone, disk, boxm], {0: p0, 1: p1, 2: p0})
    assert_array_almost_equal(a[0], [[-0.4, 0.6], [-0.3, 0.7], [0.3, 1.3]])
    assert_array_almost_equal(a[1], [[-0.6, 0.4], [-0.7, 0.3], [-0.3, -0.3]])
    assert_array_almost_equal(a[2], [[-0.5, 0.7], [-0.4, 0.8], [-0.3, 0.9]])


@pytest.mark.parametrize("backend", BACKENDS)
def test_gjk_distance_with_margin(backend):
    """test_gjk.py:476-483: a margin of 0.1 shortens the distance by 0.1."""
    box = colliders.Box(np.eye(4), np.array([2.0, 2.0, 2.0]))
    sphere = colliders.Sphere(np.array([2.0, 0.0, 0.0]), 0.5)
    r = distance_batch(backend, [(box, sphere), (colliders.Margin(box, 0.1), sphere)])
    assert approx(r["dist"][0]) == r["dist"][1] + 0.1


def mpr_batch(backend, pairs, **kw):
    cols = [c for p in pairs for c in p]
    cs = ColliderSet.from_colliders(cols)
    i1 = np.arange(0, 2 * len(pairs), 2, dtype=np.int32)
    i2 = i1 + 1
    if backend == "oracle":
        from oracle import oracle
        return oracle.mpr(cs, i1, i2, **kw)
    from distance3d_gb300.mpr import mpr_batch as run
    from distance3d_gb300.store import ColliderStore
    r = run(ColliderStore(cs), i1, i2, **kw)
    return {k: v.cpu().numpy() for k, v in r.items()}


@pytest.mark.parametrize("backend", BACKENDS)
def test_mpr_intersection_vs_gjk(backend):
    """test_mpr.py:7-20 (RandomState(24)): MPR and GJK agree on intersection."""
    rs = np.random.RandomState(24)
    pairs = [(hull(rs.rand(6, 3) * np.array([[2, 2, 2]])), hull(rs.rand(6, 3) * np.array([[1, 1, 1]])))
             for _ in range(50)]
    g = distance_batch(backend, pairs)
    m = mpr_batch(backend, pairs, penetration=False)
    assert np.array_equal(g["dist"] < 1e-16, m["hit"].astype(bool))


@pytest.mark.parametrize("backend", BACKENDS)
def test_mpr_penetration_points_segments_spheres(backend):
    """test_mpr.py:23-93: points, segments and spheres."""
    p0, p1 = hull([[0.0, 0.0, 0.0]]), hull([[1.0, 0.0, 0.0]])
    s1 = hull([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    o = colliders.Sphere(np.zeros(3), 1.0)
    pairs = [(p0, p0), (s1, s1), (s1, p0), (s1, p1), (o, colliders.Sphere(np.zeros(3), 1.0)),
             (o, colliders.Sphere(np.array([0.0, 0.0, 1.0]), 0.5)),
             (o, colliders.Sphere(np.array([1.0, 0.0, 0.0]), 0.5))]
    r = mpr_batch(backend, pairs)
    assert np.all(r["hit"])
    depth = [0.0, 1.0, 0.0, 0.0]
    dirs = [np.zeros(3), [-1, 0, 0], np.zeros(3), np.zeros(3)]
    pos = [np.zeros(3), [0.5, 0, 0], np.zeros(3), [1, 0, 0]]
    for k in range(4):
        assert approx(r["depth"][k]) == depth[k]
        assert_array_almost_equal(r["dir"][k], dirs[k])
        assert_array_almost_equal(r["pos"][k], pos[k])
    assert r["depth"][4] == 2.0
    assert approx(np.linalg.norm(r["dir"][4])) == 1.0
    assert_array_almost_equal(r["pos"][4], [0, 0, 0])
    assert r["depth"][5] == 0.5
    assert_array_almost_equal(r["dir"][5], [0, 0, 1])
    assert_array_almost_equal(r["pos"][5], [0, 0, 0.75])
    assert r["depth"][6] == 0.5
    assert_array_almost_equal(r["dir"][6], [1, 0, 0])
    assert_array_almost_equal(r["pos"][6], [0.75, 0, 0])
