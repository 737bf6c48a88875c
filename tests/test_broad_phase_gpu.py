"""Broad phase on the GPU (LBVH through the C ABI): pair sets equal the
reference's AabbTree / brute-force sets exactly."""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.aabb_tree import AabbTree, all_aabbs_overlap
from distance3d_gb300.broad_phase import BoundingVolumeHierarchy
from distance3d_gb300.bvh import LBVH
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_golden_tree_pairs(golden):
    t, cs = golden("aabb_tree")
    aabbs = ColliderStore(cs).aabbs().cpu().numpy()
    assert np.array_equal(aabbs, t["aabbs"])
    assert np.array_equal(LBVH(aabbs).self_pairs().cpu().numpy(), t["tree_pairs"])
    tree = AabbTree()
    tree.insert_aabbs(aabbs)
    for q in range(len(t["queries"])):
        want = t["query_idx"][t["query_ptr"][q]:t["query_ptr"][q + 1]]
        _, got = tree.overlaps_aabb(t["queries"][q])
        assert np.array_equal(got, want)


class _TM:
    def __init__(self):
        self.T = {}

    def add_transform(self, a, b, A2B):
        self.T[(a, b)] = A2B

    def get_transform(self, a, b):
        return self.T[(a, b)]


def test_golden_bvh_with_self(golden):
    """BoundingVolumeHierarchy.aabb_overlapping_with_self on the reference's
    colliders: the same ordered pairs (both orders, i == j dropped)."""
    from distance3d_gb300 import colliders as C
    t, cs = golden("aabb_tree")
    n = int(t["bvh_n"])
    cols = []
    for i in range(n):
        pose = np.eye(4)
        pose[:3, :3] = cs.poses[i, :9].reshape(3, 3)
        pose[:3, 3] = cs.poses[i, 9:]
        p = cs.params[i]
        ty = cs.types[i]
        if ty == 0:
            cols.append(C.Sphere(pose[:3, 3].copy(), p[0]))
        elif ty == 1:
            cols.append(C.Capsule(pose, p[0], p[1]))
        elif ty == 2:
            cols.append(C.Box(pose, p[:3].copy()))
        elif ty == 3:
            cols.append(C.Cylinder(pose, p[0], p[1]))
        elif ty == 4:
            cols.append(C.Ellipsoid(pose, p[:3].copy()))
        else:
            o, c = cs.hull_offset[i], cs.hull_count[i]
            cols.append(C.ConvexHullVertices(cs.vertices[o:o + c, :3].copy()))
    bvh = BoundingVolumeHierarchy(_TM(), "base")
    for i, c in enumerate(cols):
        bvh.add_collider(i, c)
    got = np.array(sorted((a[0], b[0]) for a, b in bvh.aabb_overlapping_with_self()), dtype=np.int32)
    assert np.array_equal(got.reshape(-1, 2), t["bvh_pairs"])
    # per-collider query with a whitelist
    k = int(t["bvh_pairs"][0, 0])
    partners = set(t["bvh_pairs"][t["bvh_pairs"][:, 0] == k, 1].tolist())
    found = bvh.aabb_overlapping_colliders(cols[k], whitelist=(k,))
    assert set(found.keys()) == partners


def test_reference_hand_boxes():
    """test_aabb_tree.py:6-56 and :87-122."""
    aabbs = np.array([[[0, 2], [0, 2], [0, 1]], [[1, 3], [1, 3], [0, 1]], [[3, 4], [0, 1], [0, 1]]], float)
    aabbs2 = np.array([[[1.5, 3.5], [0, 0.5], [0, 1]], [[1.5, 2], [2.5, 4], [0, 1]],
                       [[3.5, 4.5], [0, 0.5], [0, 1]]], float)
    tree = AabbTree()
    tree.insert_aabbs([])
    tree.insert_aabbs(aabbs, ["test"] * 3, pre_insertion_methode="shuffle")
    _, o = tree.overlaps_aabb(aabbs2[0])
    assert o[0] == 0 and o[1] == 2
    _, o = tree.overlaps_aabb(aabbs2[1])
    assert o[0] == 1
    _, o = tree.overlaps_aabb(aabbs2[2])
    assert o[0] == 2
    tree2 = AabbTree()
    tree2.insert_aabbs(aabbs2, ["2"] * 3)
    ok, t1, t2, _ = tree.overlaps_aabb_tree(tree2)
    assert ok and np.array_equal(t1, [0, 1, 2]) and np.array_equal(t2, [0, 1, 2])

    a1 = np.array([[0, 10], [0, 10], [0, 10]], float)
    a2 = np.array([[8, 12], [3, 4], [4, 5]], float)
    a3 = np.array([[20, 30], [0, 1], [0, 2]], float)
    a4 = np.array([[-50, 50], [-50, 50], [-50, 50]], float)
    tree = AabbTree()
    tree.insert_aabb(a1, 1)
    tree.insert_aabb(a2, 2)
    tree.insert_aabb(a3, 3)
    flag, ov = tree.overlaps_aabb(a1)
    ext = [tree.external_data_list[i] for i in ov]
    ins = [tree.insert_index_list[i] for i in ov]
    assert flag and 1 in ext and 2 in ext and 0 in ins and 1 in ins
    flag, ov = tree.overlaps_aabb(a4)
    ext = [tree.external_data_list[i] for i in ov]
    assert flag and {1, 2, 3} <= set(ext)


@pytest.mark.parametrize("n,half", [(2000, 3.0), (20000, 8.0)])
def test_self_pairs_match_brute_force(n, half):
    cs = workloads.scene_mixed_six(n, seed=n, half_width=half)
    aabbs = ColliderStore(cs).aabbs()
    got = LBVH(aabbs).self_pairs().cpu().numpy()
    want = oracle.self_pairs(aabbs.cpu().numpy())
    assert len(want) > 100
    assert np.array_equal(got, want)


def test_cross_query_matches_brute_force():
    a = workloads.scene_mixed_six(3000, seed=5, half_width=4.0)
    b = workloads.scene_mixed_six(2000, seed=6, half_width=4.0)
    A = oracle.aabbs(a)
    B = oracle.aabbs(b)
    want = oracle.cross_pairs(A, B)  # (i in A, j in B), sorted by i then j
    u1, u2, pairs = all_aabbs_overlap(A, B)
    assert np.array_equal(np.array(pairs, dtype=np.int32).reshape(-1, 2), want)
    assert np.array_equal(u1, np.unique(want[:, 0])) and np.array_equal(u2, np.unique(want[:, 1]))


def test_full_scene_131072():
    """The broad-phase workload: 131,072 colliders in [-20,20]^3."""
    cs = workloads.scene_mixed_six(131072, seed=3)
    aabbs = ColliderStore(cs).aabbs()
    got = LBVH(aabbs).self_pairs().cpu().numpy()
    want = oracle.self_pairs_sweep(aabbs.cpu().numpy())
    assert np.array_equal(got, want)


def test_edge_cases():
    for n in (0, 1):
        boxes = np.zeros((n, 3, 2))
        boxes[..., 1] = 1.0
        assert LBVH(boxes).self_pairs().shape == (0, 2)
    two = np.array([[[0, 1], [0, 1], [0, 1]], [[1, 2], [0, 1], [0, 1]]], float)  # touching faces overlap
    assert LBVH(two).self_pairs().cpu().numpy().tolist() == [[0, 1]]
    apart = two.copy()
    apart[1, 0] = [np.nextafter(1.0, 2.0), 2.0]
    assert LBVH(apart).self_pairs().shape == (0, 2)
    # 1,000 identical boxes: equal Morton codes, every pair overlaps, and the
    # pair count exceeds the first capacity guess
    same = np.tile(np.array([[[0, 1], [0, 1], [0, 1]]], float), (1000, 1, 1))
    p = LBVH(same).self_pairs().cpu().numpy()
    assert len(p) == 1000 * 999 // 2
    assert np.array_equal(p, oracle.self_pairs(same))
    # points (zero-size boxes) on a grid, some coincident
    rng = np.random.default_rng(0)
    pts = rng.integers(0, 20, size=(3000, 3)).astype(float)
    boxes = np.stack([pts, pts], axis=2)
    assert np.array_equal(LBVH(boxes).self_pairs().cpu().numpy(), oracle.self_pairs(boxes))
    # query with no boxes in the tree / no queries
    assert LBVH(np.zeros((0, 3, 2))).query(two).shape == (0, 2)
    assert LBVH(two).query(np.zeros((0, 3, 2))).shape == (0, 2)


def test_deterministic_output():
    cs = workloads.scene_mixed_six(30000, seed=9, half_width=10.0)
    aabbs = ColliderStore(cs).aabbs()
    a = LBVH(aabbs).self_pairs().cpu().numpy()
    b = LBVH(aabbs).self_pairs().cpu().numpy()
    assert np.array_equal(a, b)


def test_collide_scene_broad_then_narrow():
    """The broad+narrow workload path: pair set bit-exact against the sweep
    oracle, FP64 narrow phase bit-exact against the oracle's GJK on those
    pairs, mixed form within tolerance and with the same intersection flags."""
    from distance3d_gb300.pipeline import collide_scene
    cs = workloads.scene_mixed_six(131072, seed=7)
    st = ColliderStore(cs)
    pairs, r = collide_scene(st, precision="fp64")
    want = oracle.self_pairs_sweep(st.aabbs().cpu().numpy())
    p = pairs.cpu().numpy()
    assert np.array_equal(p, want) and len(p) > 1000
    ref = oracle.gjk_distance(cs, p[:, 0], p[:, 1])
    assert np.array_equal(r["dist"].cpu().numpy(), ref["dist"])
    assert np.array_equal(r["simplex"].cpu().numpy(), ref["simplex"])
    _, m = collide_scene(st, precision="mixed")
    # the mixed form against the reference, certified where the reference's
    # own distance disagrees with its closest points (see test_gjk_gpu)
    from tests.test_gjk_gpu import mixed_check
    mixed_check({k: v.cpu().numpy() for k, v in m.items()}, ref, cs, p[:, 0], p[:, 1])


def test_refit_after_moving_the_leaves():
    """Refit keeps the pair sets exact after every leaf moves."""
    rng = np.random.default_rng(3)
    cs = workloads.scene_mixed_six(20000, seed=11, half_width=8.0)
    st = ColliderStore(cs)
    a = st.aabbs().cpu().numpy()
    tree = LBVH(a)
    for step in range(3):
        shift = rng.normal(scale=0.5, size=(len(a), 3, 1))
        b = a + shift
        tree.refit(b)
        assert np.array_equal(tree.self_pairs().cpu().numpy(), oracle.self_pairs_sweep(b))
        q = b[rng.integers(0, len(b), 300)] + rng.normal(scale=0.2, size=(300, 3, 1))
        got = tree.query(q).cpu().numpy()
        want = oracle.cross_pairs(b, q)
        assert np.array_equal(got, want)
    import pytest
    with pytest.raises(ValueError):
        tree.refit(a[:10])


def test_bvh_pose_update_refits():
    """update_collider_poses moves the colliders and refits the tree: the
    pairs equal those of a BVH built from scratch at the new poses."""
    from distance3d_gb300 import colliders as C
    rng = np.random.default_rng(8)

    def scene(tm, centers, offsets):
        bvh = BoundingVolumeHierarchy(tm, "base")
        for i, c in enumerate(centers):
            pose = np.eye(4)
            pose[:3, 3] = c + offsets[i]
            tm.add_transform(i, "origin", pose)
            col = C.Box(pose, np.array([0.4, 0.3, 0.5])) if i % 2 else C.Capsule(pose, 0.2, 0.4)
            bvh.add_collider(i, col)
        return bvh

    n = 400
    centers = rng.uniform(-4, 4, (n, 3))
    tm = _TM()
    bvh = scene(tm, centers, np.zeros((n, 3)))
    before = sorted((a[0], b[0]) for a, b in bvh.aabb_overlapping_with_self())
    tree_id = id(bvh.aabbtree_)
    moves = rng.normal(scale=0.3, size=(n, 3))
    for i in range(n):
        pose = np.eye(4)
        pose[:3, 3] = centers[i] + moves[i]
        tm.add_transform(i, "origin", pose)
    bvh.update_collider_poses()
    assert id(bvh.aabbtree_) == tree_id  # refit, not rebuilt
    after = sorted((a[0], b[0]) for a, b in bvh.aabb_overlapping_with_self())
    fresh = scene(_TM(), centers, moves)
    assert after == sorted((a[0], b[0]) for a, b in fresh.aabb_overlapping_with_self())
    assert after != before
