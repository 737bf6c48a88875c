"""Device store: AABBs, support points and pose updates against the golden
vectors and the oracle, bit for bit."""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.collider_set import ColliderSet, HULL
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["gjk_mixed6", "gjk_scb", "aabb_tree"])
def test_aabbs_match_reference(golden, name):
    g, cs = golden(name)
    assert np.array_equal(ColliderStore(cs).aabbs().cpu().numpy(), g["aabbs"])


def test_aabb_scan_ties_and_nans():
    """The polytope AABB is scanned by a warp with integer keys: its values
    are those of the sequential scan (oracle), bit for bit: the first of
    equal values (-0 and +0 in the same axis), a NaN at vertex 0 kept, later
    NaNs skipped, hulls shorter and longer than a warp."""
    rng = np.random.default_rng(12)
    sizes = [1, 2, 5, 31, 32, 33, 64, 65, 200, 256, 40, 40, 40]
    verts = [rng.normal(size=(k, 3)) for k in sizes]
    verts[3][:, 0] = np.abs(verts[3][:, 0])
    verts[3][[0, 7, 30], 0] = [0.0, -0.0, -0.0]  # the minimum of x: +0 first, then -0
    verts[5][:, 1] = -np.abs(verts[5][:, 1])
    verts[5][[4, 32], 1] = [-0.0, 0.0]  # the maximum of y: -0 first (lanes 4 and 0)
    verts[10][0, 2] = np.nan  # NaN at vertex 0: kept
    verts[11][17, 2] = np.nan  # NaN later: skipped
    verts[11][3, 0] = np.nan
    verts[12][:, 0] = 1.5  # every value tied
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    n = len(sizes)
    cs = ColliderSet(np.full(n, HULL), np.tile(np.concatenate([np.eye(3).ravel(), np.zeros(3)]), (n, 1)),
                     np.zeros((n, 4)), off, sizes, np.concatenate(verts))
    got = ColliderStore(cs).aabbs().cpu().numpy()
    want = oracle.aabbs(cs)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    assert np.isnan(got[10, 2]).all() and not np.isnan(got[11]).any()
    assert not np.signbit(got[3, 0, 0]) and np.signbit(got[5, 1, 1])


def test_support_matches_oracle():
    cs = workloads.scene_mixed_six(600, seed=9, half_width=1.0)
    st = ColliderStore(cs)
    rng = np.random.default_rng(3)
    idx = np.repeat(np.arange(len(cs)), 8).astype(np.int32)
    dirs = rng.normal(size=(len(idx), 3))
    dirs[::8] = 0.0  # zero direction: each type's own fallback
    got = st.support(idx, dirs).cpu().numpy()
    want = np.stack([oracle.support(cs, i, d) for i, d in zip(idx, dirs)])
    assert np.array_equal(got, want)


def test_set_poses():
    cs = workloads.scene_mixed_six(400, seed=10, half_width=1.0)
    st = ColliderStore(cs)
    movable = np.flatnonzero(cs.types != HULL).astype(np.int32)
    new = workloads.random_colliders(np.random.default_rng(4), len(movable), [0], 2.0).poses
    st.set_poses(movable, new)
    moved = ColliderSet(cs.types, cs.poses.copy(), cs.params, cs.hull_offset, cs.hull_count, cs.vertices)
    moved.poses[movable] = new
    assert np.array_equal(st.aabbs().cpu().numpy(), oracle.aabbs(moved))
    hulls = np.flatnonzero(cs.types == HULL)
    with pytest.raises(NotImplementedError):
        st.set_poses(hulls[:1], np.eye(4)[None])


def test_collider_objects_on_gpu():
    from distance3d_gb300 import colliders
    b = colliders.Box(np.eye(4), np.array([1.0, 2.0, 3.0]))
    np.testing.assert_array_equal(b.aabb(), [[-0.5, 0.5], [-1, 1], [-1.5, 1.5]])
    # four vertices tie along +x; np.argmax keeps the first in BOX_COORDS order
    np.testing.assert_array_equal(b.support_function(np.array([1.0, 0, 0])), [0.5, -1.0, -1.5])
    np.testing.assert_array_equal(b.support_function(np.array([1.0, 1e-3, 1e-3])), [0.5, 1.0, 1.5])
    s = colliders.Sphere(np.array([0.0, 1, 2]), 3.0)
    np.testing.assert_array_equal(s.aabb(), [[-3, 3], [-2, 4], [-1, 5]])
    assert b.vertices.shape == (8, 3)
