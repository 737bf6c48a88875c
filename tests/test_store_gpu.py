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
