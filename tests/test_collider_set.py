"""The packed host format (ColliderSet) for the nine types and the Margin
wrapper: packing of collider objects, validation, and the oracle on the
packed rows (CPU only)."""
import numpy as np
import pytest

from distance3d_gb300 import colliders
from distance3d_gb300.collider_set import (ColliderSet, BOX, CONE, DISK, ELLIPSE, HULL, MARGIN, SPHERE)
from oracle import oracle


def test_from_colliders_packs_new_types():
    pose = np.eye(4)
    pose[:3, 3] = 1.0, 2.0, 3.0
    axes = np.array([[1.0, 0.0, 0.0], [0.0, 0.6, 0.8]])
    cols = [colliders.Disk(np.array([0.5, 0.0, 0.0]), 0.25, np.array([0.0, 1.0, 0.0])),
            colliders.Ellipse(np.zeros(3), axes, np.array([0.3, 0.2])),
            colliders.Cone(pose, 0.4, 1.5),
            colliders.Margin(colliders.Sphere(np.zeros(3), 1.0), 0.05),
            colliders.Margin(colliders.ConvexHullVertices(np.eye(3)), 0.0)]
    cs = ColliderSet.from_colliders(cols)
    assert list(cs.types) == [DISK, ELLIPSE, CONE, SPHERE | MARGIN, HULL | MARGIN]
    assert list(cs.base_types) == [DISK, ELLIPSE, CONE, SPHERE, HULL]
    assert list(cs.wrapped) == [False, False, False, True, True]
    R = cs.poses[:, :9].reshape(-1, 3, 3)
    np.testing.assert_array_equal(R[0][:, 2], [0.0, 1.0, 0.0])       # disk normal in column 2
    np.testing.assert_array_equal(R[1][:, :2], axes.T)               # ellipse axes in columns 0, 1
    np.testing.assert_array_equal(R[1][:, 2], np.cross(axes[0], axes[1]))
    np.testing.assert_array_equal(cs.poses[2, 9:], [1.0, 2.0, 3.0])
    np.testing.assert_array_equal(cs.params[:, 3], [0.0, 0.0, 0.0, 0.05, 0.0])
    np.testing.assert_array_equal(cs.params[2, :2], [0.4, 1.5])


def test_margin_of_margin_rejected():
    m = colliders.Margin(colliders.Margin(colliders.Sphere(np.zeros(3), 1.0), 0.1), 0.1)
    with pytest.raises(TypeError):
        ColliderSet.from_colliders([m])


def test_unknown_type_rejected():
    cs = ColliderSet.from_colliders([colliders.Sphere(np.zeros(3), 1.0)])
    for bad in (9, 0x200, -1):
        with pytest.raises(ValueError):
            ColliderSet(np.array([bad]), cs.poses, cs.params, cs.hull_offset, cs.hull_count, cs.vertices)


def test_oracle_margin_zero_keeps_supports():
    """A Margin of 0 moves no support point (it adds 0 * d/|d|), and a box's
    margin moves the support by exactly margin * d/|d|."""
    box = colliders.Box(np.eye(4), np.array([1.0, 2.0, 3.0]))
    cs = ColliderSet.from_colliders([box, colliders.Margin(box, 0.0), colliders.Margin(box, 0.5)])
    d = np.array([0.3, -0.4, 1.2])
    s0, s1, s2 = (oracle.support(cs, i, d) for i in range(3))
    np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_almost_equal(s2, s0 + 0.5 * d / np.linalg.norm(d), decimal=15)
    assert cs.types[2] == BOX | MARGIN


def test_mesh_graph_packing_and_concatenation():
    from scipy.spatial import ConvexHull
    from distance3d_gb300.collider_set import MESH, mesh_links
    rng = np.random.default_rng(0)
    v = rng.normal(size=(20, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    tri = ConvexHull(v).simplices
    pose = np.eye(4)
    pose[:3, 3] = 1.0, -2.0, 0.5
    m = colliders.MeshGraph(pose, v, tri)
    cs = ColliderSet.from_colliders([colliders.Sphere(np.zeros(3), 1.0), m, colliders.Margin(m, 0.1)])
    assert list(cs.base_types) == [SPHERE, MESH, MESH] and cs.wrapped[2]
    blk = mesh_links(v, tri)
    assert len(cs.links) == 2 * len(blk)
    for i in (1, 2):
        b = int(cs.params[i, 0])
        assert np.array_equal(cs.links[b:b + len(blk)], blk)
        assert cs.params[i, 1] == tri.min()
    # every vertex's neighbours are the vertices sharing a triangle with it
    for k in range(len(v)):
        nb = set(blk[blk[6 + k]:blk[7 + k]].tolist())
        want = set(tri[np.any(tri == k, axis=1)].ravel().tolist()) - {k}
        assert nb == want
    both = ColliderSet.concatenate([cs, cs])
    b0, b1 = int(both.params[1, 0]), int(both.params[4, 0])
    assert np.array_equal(both.links[b1:b1 + len(blk)], blk) and b1 == b0 + len(cs.links)
    # the oracle's hill climb reaches the vertex a full scan finds
    d = rng.normal(size=(50, 3))
    got = np.stack([oracle.support(cs, 1, x) for x in d])
    R = pose[:3, :3]
    world = v @ R.T + pose[:3, 3]
    want = world[np.argmax((v @ (R.T @ d.T)), axis=0)]
    np.testing.assert_allclose(got, want, atol=1e-12)


def test_mesh_graph_bad_links_rejected():
    from scipy.spatial import ConvexHull
    v = np.random.default_rng(1).normal(size=(12, 3))
    m = colliders.MeshGraph(np.eye(4), v, ConvexHull(v).simplices)
    cs = ColliderSet.from_colliders([m])
    for links in (cs.links[:10], np.where(np.arange(len(cs.links)) == len(cs.links) - 1, 99, cs.links)):
        with pytest.raises(ValueError):
            ColliderSet(cs.types, cs.poses, cs.params, cs.hull_offset, cs.hull_count, cs.vertices, links)
