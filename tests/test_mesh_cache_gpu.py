"""MeshGraph vertex caching on the GPU against the stock reference.

The reference's MeshGraph support object remembers the vertex of its last
climb and starts the next climb there (mesh.py:30, 82-85).  On tied vertices
(an axis-aligned cube along an axis) the answer depends on that start, so a
sequence of calls on shared objects gives other closest points and simplices
than climbs from the start vertex.  The fixture ``gjk_mesh_cached`` records
the stock reference's calls in a fixed order with the caches before and after
each; the batch entry point with ``mesh_cache`` and the drop-in
``gjk_distance_jolt`` on this package's MeshGraph objects reproduce them bit
for bit.
"""
import numpy as np
import pytest
import torch

from distance3d_gb300 import colliders
from distance3d_gb300.collider_set import MARGIN
from distance3d_gb300.gjk import gjk_distance_batch, gjk_distance_jolt
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu


def _assert_outputs(h, g, sel=slice(None)):
    assert np.array_equal(h["dist"], g["dist"][sel])
    assert np.array_equal(h["n_simplex"], g["n_simplex"][sel])
    assert np.array_equal(h["iterations"], g["iterations"][sel])
    assert np.array_equal(h["cp1"], g["cp1"][sel], equal_nan=True)
    assert np.array_equal(h["cp2"], g["cp2"][sel], equal_nan=True)
    written = ~np.isnan(g["simplex"][sel])
    assert np.array_equal(h["simplex"][written], g["simplex"][sel][written])
    assert np.all(h["status"] == 0)


def test_batch_with_caches(golden):
    g, cs = golden("gjk_mesh_cached")
    st = ColliderStore(cs)
    cache = torch.as_tensor(g["cache_before"], device=st.device).contiguous()
    r = gjk_distance_batch(st, g["i1"], g["i2"], mesh_cache=cache)
    h = {k: v.cpu().numpy() for k, v in r.items()}
    _assert_outputs(h, g)
    assert np.array_equal(cache.cpu().numpy(), g["cache_after"])


def test_fresh_caches_match_oracle(golden):
    """A cache of -1 is a freshly built MeshGraph (climbs start at the
    smallest vertex index of its triangles, then carry from call to call
    within the GJK run): the oracle's cached GJK from the same caches, bit
    for bit, and the caches left are the last vertices reached."""
    g, cs = golden("gjk_mesh_cached")
    st = ColliderStore(cs)
    n = len(g["i1"])
    cache = torch.full((n, 2), -1, dtype=torch.int32, device=st.device)
    h = {k: v.cpu().numpy() for k, v in gjk_distance_batch(st, g["i1"], g["i2"], mesh_cache=cache).items()}
    want = np.full((n, 2), -1, np.int32)
    o = oracle.gjk_distance_cached(cs, g["i1"], g["i2"], want)
    for k in ("dist", "cp1", "cp2", "n_simplex", "status", "iterations"):
        assert np.array_equal(h[k], o[k]), k
    rows = np.arange(4)[None, :] < o["n_simplex"][:, None]
    assert np.array_equal(h["simplex"][rows], o["simplex"][rows])
    assert np.array_equal(cache.cpu().numpy(), want)
    mesh = np.array([(int(cs.types[i]) & ~MARGIN) == 9 for i in range(len(cs))])
    assert np.all((want[:, 0] >= 0) == mesh[g["i1"]]) and np.all((want[:, 1] >= 0) == mesh[g["i2"]])


def test_mesh_cache_argument_checks(golden):
    g, cs = golden("gjk_mesh_cached")
    st = ColliderStore(cs)
    n = len(g["i1"])
    with pytest.raises(ValueError):
        gjk_distance_batch(st, g["i1"], g["i2"], precision="mixed",
                           mesh_cache=torch.full((n, 2), -1, dtype=torch.int32, device=st.device))
    with pytest.raises(ValueError):
        gjk_distance_batch(st, g["i1"], g["i2"], mesh_cache=torch.full((n, 2), -1, dtype=torch.int64,
                                                                      device=st.device))
    with pytest.raises(ValueError):
        gjk_distance_batch(st, g["i1"], g["i2"], mesh_cache=np.full((n, 2), -1, np.int32))


def _objects(g, cs):
    """This package's collider objects for the fixture's colliders."""
    out = []
    for i in range(len(cs)):
        t = int(cs.types[i]) & ~MARGIN
        pose = np.eye(4)
        pose[:3, :3] = cs.poses[i, :9].reshape(3, 3)
        pose[:3, 3] = cs.poses[i, 9:]
        p = cs.params[i]
        if t == 0:
            c = colliders.Sphere(pose[:3, 3].copy(), float(p[0]))
        elif t == 2:
            c = colliders.Box(pose, p[:3].copy())
        else:
            assert t == 9
            o, n = int(cs.hull_offset[i]), int(cs.hull_count[i])
            tri = g["triangles"][g["triangle_ptr"][i]:g["triangle_ptr"][i + 1]]
            c = colliders.MeshGraph(pose, np.ascontiguousarray(cs.vertices[o:o + n, :3]), tri)
        if int(cs.types[i]) & MARGIN:
            c = colliders.Margin(c, float(p[3]))
        out.append(c)
    return out


def test_drop_in_sequence(golden):
    """The drop-in on shared MeshGraph objects, called in the fixture's
    order: every call starts from the cache the previous calls left in the
    object and leaves the reference's cache there (first 200 calls)."""
    g, cs = golden("gjk_mesh_cached")
    objs = _objects(g, cs)

    def inner(c):
        return c.collider if isinstance(c, colliders.Margin) else c
    for k in range(200):
        c1, c2 = objs[g["i1"][k]], objs[g["i2"][k]]
        seen = [inner(c).first_idx if isinstance(inner(c), colliders.MeshGraph) else -1 for c in (c1, c2)]
        assert seen == list(g["cache_before"][k])
        d, a, b, y = gjk_distance_jolt(c1, c2)
        assert d == g["dist"][k]
        assert np.array_equal(a, g["cp1"][k]) and np.array_equal(b, g["cp2"][k])
        m = g["n_simplex"][k]
        assert np.array_equal(y[:m], g["simplex"][k, :m])
        left = [inner(c).first_idx if isinstance(inner(c), colliders.MeshGraph) else -1 for c in (c1, c2)]
        assert left == list(g["cache_after"][k])
