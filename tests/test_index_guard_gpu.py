"""Out-of-range collider indices on the device: every batch entry point
reports D3D_STATUS_BAD_INDEX (NaN results, hit 0) for a pair whose index lies
outside [0, n_colliders) and gives the other pairs the results they get in a
batch without such pairs.

No index here ever leaves the store's buffers.  The calls run on a view of a
store that declares fewer colliders than its buffers hold, with pairs that
name colliders beyond that count: those indices are out of range for the view,
so the kernels must reject them, yet every record they name exists, so a
missing check would read valid memory rather than fault.
"""
import numpy as np
import pytest
import torch

from distance3d_gb300 import _lib, workloads
from distance3d_gb300.epa import epa_batch
from distance3d_gb300.gjk import gjk_distance_batch, gjk_intersection_batch
from distance3d_gb300.mpr import mpr_batch
from distance3d_gb300.store import ColliderStore

pytestmark = pytest.mark.gpu

HIDDEN = 300  # colliders at the end of the buffers that the view does not declare


class View:
    """The buffers of `store` declaring only its first n colliders."""

    def __init__(self, store, n):
        v = store._view
        self.device = store.device
        self.n_colliders = n
        self._store = store
        self._view = _lib.D3DStore(n, v.n_vertices, v.rec64, v.rec32, v.meta, v.verts64, v.verts32, v.links,
                                   v.n_links)

    @property
    def view(self):
        import ctypes
        return ctypes.byref(self._view)

    def stream(self):
        return self._store.stream()

    def support(self, idx, dirs):
        return ColliderStore.support(self, idx, dirs)

    def aabbs(self, idx=None):
        return ColliderStore.aabbs(self, idx)


@pytest.fixture(scope="module")
def scene():
    cs, i1, i2 = workloads.pairs_mixed_six(4000, seed=61, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    n = len(cs)
    limit = n - HIDDEN
    rng = np.random.default_rng(5)
    # pairs with both, one or no index beyond the view's count, interleaved
    extra = np.arange(limit, n, dtype=np.int32)
    a = np.concatenate([i1, rng.choice(extra, 200), rng.integers(0, limit, 200, dtype=np.int32)]).astype(np.int32)
    b = np.concatenate([i2, rng.integers(0, limit, 200, dtype=np.int32), rng.choice(extra, 200)]).astype(np.int32)
    perm = rng.permutation(len(a))
    a, b = a[perm], b[perm]
    bad = (a >= limit) | (b >= limit)
    assert 300 < bad.sum() < len(a) // 4
    dev = st.device
    return st, View(st, limit), torch.as_tensor(a, device=dev), torch.as_tensor(b, device=dev), bad


def host(r):
    return {k: v.cpu().numpy() for k, v in r.items()}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gjk_distance_guard(scene, precision):
    st, view, a, b, bad = scene
    got = host(gjk_distance_batch(view, a, b, precision=precision))
    assert (got["status"][bad] == _lib.STATUS_BAD_INDEX).all()
    assert np.isnan(got["dist"][bad]).all() and np.isnan(got["cp1"][bad]).all()
    assert (got["n_simplex"][bad] == 0).all()
    good = ~bad
    ok = torch.as_tensor(np.flatnonzero(good), device=st.device)
    want = host(gjk_distance_batch(st, a[ok], b[ok], precision=precision))
    for k in ("dist", "cp1", "cp2", "simplex", "n_simplex", "status", "iterations"):
        assert np.array_equal(got[k][good], want[k], equal_nan=True), k


def test_gjk_distance_cached_guard(scene):
    """The MeshGraph-cached entry point (one thread per pair): the same
    reports, and the cache entries of a rejected pair pass through."""
    st, view, a, b, bad = scene
    n = a.numel()
    cache = torch.full((n, 2), -1, dtype=torch.int32, device=st.device)
    cache[:, 1] = 7  # entries of colliders without meshes pass through
    got = host(gjk_distance_batch(view, a, b, mesh_cache=cache))
    assert (got["status"][bad] == _lib.STATUS_BAD_INDEX).all()
    assert np.isnan(got["dist"][bad]).all()
    c = cache.cpu().numpy()
    assert (c[:, 0] == -1).all() and (c[:, 1] == 7).all()
    good = ~bad
    ok = torch.as_tensor(np.flatnonzero(good), device=st.device)
    want = host(gjk_distance_batch(st, a[ok], b[ok]))
    for k in ("dist", "cp1", "cp2", "n_simplex", "status", "iterations"):
        assert np.array_equal(got[k][good], want[k], equal_nan=True), k


def test_gjk_intersection_guard(scene):
    st, view, a, b, bad = scene
    got = host(gjk_intersection_batch(view, a, b))
    assert (got["status"][bad] == _lib.STATUS_BAD_INDEX).all() and not got["hit"][bad].any()
    ok = torch.as_tensor(np.flatnonzero(~bad), device=st.device)
    want = host(gjk_intersection_batch(st, a[ok], b[ok]))
    assert np.array_equal(got["hit"][~bad], want["hit"]) and np.array_equal(got["status"][~bad], want["status"])


@pytest.mark.parametrize("precision,kw", [("fp64", {}), ("fp64", dict(max_iter=300)),
                                          ("mixed", dict(max_faces=256, max_loose_edges=128))])
def test_epa_guard(scene, precision, kw):
    st, view, a, b, bad = scene
    g = host(gjk_distance_batch(st, a, b))  # simplices for every pair (all indices are valid for the store)
    sel = np.flatnonzero(bad | ((g["dist"] == 0.0) & (g["n_simplex"] == 4)))
    s = torch.as_tensor(sel, device=st.device)
    got = host(epa_batch(view, a[s], b[s], g["simplex"][sel], precision=precision, **kw))
    badk = bad[sel]
    assert (got["status"][badk] == _lib.STATUS_BAD_INDEX).all()
    assert np.isnan(got["mtv"][badk]).all() and (got["n_faces"][badk] == 0).all()
    ok = torch.as_tensor(sel[~badk], device=st.device)
    want = host(epa_batch(st, a[ok], b[ok], g["simplex"][sel[~badk]], precision=precision, **kw))
    for k in ("mtv", "status", "n_faces"):
        assert np.array_equal(got[k][~badk], want[k], equal_nan=True), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mpr_guard(scene, precision):
    st, view, a, b, bad = scene
    got = host(mpr_batch(view, a, b, precision=precision))
    assert (got["status"][bad] == _lib.STATUS_BAD_INDEX).all() and not got["hit"][bad].any()
    assert np.isnan(got["depth"][bad]).all()
    ok = torch.as_tensor(np.flatnonzero(~bad), device=st.device)
    want = host(mpr_batch(st, a[ok], b[ok], precision=precision))
    for k in ("hit", "depth", "dir", "pos", "status"):
        assert np.array_equal(got[k][~bad], want[k], equal_nan=True), k


def test_support_and_aabb_guard(scene):
    st, view, a, b, bad = scene
    dirs = np.random.default_rng(2).normal(size=(len(a), 3))
    got = view.support(a, dirs).cpu().numpy()
    badi = (a >= view.n_colliders).cpu().numpy()
    assert np.isnan(got[badi]).all()
    assert np.array_equal(got[~badi], st.support(a[~torch.as_tensor(badi, device=st.device)],
                                                  dirs[~badi]).cpu().numpy())
    box = view.aabbs(a).cpu().numpy()
    assert np.isnan(box[badi]).all()
    assert np.array_equal(box[~badi], st.aabbs(a.cpu().numpy()[~badi]).cpu().numpy())
