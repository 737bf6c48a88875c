"""ctypes wrapper of the C oracle (test infrastructure only).

Every function takes a ``distance3d_gb300.collider_set.ColliderSet`` and
index arrays and returns NumPy arrays.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU legs use this module.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

I32P = ctypes.POINTER(ctypes.c_int32)
I64P = ctypes.POINTER(ctypes.c_int64)
I8P = ctypes.POINTER(ctypes.c_int8)
DP = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _set_args = [I32P, DP, DP, I64P, I32P, DP, I32P]
        _lib.orc_gjk_distance.argtypes = _set_args + [
            I32P, I32P, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, DP, DP, DP, DP, I8P, I8P, I32P, ctypes.c_int]
        _lib.orc_gjk_distance_cached.argtypes = _set_args + [
            I32P, I32P, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, I32P, DP, DP, DP, DP, I8P, I8P, I32P, ctypes.c_int]
        _lib.orc_gjk_intersection.argtypes = _set_args + [
            I32P, I32P, ctypes.c_int64, ctypes.c_double, ctypes.c_int, I8P, I8P, I32P, ctypes.c_int]
        _lib.orc_epa.argtypes = _set_args + [
            I32P, I32P, ctypes.c_int64, DP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_double, DP, I8P, I32P, DP, ctypes.c_int]
        _lib.orc_aabbs.argtypes = _set_args + [ctypes.c_int64, DP, ctypes.c_int]
        _lib.orc_support.argtypes = _set_args + [ctypes.c_int, DP, DP]
        _lib.orc_self_pairs.argtypes = [DP, ctypes.c_int64, I32P, ctypes.c_int64]
        _lib.orc_self_pairs.restype = ctypes.c_int64
        _lib.orc_cross_pairs.argtypes = [DP, ctypes.c_int64, DP, ctypes.c_int64, I32P, ctypes.c_int64]
        _lib.orc_cross_pairs.restype = ctypes.c_int64
        _lib.orc_self_pairs_sweep.argtypes = [DP, ctypes.c_int64, I32P, ctypes.c_int64]
        _lib.orc_self_pairs_sweep.restype = ctypes.c_int64
        _lib.orc_support_batch.argtypes = _set_args + [I32P, DP, ctypes.c_int64, DP, ctypes.c_int]
        _lib.orc_mpr.argtypes = _set_args + [
            I32P, I32P, ctypes.c_int64, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            I8P, DP, DP, DP, I8P, ctypes.c_int]
        _lib.orc_max_threads.restype = ctypes.c_int
        _lib.orc_box_vertices.argtypes = [DP, DP, DP]
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _set(cs):
    links = cs.links if len(cs.links) else None
    return [_p(cs.types, I32P), _p(cs.poses, DP), _p(cs.params, DP),
            _p(cs.hull_offset, I64P), _p(cs.hull_count, I32P), _p(cs.vertices, DP), _p(links, I32P)]


def max_threads():
    return lib().orc_max_threads()


def _idx(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def gjk_distance(cs, i1, i2, tolerance=1e-10, max_distance_squared=100000.0,
                 sanity_check=1e-8, max_iter=1024, nthreads=0):
    i1, i2 = _idx(i1), _idx(i2)
    n = len(i1)
    out = dict(dist=np.empty(n), cp1=np.empty((n, 3)), cp2=np.empty((n, 3)),
               simplex=np.empty((n, 4, 3)), n_simplex=np.empty(n, np.int8),
               status=np.empty(n, np.int8), iterations=np.empty(n, np.int32))
    lib().orc_gjk_distance(*_set(cs), _p(i1, I32P), _p(i2, I32P), n, tolerance,
                           max_distance_squared, sanity_check, max_iter,
                           _p(out["dist"], DP), _p(out["cp1"], DP), _p(out["cp2"], DP),
                           _p(out["simplex"], DP), _p(out["n_simplex"], I8P),
                           _p(out["status"], I8P), _p(out["iterations"], I32P), nthreads)
    return out


def gjk_distance_cached(cs, i1, i2, mesh_cache, tolerance=1e-10, max_distance_squared=100000.0,
                        sanity_check=1e-8, max_iter=1024, nthreads=0):
    """gjk_distance with the MeshGraph vertex cache (mesh.py:30, 82-85):
    ``mesh_cache`` (n,2) int32, -1 for the start vertex, is updated in place."""
    i1, i2 = _idx(i1), _idx(i2)
    n = len(i1)
    if (not isinstance(mesh_cache, np.ndarray) or mesh_cache.dtype != np.int32
            or mesh_cache.shape != (n, 2) or not mesh_cache.flags.c_contiguous):
        raise ValueError("mesh_cache must be a C-contiguous (n, 2) int32 array")
    out = dict(dist=np.empty(n), cp1=np.empty((n, 3)), cp2=np.empty((n, 3)),
               simplex=np.empty((n, 4, 3)), n_simplex=np.empty(n, np.int8),
               status=np.empty(n, np.int8), iterations=np.empty(n, np.int32))
    lib().orc_gjk_distance_cached(*_set(cs), _p(i1, I32P), _p(i2, I32P), n, tolerance,
                                  max_distance_squared, sanity_check, max_iter, _p(mesh_cache, I32P),
                                  _p(out["dist"], DP), _p(out["cp1"], DP), _p(out["cp2"], DP),
                                  _p(out["simplex"], DP), _p(out["n_simplex"], I8P),
                                  _p(out["status"], I8P), _p(out["iterations"], I32P), nthreads)
    return out


def gjk_intersection(cs, i1, i2, tolerance=1e-10, max_iter=1024, nthreads=0):
    i1, i2 = _idx(i1), _idx(i2)
    n = len(i1)
    hit = np.empty(n, np.int8)
    status = np.empty(n, np.int8)
    iters = np.empty(n, np.int32)
    lib().orc_gjk_intersection(*_set(cs), _p(i1, I32P), _p(i2, I32P), n, tolerance, max_iter,
                               _p(hit, I8P), _p(status, I8P), _p(iters, I32P), nthreads)
    return dict(hit=hit.astype(bool), status=status, iterations=iters)


def epa(cs, i1, i2, simplices, max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8,
        want_faces=False, nthreads=0):
    i1, i2 = _idx(i1), _idx(i2)
    n = len(i1)
    simplices = np.ascontiguousarray(simplices, dtype=np.float64).reshape(n, 4, 3)
    mtv = np.empty((n, 3))
    status = np.empty(n, np.int8)
    nf = np.empty(n, np.int32)
    faces = np.zeros((n, max_faces, 4, 3)) if want_faces else None
    lib().orc_epa(*_set(cs), _p(i1, I32P), _p(i2, I32P), n, _p(simplices, DP), max_iter,
                  max_loose_edges, max_faces, epsilon, _p(mtv, DP), _p(status, I8P),
                  _p(nf, I32P), _p(faces, DP), nthreads)
    out = dict(mtv=mtv, status=status, n_faces=nf)
    if want_faces:
        out["faces"] = faces
    return out


def mpr(cs, i1, i2, tolerance=0.0001, max_iterations=100, refine_limit=10000, penetration=True, nthreads=0):
    """MPR (mpr.py:21-110): hit, depth, dir, pos (NaN where the reference
    returns None), status."""
    i1, i2 = _idx(i1), _idx(i2)
    n = len(i1)
    out = dict(hit=np.empty(n, np.int8), depth=np.empty(n), dir=np.empty((n, 3)), pos=np.empty((n, 3)),
               status=np.empty(n, np.int8))
    lib().orc_mpr(*_set(cs), _p(i1, I32P), _p(i2, I32P), n, tolerance, max_iterations, refine_limit,
                  1 if penetration else 0, _p(out["hit"], I8P), _p(out["depth"], DP), _p(out["dir"], DP),
                  _p(out["pos"], DP), _p(out["status"], I8P), nthreads)
    out["hit"] = out["hit"].astype(bool)
    return out


def aabbs(cs, nthreads=0):
    n = len(cs)
    out = np.empty((n, 3, 2))
    lib().orc_aabbs(*_set(cs), n, _p(out, DP), nthreads)
    return out


def support(cs, idx, direction):
    d = np.ascontiguousarray(direction, dtype=np.float64)
    out = np.empty(3)
    lib().orc_support(*_set(cs), int(idx), _p(d, DP), _p(out, DP))
    return out


def box_vertices(pose12, size):
    pose12 = np.ascontiguousarray(pose12, dtype=np.float64)
    size = np.ascontiguousarray(size, dtype=np.float64)
    out = np.empty((8, 4))
    lib().orc_box_vertices(_p(pose12, DP), _p(size, DP), _p(out, DP))
    return out[:, :3]


def self_pairs(aabbs_):
    a = np.ascontiguousarray(aabbs_, dtype=np.float64).reshape(-1, 3, 2)
    n = lib().orc_self_pairs(_p(a, DP), len(a), None, 0)
    out = np.empty((n, 2), np.int32)
    lib().orc_self_pairs(_p(a, DP), len(a), _p(out, I32P), n)
    return out


def cross_pairs(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3, 2)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1, 3, 2)
    n = lib().orc_cross_pairs(_p(a, DP), len(a), _p(b, DP), len(b), None, 0)
    out = np.empty((n, 2), np.int32)
    lib().orc_cross_pairs(_p(a, DP), len(a), _p(b, DP), len(b), _p(out, I32P), n)
    return out


def self_pairs_sweep(aabbs_):
    """Same pair set as self_pairs (i < j, sorted), by sort and sweep."""
    a = np.ascontiguousarray(aabbs_, dtype=np.float64).reshape(-1, 3, 2)
    n = lib().orc_self_pairs_sweep(_p(a, DP), len(a), None, 0)
    out = np.empty((n, 2), np.int32)
    lib().orc_self_pairs_sweep(_p(a, DP), len(a), _p(out, I32P), n)
    return out[np.lexsort((out[:, 1], out[:, 0]))]


def support_batch(cs, idx, directions, nthreads=0):
    """(n,3) support points of colliders idx[k] along directions[k]."""
    idx = _idx(idx)
    d = np.ascontiguousarray(directions, dtype=np.float64).reshape(-1, 3)
    out = np.empty((len(idx), 3))
    lib().orc_support_batch(*_set(cs), _p(idx, I32P), _p(d, DP), len(idx), _p(out, DP), nthreads)
    return out


def distance_bracket(cs, i1, i2, cp1, cp2):
    """Certified bracket of the GJK distance from a candidate pair of points:
    ub = |cp1 - cp2| (the points are convex combinations of support points,
    so inside the shapes) and lb = u . (s1(-u) - s2(u)) with u the unit
    direction cp1 - cp2 (the support-function lower bound).  Returns (lb, ub)."""
    v = np.asarray(cp1) - np.asarray(cp2)
    ub = np.linalg.norm(v, axis=1)
    u = v / np.maximum(ub, 1e-300)[:, None]
    w = support_batch(cs, i1, -u) - support_batch(cs, i2, u)
    return np.sum(u * w, axis=1), ub


def depth_upper_bound(cs, i1, i2, normals):
    """h(n) = n . (s1(n) - s2(-n)) for unit normals: an upper bound on the
    penetration depth for every n (the depth is its minimum over n)."""
    n = np.asarray(normals, dtype=np.float64)
    w = support_batch(cs, i1, n) - support_batch(cs, i2, -n)
    return np.sum(n * w, axis=1)
