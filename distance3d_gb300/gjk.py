"""GJK on the GPU with distance3d's call surface.

Drop-in functions (distance3d gjk/__init__.py:26-28, gjk/_gjk_jolt.py):

* ``gjk_distance_jolt(collider1, collider2, tolerance=1e-10,
  max_distance_squared=100000.0, sanity_check=1e-8)`` -> ``(distance,
  closest_point1, closest_point2, simplex)``; aliases ``gjk`` and
  ``gjk_distance``.
* ``gjk_intersection_jolt(collider1, collider2, tolerance=1e-10)`` -> bool;
  alias ``gjk_intersection``.

Batched functions (new): ``gjk_distance_batch`` and
``gjk_intersection_batch`` take a ``ColliderStore`` and two index arrays and
return device tensors.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .collider_set import ColliderSet
from .store import ColliderStore, as_index, _ptr

MAX_FLOAT = np.finfo(float).max
DEFAULT_MAX_ITERATIONS = 1024
_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def gjk_distance_batch(store, i1, i2, *, tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8,
                       max_iterations=DEFAULT_MAX_ITERATIONS, precision="fp64", out=None, mesh_cache=None):
    """Jolt GJK distance for pairs (i1[k], i2[k]) of ``store``.

    Returns a dict of device tensors: ``dist`` (n,) float64, ``cp1``/``cp2``
    (n,3), ``simplex`` (n,4,3), ``n_simplex`` (n,) int8, ``status`` (n,) int8
    (see ``distance3d_gb300.STATUS_*``), ``iterations`` (n,) int32.
    ``precision="fp64"`` reproduces the reference bit for bit;
    ``precision="mixed"`` runs the iterations in FP32 and refines in FP64.
    ``out`` may pass preallocated tensors with those keys.

    ``mesh_cache`` (an (n,2) int32 device tensor, updated in place) gives the
    MeshGraph supports of each pair the reference's vertex caching: the
    climbs of pair k start from mesh_cache[k] (-1: the mesh's start vertex)
    and leave their last answers there (d3d_gjk_distance_cached; FP64 only).
    """
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
    if mesh_cache is not None and precision != "fp64":
        raise ValueError("mesh_cache is the reference's vertex caching: precision must be 'fp64'")
    dev = store.device
    with torch.cuda.device(dev):
        a = as_index(i1, dev, store.n_colliders)
        b = as_index(i2, dev, store.n_colliders)
        if a.shape != b.shape or a.ndim != 1:
            raise ValueError("i1 and i2 must be 1-D of equal length")
        n = a.numel()
        if out is None:
            out = dict(dist=torch.empty(n, dtype=torch.float64, device=dev),
                       cp1=torch.empty((n, 3), dtype=torch.float64, device=dev),
                       cp2=torch.empty((n, 3), dtype=torch.float64, device=dev),
                       simplex=torch.empty((n, 4, 3), dtype=torch.float64, device=dev),
                       n_simplex=torch.empty(n, dtype=torch.int8, device=dev),
                       status=torch.empty(n, dtype=torch.int8, device=dev),
                       iterations=torch.empty(n, dtype=torch.int32, device=dev))
        opt = _lib.GjkOptions(tolerance, max_distance_squared, sanity_check, int(max_iterations),
                              _PRECISIONS[precision])
        if mesh_cache is not None:
            if (not isinstance(mesh_cache, torch.Tensor) or mesh_cache.device != torch.device(dev)
                    or mesh_cache.dtype != torch.int32 or tuple(mesh_cache.shape) != (n, 2)
                    or not mesh_cache.is_contiguous()):
                raise ValueError("mesh_cache must be a contiguous (n, 2) int32 tensor on the store's device")
            _lib.check(_lib.load().d3d_gjk_distance_cached(
                store.view, _ptr(a), _ptr(b), n, ctypes.byref(opt), _ptr(mesh_cache), _ptr(out["dist"]),
                _ptr(out["cp1"]), _ptr(out["cp2"]), _ptr(out["simplex"]), _ptr(out["n_simplex"]),
                _ptr(out["status"]), _ptr(out.get("iterations")), store.stream()))
            return out
        _lib.check(_lib.load().d3d_gjk_distance(
            store.view, _ptr(a), _ptr(b), n, ctypes.byref(opt), _ptr(out["dist"]), _ptr(out["cp1"]),
            _ptr(out["cp2"]), _ptr(out["simplex"]), _ptr(out["n_simplex"]), _ptr(out["status"]),
            _ptr(out.get("iterations")), store.stream()))
        return out


def gjk_intersection_batch(store, i1, i2, *, tolerance=1e-10, max_iterations=DEFAULT_MAX_ITERATIONS):
    """Jolt GJK intersection test for pairs (i1[k], i2[k]); dict with ``hit``
    (n,) bool and ``status`` (n,) int8 device tensors."""
    dev = store.device
    with torch.cuda.device(dev):
        a = as_index(i1, dev, store.n_colliders)
        b = as_index(i2, dev, store.n_colliders)
        n = a.numel()
        hit = torch.empty(n, dtype=torch.int8, device=dev)
        status = torch.empty(n, dtype=torch.int8, device=dev)
        _lib.check(_lib.load().d3d_gjk_intersection(store.view, _ptr(a), _ptr(b), n, tolerance,
                                                    int(max_iterations), _ptr(hit), _ptr(status), store.stream()))
        return dict(hit=hit.bool(), status=status)


def _pair_store(collider1, collider2):
    return ColliderStore(ColliderSet.from_colliders([collider1, collider2]))


def _mesh_cache_holder(c):
    """The object that holds a MeshGraph collider's vertex cache (``first_idx``):
    this package's MeshGraph, or the support object of distance3d's own
    (mesh.py:30, 85), also inside a Margin; None for other colliders."""
    if type(c).__name__ == "Margin":
        c = getattr(c, "collider", None)
    if c is None or type(c).__name__ != "MeshGraph":
        return None
    sf = getattr(c, "_support_function", None)
    return sf if sf is not None and hasattr(sf, "first_idx") else c


def gjk_distance_jolt(collider1, collider2, tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8):
    """Drop-in for distance3d.gjk.gjk_distance_jolt (_gjk_jolt.py:138-221).

    Returns ``(distance, closest_point1, closest_point2, simplex)``;
    ``(MAX_FLOAT, None, None, None)`` when the pair is clipped.  Raises
    AssertionError where the reference's sanity check (:215-216) fails.
    The simplex is (4,3); rows past the valid ones keep the reference's stale
    rows, and rows GJK never wrote are zero.
    """
    store = _pair_store(collider1, collider2)
    holders = [_mesh_cache_holder(collider1), _mesh_cache_holder(collider2)]
    cache = None
    if any(x is not None for x in holders):
        cache = torch.tensor([[int(x.first_idx) if x is not None else -1 for x in holders]], dtype=torch.int32,
                             device=store.device)
    r = gjk_distance_batch(store, [0], [1], tolerance=tolerance, max_distance_squared=max_distance_squared,
                           sanity_check=sanity_check, mesh_cache=cache)
    h = {k: v.cpu().numpy() for k, v in r.items()}
    if cache is not None:
        for x, v in zip(holders, cache.cpu().numpy()[0]):
            if x is not None:
                x.first_idx = int(v)
    status = int(h["status"][0])
    if status == _lib.STATUS_CLIPPED:
        return MAX_FLOAT, None, None, None
    if status == _lib.STATUS_SANITY:
        raise AssertionError("Sanity check failed")
    if status == _lib.STATUS_MAX_ITER:
        raise RuntimeError("GJK did not converge within the iteration bound")
    return float(h["dist"][0]), h["cp1"][0], h["cp2"][0], h["simplex"][0]


def gjk_intersection_jolt(collider1, collider2, tolerance=1e-10):
    """Drop-in for distance3d.gjk.gjk_intersection_jolt (_gjk_jolt.py:29-80)."""
    store = _pair_store(collider1, collider2)
    r = gjk_intersection_batch(store, [0], [1], tolerance=tolerance)
    if int(r["status"][0]) == _lib.STATUS_MAX_ITER:
        raise RuntimeError("GJK did not converge within the iteration bound")
    return bool(r["hit"][0])


gjk = gjk_distance_jolt
gjk_distance = gjk_distance_jolt
gjk_intersection = gjk_intersection_jolt
