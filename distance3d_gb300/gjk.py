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
                       max_iterations=DEFAULT_MAX_ITERATIONS, precision="fp64", out=None):
    """Jolt GJK distance for pairs (i1[k], i2[k]) of ``store``.

    Returns a dict of device tensors: ``dist`` (n,) float64, ``cp1``/``cp2``
    (n,3), ``simplex`` (n,4,3), ``n_simplex`` (n,) int8, ``status`` (n,) int8
    (see ``distance3d_gb300.STATUS_*``), ``iterations`` (n,) int32.
    ``precision="fp64"`` reproduces the reference bit for bit;
    ``precision="mixed"`` runs the iterations in FP32 and refines in FP64.
    ``out`` may pass preallocated tensors with those keys.
    """
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
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


def gjk_distance_jolt(collider1, collider2, tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8):
    """Drop-in for distance3d.gjk.gjk_distance_jolt (_gjk_jolt.py:138-221).

    Returns ``(distance, closest_point1, closest_point2, simplex)``;
    ``(MAX_FLOAT, None, None, None)`` when the pair is clipped.  Raises
    AssertionError where the reference's sanity check (:215-216) fails.
    The simplex is (4,3); rows past the valid ones keep the reference's stale
    rows, and rows GJK never wrote are zero.
    """
    store = _pair_store(collider1, collider2)
    r = gjk_distance_batch(store, [0], [1], tolerance=tolerance, max_distance_squared=max_distance_squared,
                           sanity_check=sanity_check)
    h = {k: v.cpu().numpy() for k, v in r.items()}
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
