"""Minkowski portal refinement (MPR) on the GPU with distance3d's call
surface (mpr.py:21-110).

Drop-in functions:

* ``mpr_intersection(collider1, collider2, mpr_tolerance=0.0001,
  max_iterations=100)`` -> bool
* ``mpr_penetration(collider1, collider2, mpr_tolerance=0.0001,
  max_iterations=100)`` -> ``(intersection, depth, penetration_direction,
  contact_position)``, with ``None`` for the last three when the colliders do
  not intersect.

Batched function (new): ``mpr_batch`` takes a ``ColliderStore`` and two index
arrays and returns device tensors.  ``precision="fp64"`` (the default and the
drop-ins) gives the reference's results bit for bit; ``precision="mixed"``
searches the portal in FP32 and evaluates the final portal in FP64.
"""
import ctypes

import torch

from . import _lib
from .collider_set import ColliderSet
from .store import ColliderStore, as_index, _ptr

DEFAULT_REFINE_LIMIT = 10000
_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def mpr_batch(store, i1, i2, *, mpr_tolerance=0.0001, max_iterations=100, penetration=True,
              refine_limit=DEFAULT_REFINE_LIMIT, precision="fp64"):
    """MPR for pairs (i1[k], i2[k]) of ``store``.

    Returns a dict of device tensors: ``hit`` (n,) bool and ``status`` (n,)
    int8, and with ``penetration`` also ``depth`` (n,), ``dir`` (n,3) and
    ``pos`` (n,3) float64 (NaN where the pair does not intersect).
    ``status`` is ``STATUS_MAX_ITER`` where the portal refinement, which the
    reference runs without bound, took more than ``refine_limit`` steps.
    ``precision="mixed"`` runs the portal search in FP32 (pairs whose FP32
    refinement hits the bound rerun in FP64).
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
        hit = torch.empty(n, dtype=torch.int8, device=dev)
        status = torch.empty(n, dtype=torch.int8, device=dev)
        out = dict(status=status)
        if penetration:
            out.update(depth=torch.empty(n, dtype=torch.float64, device=dev),
                       dir=torch.empty((n, 3), dtype=torch.float64, device=dev),
                       pos=torch.empty((n, 3), dtype=torch.float64, device=dev))
        opt = _lib.MprOptions(float(mpr_tolerance), int(max_iterations), int(refine_limit), 1 if penetration else 0,
                              _PRECISIONS[precision])
        _lib.check(_lib.load().d3d_mpr(store.view, _ptr(a), _ptr(b), n, ctypes.byref(opt), _ptr(hit),
                                       _ptr(out.get("depth")), _ptr(out.get("dir")), _ptr(out.get("pos")),
                                       _ptr(status), store.stream()))
        out["hit"] = hit.bool()
        return out


def _pair(collider1, collider2):
    return ColliderStore(ColliderSet.from_colliders([collider1, collider2]))


def _check(r):
    if int(r["status"][0]) == _lib.STATUS_MAX_ITER:
        raise RuntimeError("MPR portal refinement did not finish within the iteration bound")


def mpr_intersection(collider1, collider2, mpr_tolerance=0.0001, max_iterations=100):
    """Drop-in for distance3d.mpr.mpr_intersection (mpr.py:21-50)."""
    r = mpr_batch(_pair(collider1, collider2), [0], [1], mpr_tolerance=mpr_tolerance,
                  max_iterations=max_iterations, penetration=False)
    _check(r)
    return bool(r["hit"][0])


def mpr_penetration(collider1, collider2, mpr_tolerance=0.0001, max_iterations=100):
    """Drop-in for distance3d.mpr.mpr_penetration (mpr.py:53-110)."""
    r = mpr_batch(_pair(collider1, collider2), [0], [1], mpr_tolerance=mpr_tolerance,
                  max_iterations=max_iterations, penetration=True)
    _check(r)
    h = {k: v.cpu().numpy() for k, v in r.items()}
    if not h["hit"][0]:
        return False, None, None, None
    return True, float(h["depth"][0]), h["dir"][0], h["pos"][0]
