"""Launch parameters of the batch kernels and their autotuner.

``get_tuning()`` / ``set_tuning(**fields)`` read and set the process-wide
``d3d_tuning`` (GJK threads per block, resident GJK warps per SM, warp-EPA
pairs per block, type-sorting threshold); ``autotune(store, i1, i2)`` times
candidate settings on a sample of pairs (``d3d_autotune``), keeps the fastest
and returns it.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .store import as_index, _ptr

FIELDS = ("gjk_block", "gjk_warps_per_sm", "epa_warps", "sort_min")
_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def get_tuning():
    t = _lib.Tuning()
    _lib.check(_lib.load().d3d_get_tuning(ctypes.byref(t)))
    return {k: getattr(t, k) for k in FIELDS}


def set_tuning(**fields):
    cur = get_tuning()
    unknown = set(fields) - set(FIELDS)
    if unknown:
        raise ValueError(f"unknown tuning fields {sorted(unknown)}")
    cur.update(fields)
    t = _lib.Tuning(*[int(cur[k]) for k in FIELDS])
    _lib.check(_lib.load().d3d_set_tuning(ctypes.byref(t)))
    return cur


def autotune(store, i1, i2, *, precision="mixed", epa_kw=None, gjk_kw=None):
    """Time the candidates on pairs (i1[k], i2[k]) of ``store`` and keep the
    fastest setting; returns it as a dict."""
    ek = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
    ek.update(epa_kw or {})
    gk = dict(tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8, max_iterations=1024)
    gk.update(gjk_kw or {})
    gopt = _lib.GjkOptions(gk["tolerance"], gk["max_distance_squared"], gk["sanity_check"],
                           int(gk["max_iterations"]), _PRECISIONS[precision])
    eopt = _lib.EpaOptions(int(ek["max_iter"]), int(ek["max_loose_edges"]), int(ek["max_faces"]),
                           _PRECISIONS[precision], float(ek["epsilon"]))
    dev = store.device
    with torch.cuda.device(dev):
        a = as_index(i1, dev, store.n_colliders)
        b = as_index(i2, dev, store.n_colliders)
        t = _lib.Tuning()
        _lib.check(_lib.load().d3d_autotune(store.view, _ptr(a), _ptr(b), a.numel(), ctypes.byref(gopt),
                                            ctypes.byref(eopt), ctypes.byref(t), store.stream()))
    return {k: getattr(t, k) for k in FIELDS}
