"""Broad phase then narrow phase over a whole scene, on the device.

``collide_scene(store)`` computes every collider's FP64 AABB (containment.py
formulas), builds the LBVH, takes the overlapping pairs (i < j, sorted,
the pair set of ``BoundingVolumeHierarchy.aabb_overlapping_with_self`` /
``AabbTree.overlaps_aabb_tree``, broad_phase.py:229-252, aabb_tree.py:121-191)
and runs GJK distance and EPA (``d3d_collide``) on them -- the reference's
broad phase followed by gjk() / epa() per candidate pair.
"""
import ctypes
import time

import torch

from . import _lib
from .bvh import LBVH
from .store import _ptr

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def collide_scene(store, *, precision="mixed", epa_kw=None, gjk_kw=None, timings=False):
    """Returns (pairs (P,2) int32 device tensor, results dict of device
    tensors as d3d_collide's outputs: dist, cp1, cp2, simplex, n_simplex,
    status, iterations, mtv, epa_status (-1: no EPA), n_faces).  With
    ``timings``, a third item gives device milliseconds per stage (aabbs,
    lbvh_build, self_pairs, gjk_epa)."""
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
    ek = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
    ek.update(epa_kw or {})
    gk = dict(tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8, max_iterations=1024)
    gk.update(gjk_kw or {})
    gopt = _lib.GjkOptions(gk["tolerance"], gk["max_distance_squared"], gk["sanity_check"],
                           int(gk["max_iterations"]), _PRECISIONS[precision])
    eopt = _lib.EpaOptions(int(ek["max_iter"]), int(ek["max_loose_edges"]), int(ek["max_faces"]),
                           _PRECISIONS[precision], float(ek["epsilon"]))
    dev = store.device
    lib = _lib.load()
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(stream)
        aabbs = store.aabbs()
        ev[1].record(stream)
        tree = LBVH(aabbs, device=dev)
        ev[2].record(stream)
        pairs = tree.self_pairs()
        ev[3].record(stream)
        n = pairs.shape[0]
        out = {"dist": torch.empty(n, dtype=torch.float64, device=dev),
               "cp1": torch.empty((n, 3), dtype=torch.float64, device=dev),
               "cp2": torch.empty((n, 3), dtype=torch.float64, device=dev),
               "simplex": torch.empty((n, 4, 3), dtype=torch.float64, device=dev),
               "n_simplex": torch.empty(n, dtype=torch.int8, device=dev),
               "status": torch.empty(n, dtype=torch.int8, device=dev),
               "iterations": torch.empty(n, dtype=torch.int32, device=dev),
               "mtv": torch.empty((n, 3), dtype=torch.float64, device=dev),
               "epa_status": torch.empty(n, dtype=torch.int8, device=dev),
               "n_faces": torch.empty(n, dtype=torch.int32, device=dev)}
        if n:
            i1 = pairs[:, 0].contiguous()
            i2 = pairs[:, 1].contiguous()
            n_dev = torch.full((1,), n, dtype=torch.int64, device=dev)
            scratch = torch.empty(lib.d3d_collide_scratch_bytes(n, ctypes.byref(gopt), ctypes.byref(eopt)),
                                  dtype=torch.uint8, device=dev)
            o = out
            _lib.check(lib.d3d_collide(store.view, _ptr(i1), _ptr(i2), n, _ptr(n_dev), ctypes.byref(gopt),
                                       ctypes.byref(eopt), _ptr(o["dist"]), _ptr(o["cp1"]), _ptr(o["cp2"]),
                                       _ptr(o["simplex"]), _ptr(o["n_simplex"]), _ptr(o["status"]),
                                       _ptr(o["iterations"]), _ptr(o["mtv"]), _ptr(o["epa_status"]),
                                       _ptr(o["n_faces"]), _ptr(scratch), scratch.numel(), store.stream()))
        ev[4].record(stream)
        if not timings:
            return pairs, out
        ev[4].synchronize()
        names = ("aabbs", "lbvh_build", "self_pairs", "gjk_epa")
        return pairs, out, {k: ev[j].elapsed_time(ev[j + 1]) for j, k in enumerate(names)}
