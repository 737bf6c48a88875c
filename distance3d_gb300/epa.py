"""EPA on the GPU with distance3d's call surface.

* ``epa(simplex, collider1, collider2, max_iter=64, max_loose_edges=32,
  max_faces=64, epsilon=1e-8)`` -> ``(mtv, faces, success)``: drop-in for
  distance3d epa.epa (epa.py:9-78).  Raises AssertionError where the
  reference does (face buffer overflow, epa.py:128).
* ``epa_batch(store, i1, i2, simplex, ...)``: batched form on a
  ``ColliderStore``; per-pair ``status`` instead of exceptions.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .collider_set import ColliderSet
from .store import ColliderStore, as_index, _ptr


_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def _options(max_iter, max_loose_edges, max_faces, epsilon, precision="fp64"):
    if max_faces < 4:
        raise ValueError("max_faces must be >= 4")
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
    return _lib.EpaOptions(int(max_iter), int(max_loose_edges), int(max_faces), _PRECISIONS[precision],
                           float(epsilon))


def epa_batch(store, i1, i2, simplex, *, max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8,
              return_faces=False, scratch=None, precision="fp64"):
    """EPA for pairs (i1[k], i2[k]) starting from GJK simplices (n,4,3).

    Returns a dict of device tensors: ``mtv`` (n,3), ``status`` (n,) int8
    (0 converged, 4 max_iter, 5 face overflow, 6 degenerate), ``n_faces``
    (n,) int32 and, with ``return_faces``, ``faces`` (n,max_faces,4,3) whose
    first n_faces rows are valid.  ``scratch`` may pass a uint8 device tensor
    of at least ``epa_scratch_bytes(n, ...)`` bytes.  ``precision="fp64"``
    reproduces the reference bit for bit; ``"mixed"`` searches the polytope in
    FP32 and refines the final face in FP64.
    """
    dev = store.device
    lib = _lib.load()
    opt = _options(max_iter, max_loose_edges, max_faces, epsilon, precision)
    with torch.cuda.device(dev):
        a = as_index(i1, dev, store.n_colliders)
        b = as_index(i2, dev, store.n_colliders)
        n = a.numel()
        s = torch.as_tensor(simplex, dtype=torch.float64).reshape(n, 4, 3).to(dev).contiguous()
        mtv = torch.empty((n, 3), dtype=torch.float64, device=dev)
        status = torch.empty(n, dtype=torch.int8, device=dev)
        nf = torch.empty(n, dtype=torch.int32, device=dev)
        faces = torch.empty((n, max_faces, 4, 3), dtype=torch.float64, device=dev) if return_faces else None
        need = lib.d3d_epa_scratch_bytes(n, ctypes.byref(opt))
        if scratch is None or scratch.numel() < need:
            scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=dev)
        _lib.check(lib.d3d_epa(store.view, _ptr(a), _ptr(b), n, _ptr(s), ctypes.byref(opt), _ptr(mtv),
                               _ptr(status), _ptr(nf), _ptr(faces), _ptr(scratch), scratch.numel(),
                               store.stream()))
        out = dict(mtv=mtv, status=status, n_faces=nf)
        if return_faces:
            out["faces"] = faces
        return out


def epa_scratch_bytes(n, max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8, precision="fp64"):
    return int(_lib.load().d3d_epa_scratch_bytes(n, ctypes.byref(
        _options(max_iter, max_loose_edges, max_faces, epsilon, precision))))


def epa(simplex, collider1, collider2, max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8):
    """Drop-in for distance3d.epa.epa: ``(mtv, faces, success)``."""
    store = ColliderStore(ColliderSet.from_colliders([collider1, collider2]))
    r = epa_batch(store, [0], [1], np.asarray(simplex, dtype=np.float64).reshape(1, 4, 3), max_iter=max_iter,
                  max_loose_edges=max_loose_edges, max_faces=max_faces, epsilon=epsilon, return_faces=True)
    status = int(r["status"][0])
    if status == _lib.STATUS_EPA_FACE_OVERFLOW:
        raise AssertionError("EPA face buffer overflow (max_faces reached)")
    if status == _lib.STATUS_EPA_DEGENERATE:
        raise ValueError("EPA polytope lost every face")
    nf = int(r["n_faces"][0])
    return r["mtv"][0].cpu().numpy(), r["faces"][0, :nf].cpu().numpy(), status == _lib.STATUS_OK
