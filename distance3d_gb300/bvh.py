"""Linear BVH over FP64 axis-aligned boxes on the GPU (d3d_bvh_* in
include/d3d_gb300.h).

``LBVH(aabbs)`` builds the tree over ``aabbs`` (n,3,2) ([axis][min,max]);
``self_pairs()`` returns every overlapping pair (i, j), i < j, ascending, and
``query(boxes)`` every (leaf, query) pair, ascending.  Overlap is the
reference's closed-interval test (distance3d aabb_tree.py:504-527), evaluated
on the exact FP64 boxes, so the pair sets equal the reference's.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .store import _ptr


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def as_boxes(aabbs, device):
    t = torch.as_tensor(np.asarray(aabbs, dtype=np.float64)) if not isinstance(aabbs, torch.Tensor) else aabbs
    t = t.to(device=device, dtype=torch.float64).reshape(-1, 3, 2).contiguous()
    return t


class LBVH:
    """A built tree; keeps a reference to its boxes."""

    def __init__(self, aabbs, device="cuda"):
        lib = _lib.load()
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        with torch.cuda.device(self.device):
            self.aabbs = as_boxes(aabbs, self.device)
            self.n = self.aabbs.shape[0]
            nbytes = lib.d3d_bvh_bytes(self.n)
            self.tree = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
            _lib.check(lib.d3d_bvh_build(_ptr(self.aabbs), self.n, _ptr(self.tree), self.tree.numel(),
                                         _stream(self.device)))
        self._capacity = max(1024, 4 * self.n)

    def _run(self, fn, *args):
        lib = _lib.load()
        cap = self._capacity
        for _ in range(3):
            scratch = torch.empty(lib.d3d_bvh_query_bytes(cap), dtype=torch.uint8, device=self.device)
            pairs = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=self.device)
            count = ctypes.c_int64(0)
            rc = fn(_ptr(self.aabbs), self.n, _ptr(self.tree), *args, _ptr(pairs), cap, ctypes.byref(count),
                    _ptr(scratch), scratch.numel(), _stream(self.device))
            if rc == _lib.D3D_ERR_CAPACITY and count.value > cap:
                cap = int(count.value)
                self._capacity = cap
                continue
            _lib.check(rc)
            return pairs[:count.value]
        raise _lib.D3DError(_lib.D3D_ERR_CAPACITY, "pair count kept growing")

    def refit(self, aabbs):
        """Move the leaves to new boxes (same count and order of leaves),
        keeping the tree's topology (d3d_bvh_refit)."""
        with torch.cuda.device(self.device):
            b = as_boxes(aabbs, self.device)
            if b.shape[0] != self.n:
                raise ValueError(f"refit needs {self.n} boxes, got {b.shape[0]}")
            self.aabbs = b
            _lib.check(_lib.load().d3d_bvh_refit(_ptr(self.aabbs), self.n, _ptr(self.tree), self.tree.numel(),
                                                 _stream(self.device)))
        return self

    def self_pairs(self):
        """(P,2) int32 device tensor of overlapping pairs (i, j), i < j, sorted."""
        with torch.cuda.device(self.device):
            return self._run(_lib.load().d3d_bvh_self_pairs)

    def query(self, boxes):
        """(P,2) int32 device tensor of (leaf, query) overlapping pairs, sorted."""
        with torch.cuda.device(self.device):
            b = as_boxes(boxes, self.device)
            lib = _lib.load()
            return self._run(lambda a, n, t, *rest: lib.d3d_bvh_query(a, n, t, _ptr(b), b.shape[0], *rest))
