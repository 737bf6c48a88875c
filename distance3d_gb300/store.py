"""Device-resident collider store.

A ``ColliderStore`` holds one packed batch of colliders in HBM as the kernels
read it (see include/d3d_gb300.h, ``d3d_store``): a 128-byte FP64 record and a
64-byte FP32 record per collider (pose and size parameters, 16-byte aligned
for 128-bit loads), a 16-byte meta record (type, vertex count, vertex
offset), and a vertex pool in FP64 and FP32 with every vertex padded to four
components.  Hull vertices are copied in as given; every box gets 8 derived
vertices appended after them (geometry.py:138-157).

Tensors are allocated through PyTorch (caching allocator) on the store's
device; every call enqueues work on the current PyTorch stream of that device.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .collider_set import ColliderSet, BOX, HULL, MARGIN


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def as_index(x, device, n=None):
    """int32 device tensor from an index sequence.

    A host sequence (NumPy array, list, CPU tensor) with an entry outside
    [0, n) raises IndexError before anything is copied to the device.  Device
    tensors are not read back here: the kernels check their entries and
    report D3D_STATUS_BAD_INDEX for each pair with an index out of range.
    """
    if isinstance(x, torch.Tensor) and x.device.type != "cpu":
        return x.to(device=device, dtype=torch.int32).contiguous()
    a = np.asarray(x.numpy() if isinstance(x, torch.Tensor) else x)
    if a.size and not np.issubdtype(a.dtype, np.integer):
        raise TypeError(f"collider indices must be integers, got {a.dtype}")
    if n is not None and a.size:
        lo, hi = int(a.min()), int(a.max())
        if lo < 0 or hi >= n:
            raise IndexError(f"collider index {lo if lo < 0 else hi} out of range [0, {n})")
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device)


class PinnedColliderSet:
    """A ColliderSet staged in page-locked host memory, so that building a
    store from it is a set of asynchronous host-to-device copies."""

    def __init__(self, cs):
        boxes = np.flatnonzero(cs.base_types == BOX)
        offsets = cs.hull_offset.copy()
        counts = cs.hull_count.copy()
        offsets[boxes] = cs.n_vertices + 8 * np.arange(len(boxes), dtype=np.int64)
        counts[boxes] = 8
        self.n = len(cs)
        self.n_hull_vertices = cs.n_vertices
        self.n_vertices = cs.n_vertices + 8 * len(boxes)
        self.types_host = cs.types.copy()

        def pin(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        self.types = pin(cs.types)
        self.poses = pin(cs.poses)
        self.params = pin(cs.params)
        self.offsets = pin(offsets)
        self.counts = pin(counts)
        self.vertices = pin(cs.vertices)
        self.links = pin(cs.links)

    def nbytes(self):
        return sum(t.numel() * t.element_size() for t in
                   (self.types, self.poses, self.params, self.offsets, self.counts, self.vertices, self.links))


class ColliderStore:
    """Packed colliders resident on one CUDA device.

    ``colliders`` is a ColliderSet, a PinnedColliderSet (copied
    asynchronously on the current stream) or a sequence of collider objects.
    """

    def __init__(self, colliders, device="cuda"):
        if isinstance(colliders, PinnedColliderSet):
            self._init_pinned(colliders, device)
            return
        if not isinstance(colliders, ColliderSet):
            colliders = ColliderSet.from_colliders(list(colliders))
        lib = _lib.load()
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("ColliderStore needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        cs = colliders
        n = len(cs)
        boxes = np.flatnonzero(cs.base_types == BOX)
        nv_hull = cs.n_vertices
        n_vertices = nv_hull + 8 * len(boxes)
        offsets = cs.hull_offset.copy()
        counts = cs.hull_count.copy()
        offsets[boxes] = nv_hull + 8 * np.arange(len(boxes), dtype=np.int64)
        counts[boxes] = 8
        dev = self.device
        self.n_colliders = n
        self.n_vertices = n_vertices
        self.types_host = cs.types.copy()
        with torch.cuda.device(dev):
            self.rec64 = torch.empty((max(n, 1), 16), dtype=torch.float64, device=dev)
            self.rec32 = torch.empty((max(n, 1), 16), dtype=torch.float32, device=dev)
            self.meta = torch.empty((max(n, 1), 4), dtype=torch.int32, device=dev)
            self.verts64 = torch.zeros((max(n_vertices, 1), 4), dtype=torch.float64, device=dev)
            self.verts32 = torch.empty((max(n_vertices, 1), 4), dtype=torch.float32, device=dev)
            if nv_hull:
                self.verts64[:nv_hull].copy_(torch.from_numpy(cs.vertices))
            self.links = torch.from_numpy(cs.links).to(dev) if len(cs.links) else None
            types = torch.from_numpy(cs.types).to(dev)
            poses = torch.from_numpy(cs.poses).to(dev)
            params = torch.from_numpy(cs.params).to(dev)
            offs = torch.from_numpy(offsets).to(dev)
            cnts = torch.from_numpy(counts).to(dev)
            self._view = _lib.D3DStore(n, n_vertices, self.rec64.data_ptr(), self.rec32.data_ptr(),
                                       self.meta.data_ptr(), self.verts64.data_ptr(), self.verts32.data_ptr(),
                                       self.links.data_ptr() if self.links is not None else None,
                                       len(cs.links))
            _lib.check(lib.d3d_store_pack(ctypes.byref(self._view), _ptr(types), _ptr(poses), _ptr(params),
                                          _ptr(offs), _ptr(cnts), nv_hull, _stream(dev)))

    def _init_pinned(self, p, device):
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        dev = self.device
        n, nv = p.n, p.n_vertices
        self.n_colliders = n
        self.n_vertices = nv
        self.types_host = p.types_host
        with torch.cuda.device(dev):
            self.rec64 = torch.empty((max(n, 1), 16), dtype=torch.float64, device=dev)
            self.rec32 = torch.empty((max(n, 1), 16), dtype=torch.float32, device=dev)
            self.meta = torch.empty((max(n, 1), 4), dtype=torch.int32, device=dev)
            self.verts64 = torch.empty((max(nv, 1), 4), dtype=torch.float64, device=dev)
            self.verts32 = torch.empty((max(nv, 1), 4), dtype=torch.float32, device=dev)
            self.links = torch.empty(p.links.numel(), dtype=torch.int32, device=dev) if p.links.numel() else None
            self._staging = {k: torch.empty(getattr(p, k).shape, dtype=getattr(p, k).dtype, device=dev)
                             for k in ("types", "poses", "params", "offsets", "counts")}
            self._view = _lib.D3DStore(n, nv, self.rec64.data_ptr(), self.rec32.data_ptr(),
                                       self.meta.data_ptr(), self.verts64.data_ptr(), self.verts32.data_ptr(),
                                       self.links.data_ptr() if self.links is not None else None,
                                       p.links.numel())
        self._shape = (p.n, p.n_vertices, p.n_hull_vertices, p.links.numel())
        self.update(p)

    def update(self, p):
        """Copy the colliders of a PinnedColliderSet of this store's shape
        (same collider, vertex and link counts, the same boxes) into this
        store and pack them again, asynchronously on the current stream (the
        packing validates the records and synchronises with that stream).
        The store's device buffers stay the same, so CUDA graphs captured on
        it (``serve.CollisionBatch``) serve the new colliders."""
        if not isinstance(p, PinnedColliderSet) or getattr(self, "_shape", None) != (
                p.n, p.n_vertices, p.n_hull_vertices, p.links.numel()):
            raise ValueError("update() needs a PinnedColliderSet of the shape this store was built from")
        dev = self.device
        with torch.cuda.device(dev):
            if p.n_hull_vertices:
                self.verts64[:p.n_hull_vertices].copy_(p.vertices, non_blocking=True)
            if self.links is not None:
                self.links.copy_(p.links, non_blocking=True)
            st = self._staging
            for k in st:
                st[k].copy_(getattr(p, k), non_blocking=True)
            _lib.check(_lib.load().d3d_store_pack(ctypes.byref(self._view), _ptr(st["types"]), _ptr(st["poses"]),
                                                  _ptr(st["params"]), _ptr(st["offsets"]), _ptr(st["counts"]),
                                                  p.n_hull_vertices, _stream(dev)))

    def __len__(self):
        return self.n_colliders

    @property
    def view(self):
        """ctypes ``d3d_store`` pointing at this store's tensors."""
        return ctypes.byref(self._view)

    def stream(self):
        return _stream(self.device)

    def nbytes(self):
        return sum(t.numel() * t.element_size() for t in
                   (self.rec64, self.rec32, self.meta, self.verts64, self.verts32)) + \
            (self.links.numel() * 4 if self.links is not None else 0)

    def set_poses(self, idx, poses):
        """Set 4x4 (or 12-value R|t) poses of colliders ``idx`` (not hulls)."""
        idx_np = np.asarray(idx.cpu() if isinstance(idx, torch.Tensor) else idx, dtype=np.int64).reshape(-1)
        ii = as_index(idx_np, self.device, self.n_colliders)
        if np.any((self.types_host[idx_np] & ~MARGIN) == HULL):
            raise NotImplementedError("update_pose is not implemented for ConvexHullVertices")
        p = torch.as_tensor(poses, dtype=torch.float64)
        if p.ndim == 3:
            p = torch.cat([p[:, :3, :3].reshape(-1, 9), p[:, :3, 3]], dim=1)
        p = p.reshape(-1, 12).to(self.device).contiguous()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().d3d_store_set_poses(self.view, _ptr(ii), _ptr(p), len(ii), self.stream()))

    def aabbs(self, idx=None):
        """(n,3,2) FP64 AABBs ([axis][min,max]) of colliders ``idx`` (all if None)."""
        with torch.cuda.device(self.device):
            if idx is None:
                n = self.n_colliders
                ii = None
            else:
                ii = as_index(idx, self.device, self.n_colliders)
                n = len(ii)
            out = torch.empty((n, 3, 2), dtype=torch.float64, device=self.device)
            _lib.check(_lib.load().d3d_aabbs(self.view, _ptr(ii), n, _ptr(out), self.stream()))
            return out

    def support(self, idx, directions):
        """(n,3) FP64 support points of colliders ``idx`` along ``directions``."""
        with torch.cuda.device(self.device):
            ii = as_index(idx, self.device, self.n_colliders)
            d = torch.as_tensor(directions, dtype=torch.float64).reshape(-1, 3).to(self.device).contiguous()
            out = torch.empty((len(ii), 3), dtype=torch.float64, device=self.device)
            _lib.check(_lib.load().d3d_support(self.view, _ptr(ii), _ptr(d), len(ii), _ptr(out), self.stream()))
            return out
