"""Batched self-collision checks of serial robot arms.

``SerialArm`` describes a serial chain of revolute joints with collision
bodies fixed to its links (what distance3d builds from a URDF with
``BoundingVolumeHierarchy.fill_tree_with_colliders``, broad_phase.py:53-127);
``SerialArm.synthetic`` draws a 7-DoF arm with 30 bodies (capsules, boxes,
cylinders).  ``pair_table`` lists the body pairs a self-collision check tests:
all pairs except those on the same, the parent or the child link
(self_collision_whitelists, urdf_utils.py:39-64).

``SelfCollisionBatch`` checks many joint configurations at once: forward
kinematics on the device (``d3d_chain_fk``), pose update of the resident
store, then GJK distance and EPA on every listed pair of every configuration
(``d3d_collide``), captured as one CUDA graph.  ``contacts`` has, per
configuration and body, what distance3d's ``self_collision.detect``
(self_collision.py:5-37) returns per collider frame: whether the body
intersects any body outside its whitelist; ``any`` is ``detect_any``
(self_collision.py:40-64).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .collider_set import BOX, CAPSULE, CYLINDER, ColliderSet
from .store import ColliderStore, _ptr

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def _rt(R, t):
    return np.concatenate([np.asarray(R, dtype=np.float64).reshape(9), np.asarray(t, dtype=np.float64)])


def _compose(A, B):
    """12-value transforms, the device kernel's rounding order."""
    Ra, ta, Rb, tb = A[:9], A[9:], B[:9], B[9:]
    R = np.empty(9)
    t = np.empty(3)
    for i in range(3):
        for j in range(3):
            R[3 * i + j] = Ra[3 * i] * Rb[j] + Ra[3 * i + 1] * Rb[3 + j] + Ra[3 * i + 2] * Rb[6 + j]
        t[i] = Ra[3 * i] * tb[0] + Ra[3 * i + 1] * tb[1] + Ra[3 * i + 2] * tb[2] + ta[i]
    return np.concatenate([R, t])


def _axis_angle(a, q):
    s, c = np.sin(q), np.cos(q)
    C = 1.0 - c
    x, y, z = a
    return np.array([c + x * x * C, x * y * C - z * s, x * z * C + y * s,
                     y * x * C + z * s, c + y * y * C, y * z * C - x * s,
                     z * x * C - y * s, z * y * C + x * s, c + z * z * C, 0.0, 0.0, 0.0])


class SerialArm:
    """Serial chain: joint j (revolute, unit axis ``joint_axis[j]``) sits at
    ``joint_origin[j]`` of link j and moves link j+1; body b (type, params as
    ``ColliderSet``) is fixed to link ``body_link[b]`` at ``body_origin[b]``.
    Transforms are 12 values (R row-major, t)."""

    def __init__(self, joint_axis, joint_origin, body_link, body_origin, body_type, body_params):
        self.joint_axis = np.asarray(joint_axis, dtype=np.float64).reshape(-1, 3)
        self.joint_origin = np.asarray(joint_origin, dtype=np.float64).reshape(-1, 12)
        self.body_link = np.asarray(body_link, dtype=np.int32)
        self.body_origin = np.asarray(body_origin, dtype=np.float64).reshape(-1, 12)
        self.body_type = np.asarray(body_type, dtype=np.int32)
        self.body_params = np.asarray(body_params, dtype=np.float64).reshape(-1, 4)
        if np.any(self.body_type == 5):
            raise ValueError("bodies must be posable (no ConvexHullVertices)")
        self.dof = len(self.joint_axis)
        self.n_bodies = len(self.body_link)

    @classmethod
    def synthetic(cls, seed=0, dof=7, n_bodies=30):
        """Link lengths U[0.1, 0.4] m along each link's z, joint axes
        alternating z and y; bodies spread over the base and the links:
        capsules (r 0.04-0.08), boxes and cylinders along their link."""
        rng = np.random.default_rng(seed)
        lengths = rng.uniform(0.1, 0.4, dof)
        axes = np.array([[0.0, 0.0, 1.0] if j % 2 == 0 else [0.0, 1.0, 0.0] for j in range(dof)])
        origins = [_rt(np.eye(3), [0.0, 0.0, 0.0 if j == 0 else lengths[j - 1]]) for j in range(dof)]
        link = np.sort(rng.integers(0, dof + 1, n_bodies)).astype(np.int32)
        types, params, borigin = [], [], []
        for b in range(n_bodies):
            L = lengths[link[b] - 1] if link[b] > 0 else 0.15
            kind = rng.integers(0, 3)
            # small tilt about a random horizontal axis, placed along the link
            ang = rng.uniform(-0.3, 0.3)
            ax = rng.normal(size=2)
            ax = np.array([ax[0], ax[1], 0.0]) / np.linalg.norm(ax)
            R = _axis_angle(ax, ang)[:9].reshape(3, 3)
            t = [rng.uniform(-0.03, 0.03), rng.uniform(-0.03, 0.03), rng.uniform(0.1, 0.9) * L]
            borigin.append(_rt(R, t))
            if kind == 0:
                types.append(CAPSULE)
                params.append([rng.uniform(0.04, 0.08), rng.uniform(0.3, 0.8) * L, 0.0, 0.0])
            elif kind == 1:
                types.append(BOX)
                params.append([rng.uniform(0.04, 0.12), rng.uniform(0.04, 0.12), rng.uniform(0.3, 0.8) * L, 0.0])
            else:
                types.append(CYLINDER)
                params.append([rng.uniform(0.04, 0.08), rng.uniform(0.3, 0.8) * L, 0.0, 0.0])
        return cls(axes, np.array(origins), link, np.array(borigin), types, params)

    def pair_table(self):
        """(P,2) body pairs a < b whose links differ by more than one (the
        whitelist excludes the same, the parent and the child link)."""
        a, b = np.triu_indices(self.n_bodies, k=1)
        keep = np.abs(self.body_link[a] - self.body_link[b]) > 1
        return np.stack([a[keep], b[keep]], axis=1).astype(np.int32)

    def fk(self, q):
        """Body poses (n_bodies, 12) for one configuration (NumPy, the device
        kernel's arithmetic; sin/cos may differ by an ulp)."""
        T = [np.array([1.0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0])]
        for j in range(self.dof):
            T.append(_compose(_compose(T[-1], self.joint_origin[j]), _axis_angle(self.joint_axis[j], q[j])))
        return np.array([_compose(T[self.body_link[b]], self.body_origin[b]) for b in range(self.n_bodies)])

    def collider_set(self, n_configs):
        """ColliderSet of n_configs copies of the bodies (identity poses),
        collider c * n_bodies + b = body b of configuration c."""
        n = n_configs * self.n_bodies
        poses = np.tile(np.array([1.0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]), (n, 1))
        return ColliderSet(np.tile(self.body_type, n_configs), poses, np.tile(self.body_params, (n_configs, 1)),
                           np.full(n, -1, dtype=np.int64), np.zeros(n, dtype=np.int32), np.zeros((0, 4)))


class SelfCollisionBatch:
    """Self-collision checks of ``n_configs`` configurations of ``arm`` per
    call, on one GPU; ``run(q)`` with q (n_configs, dof) joint values."""

    def __init__(self, arm, n_configs, *, precision="mixed", epa_kw=None, graph=True, device="cuda"):
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
        self.arm = arm
        self.n_configs = int(n_configs)
        dev = torch.device(device)
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        ek = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
        ek.update(epa_kw or {})
        self._gjk = _lib.GjkOptions(1e-10, 100000.0, 1e-8, 1024, _PRECISIONS[precision])
        self._epa = _lib.EpaOptions(int(ek["max_iter"]), int(ek["max_loose_edges"]), int(ek["max_faces"]),
                                    _PRECISIONS[precision], float(ek["epsilon"]))
        lib = _lib.load()
        nb = arm.n_bodies
        table = arm.pair_table()
        self.n_pair_types = len(table)
        with torch.cuda.device(dev):
            self.store = ColliderStore(arm.collider_set(self.n_configs), device=dev)
            t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
            self._axis = t(arm.joint_axis, torch.float64)
            self._origin = t(arm.joint_origin, torch.float64)
            self._blink = t(arm.body_link, torch.int32)
            self._borigin = t(arm.body_origin, torch.float64)
            self._chain = _lib.Chain(arm.dof, nb, _ptr(self._axis), _ptr(self._origin), _ptr(self._blink),
                                     _ptr(self._borigin))
            base = torch.arange(self.n_configs, dtype=torch.int64, device=dev)[:, None] * nb
            self.i1 = (base + t(table[:, 0], torch.int64)[None, :]).reshape(-1).to(torch.int32).contiguous()
            self.i2 = (base + t(table[:, 1], torch.int64)[None, :]).reshape(-1).to(torch.int32).contiguous()
            self._pa = t(table[:, 0], torch.int64)
            self._pb = t(table[:, 1], torch.int64)
            self.n_pairs = self.i1.numel()
            self.q = torch.zeros((self.n_configs, arm.dof), dtype=torch.float64, device=dev)
            self.poses = torch.empty((self.n_configs * nb, 12), dtype=torch.float64, device=dev)
            self.idx = torch.arange(self.n_configs * nb, dtype=torch.int32, device=dev)
            self.n_dev = torch.full((1,), self.n_pairs, dtype=torch.int64, device=dev)
            n = self.n_pairs
            self.out = {"dist": torch.empty(n, dtype=torch.float64, device=dev),
                        "cp1": torch.empty((n, 3), dtype=torch.float64, device=dev),
                        "cp2": torch.empty((n, 3), dtype=torch.float64, device=dev),
                        "simplex": torch.empty((n, 4, 3), dtype=torch.float64, device=dev),
                        "n_simplex": torch.empty(n, dtype=torch.int8, device=dev),
                        "status": torch.empty(n, dtype=torch.int8, device=dev),
                        "iterations": torch.empty(n, dtype=torch.int32, device=dev),
                        "mtv": torch.empty((n, 3), dtype=torch.float64, device=dev),
                        "epa_status": torch.empty(n, dtype=torch.int8, device=dev),
                        "n_faces": torch.empty(n, dtype=torch.int32, device=dev)}
            self.scratch = torch.empty(lib.d3d_collide_scratch_bytes(n, ctypes.byref(self._gjk),
                                                                     ctypes.byref(self._epa)),
                                       dtype=torch.uint8, device=dev)
            self.contacts = torch.zeros((self.n_configs, nb), dtype=torch.bool, device=dev)
            self.stream = torch.cuda.Stream(dev)
            self.graph = None
            with torch.cuda.stream(self.stream):
                self._launch()
            self.stream.synchronize()
            if graph:
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=self.stream):
                    self._launch()
                self.graph = g

    def _launch(self):
        lib = _lib.load()
        s = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(lib.d3d_chain_fk(ctypes.byref(self._chain), _ptr(self.q), self.n_configs, _ptr(self.poses), s))
        _lib.check(lib.d3d_store_set_poses(self.store.view, _ptr(self.idx), _ptr(self.poses), self.idx.numel(), s))
        o = self.out
        _lib.check(lib.d3d_collide(self.store.view, _ptr(self.i1), _ptr(self.i2), self.n_pairs, _ptr(self.n_dev),
                                   ctypes.byref(self._gjk), ctypes.byref(self._epa), _ptr(o["dist"]),
                                   _ptr(o["cp1"]), _ptr(o["cp2"]), _ptr(o["simplex"]), _ptr(o["n_simplex"]),
                                   _ptr(o["status"]), _ptr(o["iterations"]), _ptr(o["mtv"]),
                                   _ptr(o["epa_status"]), _ptr(o["n_faces"]), _ptr(self.scratch),
                                   self.scratch.numel(), s))
        # contacts[c, body] = the body touches any listed partner (detect, self_collision.py:5-37)
        hit = (o["dist"] == 0.0).view(self.n_configs, self.n_pair_types)
        self.contacts.zero_()
        self.contacts.index_put_((torch.arange(self.n_configs, device=self.device)[:, None], self._pa[None, :]),
                                 hit, accumulate=True)
        self.contacts.index_put_((torch.arange(self.n_configs, device=self.device)[:, None], self._pb[None, :]),
                                 hit, accumulate=True)

    def run(self, q, sync=True):
        """Check configurations q (n_configs, dof); returns the outputs as
        device tensors: ``dist`` (n_configs, P) and ``mtv`` (n_configs, P, 3)
        per listed pair, ``contacts`` (n_configs, n_bodies) and ``any``
        (n_configs,)."""
        with torch.cuda.device(self.device):
            self.q.copy_(torch.as_tensor(q, dtype=torch.float64), non_blocking=True)
            cur = torch.cuda.current_stream(self.device)
            self.stream.wait_stream(cur)
            with torch.cuda.stream(self.stream):
                if self.graph is not None:
                    self.graph.replay()
                else:
                    self._launch()
            cur.wait_stream(self.stream)
            if sync:
                cur.synchronize()
            C, P = self.n_configs, self.n_pair_types
            return {"dist": self.out["dist"].view(C, P), "mtv": self.out["mtv"].view(C, P, 3),
                    "contacts": self.contacts, "any": self.contacts.any(dim=1)}
