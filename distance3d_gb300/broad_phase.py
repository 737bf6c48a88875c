"""Bounding volume hierarchy with distance3d's interface (broad_phase.py).

``BoundingVolumeHierarchy(tm, base_frame, base_frame2origin)`` keeps a
frame -> collider map and an ``AabbTree`` of the colliders' boxes.  Boxes are
computed on the GPU in one batch (containment.py formulas, exact FP64) and the
tree is the GPU LBVH.  ``tm`` is any object with ``add_transform(a, b, A2B)``
and ``get_transform(a, b)`` (pytransform3d's TransformManager has both).
Building colliders from URDF files (``fill_tree_with_colliders``,
broad_phase.py:53-127) is not provided.
"""
import numpy as np

from .aabb_tree import AabbTree
from .collider_set import ColliderSet


def collider_aabbs(colliders, device="cuda"):
    """(n,3,2) FP64 boxes of collider objects, computed on the GPU."""
    from .store import ColliderStore
    if len(colliders) == 0:
        return np.empty((0, 3, 2))
    return ColliderStore(ColliderSet.from_colliders(list(colliders)), device=device).aabbs().cpu().numpy()


class BoundingVolumeHierarchy:
    """Broad-phase BVH over colliders connected by transformations."""

    def __init__(self, tm, base_frame, base_frame2origin=np.eye(4), device="cuda"):
        tm.add_transform(base_frame, "origin", base_frame2origin)
        self.tm = tm
        self.base_frame = base_frame
        self.base_frame2origin = base_frame2origin
        self.device = device
        self.collider_frames = set()
        self.aabbtree_ = AabbTree(device=device)
        self.colliders_ = {}
        self.self_collision_whitelists_ = {}
        self._pending = []

    def fill_tree_with_colliders(self, tm, make_artists=False, fill_self_collision_whitelists=False,
                                 use_visuals=False):
        raise NotImplementedError("URDF loading is not part of distance3d_gb300")

    def add_collider(self, frame, collider):
        """Add a collider (broad_phase.py:129-142)."""
        self.collider_frames.add(frame)
        self.colliders_[frame] = collider
        self._pending.append((frame, collider))

    def _flush(self):
        if self._pending:
            boxes = collider_aabbs([c for _, c in self._pending], self.device)
            self.aabbtree_.insert_aabbs(boxes, list(self._pending))
            self._pending = []

    def update_collider_poses(self):
        """Read every collider's pose from ``tm`` (broad_phase.py:144-151).
        The reference rebuilds its tree; here the boxes are recomputed on
        the GPU and the tree is refit when its leaves are the same colliders
        (same pair sets, no rebuild)."""
        self._flush()
        for frame, collider in self.colliders_.items():
            collider.update_pose(self.tm.get_transform(frame, "origin"))
        leaves = [c for _, c in self.aabbtree_.external_data_list]
        if len(leaves) == len(self.colliders_) and all(a is b for a, b in zip(leaves, self.colliders_.values())):
            self.aabbtree_.update_aabbs(collider_aabbs(leaves, self.device))
            return
        self.aabbtree_ = AabbTree(device=self.device)
        self._pending = list(self.colliders_.items())
        self._flush()

    def get_colliders(self):
        return self.colliders_.values()

    def get_artists(self):
        return [c.artist_ for c in self.colliders_.values() if getattr(c, "artist_", None) is not None]

    def get_collider_frames(self):
        return self.collider_frames

    def aabb_overlapping_colliders(self, collider, whitelist=()):
        """frame -> collider for every collider whose box overlaps
        ``collider``'s (broad_phase.py:174-200)."""
        self._flush()
        box = collider_aabbs([collider], self.device)[0]
        _, overlaps = self.aabbtree_.overlaps_aabb(box)
        colliders = dict(self.aabbtree_.external_data_list[i] for i in overlaps)
        for frame in whitelist:
            colliders.pop(frame, None)
        return colliders

    def aabb_overlapping_with_other_bvh(self, other_bvh):
        """[((frame, collider), (frame, collider)), ...] across two BVHs
        (broad_phase.py:202-227)."""
        self._flush()
        other_bvh._flush()
        _, _, _, pairs = self.aabbtree_.overlaps_aabb_tree(other_bvh.aabbtree_)
        return [(self.aabbtree_.external_data_list[i], other_bvh.aabbtree_.external_data_list[j])
                for i, j in pairs]

    def aabb_overlapping_with_self(self):
        """Both orders of every overlapping pair, i == j dropped
        (broad_phase.py:229-252)."""
        self._flush()
        _, _, _, pairs = self.aabbtree_.overlaps_aabb_tree(self.aabbtree_)
        ext = self.aabbtree_.external_data_list
        return [(ext[i], ext[j]) for i, j in pairs if i != j]
