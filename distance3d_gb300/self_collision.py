"""Self-collision detection with distance3d's call surface
(self_collision.py:5-64).

``detect(bvh)`` and ``detect_any(bvh)`` take a ``BoundingVolumeHierarchy``
of this package whose ``self_collision_whitelists_`` maps every collider
frame to the frames it may touch (the collider's own frame and its
neighbours), as the reference requires.  The reference queries the tree once
per collider and runs one GJK intersection test after another; here the
candidate pairs of every collider come from one self-overlap query of the
GPU tree and the GJK intersection tests of all candidate pairs run as one
batch on the GPU (FP64, the reference's results).  The reference's control
flow -- colliders in insertion order, candidates in leaf order, the first
intersecting candidate marking both frames, frames already marked skipped --
is then replayed on these flags, so the result is the reference's for the
same candidate order.

For many joint configurations at once, ``distance3d_gb300.robot`` runs
forward kinematics, pose updates and the narrow phase of a whole batch on the
device.
"""
import numpy as np

from .collider_set import ColliderSet
from .gjk import gjk_intersection_batch
from .store import ColliderStore


def _candidates(bvh):
    """(frames, colliders, candidate lists of leaf indices, flag lookup)."""
    bvh._flush()
    tree = bvh.aabbtree_
    ext = tree.external_data_list
    frames = [f for f, _ in ext]
    leaf = {f: k for k, f in enumerate(frames)}
    _, _, _, pairs = tree.overlaps_aabb_tree(tree)
    cand = [[] for _ in frames]
    for i, j in pairs:
        cand[i].append(j)
    order = [leaf[f] for f in bvh.colliders_]
    lists = {}
    todo = []
    for i in order:
        white = bvh.self_collision_whitelists_[frames[i]]
        c = [j for j in cand[i] if frames[j] not in white]
        lists[i] = c
        todo.extend((i, j) for j in c)
    hit = {}
    if todo:
        cs = ColliderSet.from_colliders([c for _, c in ext])
        p = np.asarray(todo, dtype=np.int32)
        flags = gjk_intersection_batch(ColliderStore(cs, device=bvh.device), p[:, 0], p[:, 1])["hit"].cpu().numpy()
        hit = {(int(a), int(b)): bool(h) for (a, b), h in zip(todo, flags)}
    return frames, order, lists, hit


def detect(bvh):
    """Frame -> whether the collider is in contact with another
    (self_collision.py:5-36)."""
    frames, order, lists, hit = _candidates(bvh)
    contacts = {}
    for i in order:
        if frames[i] in contacts:
            continue
        contacts[frames[i]] = False
        for j in lists[i]:
            if hit[(i, j)]:
                contacts[frames[i]] = True
                contacts[frames[j]] = True
                break
    return contacts


def detect_any(bvh):
    """Whether any collider is in contact with another
    (self_collision.py:39-64)."""
    frames, order, lists, hit = _candidates(bvh)
    return any(hit[(i, j)] for i in order for j in lists[i])
