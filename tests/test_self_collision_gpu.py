"""self_collision.detect / detect_any on the GPU tree and GJK against the
reference's control flow replayed on oracle flags (brute-force candidate
lists, the oracle's GJK intersection)."""
import numpy as np
import pytest

from distance3d_gb300 import colliders, self_collision
from distance3d_gb300.broad_phase import BoundingVolumeHierarchy
from distance3d_gb300.collider_set import BOX, CAPSULE
from distance3d_gb300.robot import SerialArm
from oracle import oracle

pytestmark = pytest.mark.gpu


class FakeTM:
    def __init__(self):
        self.T = {}

    def add_transform(self, a, b, A2B):
        self.T[(a, b)] = A2B

    def get_transform(self, a, b):
        return self.T[(a, b)]


def body_collider(t, p, pose):
    if t == CAPSULE:
        return colliders.Capsule(pose, p[0], p[1])
    if t == BOX:
        return colliders.Box(pose, p[:3].copy())
    return colliders.Cylinder(pose, p[0], p[1])


def arm_bvh(arm, q):
    tm = FakeTM()
    bvh = BoundingVolumeHierarchy(tm, "base")
    poses = arm.fk(q)
    for b in range(arm.n_bodies):
        pose = np.eye(4)
        pose[:3, :3] = poses[b, :9].reshape(3, 3)
        pose[:3, 3] = poses[b, 9:]
        frame = f"body{b}"
        tm.add_transform(frame, "origin", pose)
        bvh.add_collider(frame, body_collider(arm.body_type[b], arm.body_params[b], pose))
    for b in range(arm.n_bodies):
        near = np.flatnonzero(np.abs(arm.body_link - arm.body_link[b]) <= 1)
        bvh.self_collision_whitelists_[f"body{b}"] = [f"body{k}" for k in near]
    return bvh


def oracle_detect(bvh):
    """The reference's detect / detect_any (self_collision.py:5-64) with
    brute-force candidates in leaf order and the oracle's GJK."""
    from distance3d_gb300.collider_set import ColliderSet
    frames = list(bvh.colliders_)
    cols = list(bvh.colliders_.values())
    cs = ColliderSet.from_colliders(cols)
    boxes = oracle.aabbs(cs)
    pairs = oracle.self_pairs(boxes)
    cand = [[] for _ in frames]
    for i, j in pairs:
        cand[i].append(j)
        cand[j].append(i)
    for i in range(len(frames)):
        cand[i] = sorted(cand[i] + [i])
    contacts, any_hit = {}, False
    for i, f in enumerate(frames):
        white = bvh.self_collision_whitelists_[f]
        c = [j for j in cand[i] if frames[j] not in white]
        flags = oracle.gjk_intersection(cs, np.full(len(c), i), np.array(c, dtype=np.int32))["hit"] if c else []
        any_hit = any_hit or bool(np.any(flags))
        if f in contacts:
            continue
        contacts[f] = False
        for j, h in zip(c, flags):
            if h:
                contacts[f] = True
                contacts[frames[j]] = True
                break
    return contacts, any_hit


def test_detect_matches_reference_control_flow():
    arm = SerialArm.synthetic(seed=3)
    rng = np.random.default_rng(4)
    seen_hit = seen_free = False
    for _ in range(12):
        q = rng.uniform(-np.pi, np.pi, arm.dof)
        bvh = arm_bvh(arm, q)
        want, want_any = oracle_detect(bvh)
        got = self_collision.detect(bvh)
        assert got == want
        assert self_collision.detect_any(bvh) == want_any
        seen_hit |= want_any
        seen_free |= not want_any
    assert seen_hit


def test_detect_after_pose_update_and_missing_whitelist():
    arm = SerialArm.synthetic(seed=5)
    bvh = arm_bvh(arm, np.zeros(arm.dof))
    q = np.full(arm.dof, 0.7)
    poses = arm.fk(q)
    for b in range(arm.n_bodies):
        pose = np.eye(4)
        pose[:3, :3] = poses[b, :9].reshape(3, 3)
        pose[:3, 3] = poses[b, 9:]
        bvh.tm.add_transform(f"body{b}", "origin", pose)
    bvh.update_collider_poses()
    want, want_any = oracle_detect(bvh)
    assert self_collision.detect(bvh) == want
    assert self_collision.detect_any(bvh) == want_any
    del bvh.self_collision_whitelists_["body0"]
    with pytest.raises(KeyError):
        self_collision.detect(bvh)
