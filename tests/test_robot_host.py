"""Synthetic arm and its self-collision pair table (no GPU)."""
import numpy as np

from distance3d_gb300.robot import SerialArm


def test_pair_table_whitelist():
    arm = SerialArm.synthetic(seed=4)
    t = arm.pair_table()
    assert np.all(np.abs(arm.body_link[t[:, 0]] - arm.body_link[t[:, 1]]) > 1)
    assert np.all(t[:, 0] < t[:, 1])
    all_pairs = arm.n_bodies * (arm.n_bodies - 1) // 2
    adjacent = sum(1 for a in range(arm.n_bodies) for b in range(a + 1, arm.n_bodies)
                   if abs(arm.body_link[a] - arm.body_link[b]) <= 1)
    assert len(t) == all_pairs - adjacent


def test_fk_chain_properties():
    arm = SerialArm.synthetic(seed=4)
    p = arm.fk(np.zeros(arm.dof))
    R = p[:, :9].reshape(-1, 3, 3)
    assert np.allclose(R @ R.transpose(0, 2, 1), np.eye(3), atol=1e-12)
    # a base body does not move with the joints
    q = np.random.default_rng(0).uniform(-np.pi, np.pi, arm.dof)
    base = arm.body_link == 0
    assert np.allclose(arm.fk(q)[base], p[base])
