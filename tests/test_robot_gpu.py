"""Batched self-collision checks: device forward kinematics against the NumPy
chain, the FP64 form's distances bit for bit against the oracle on the posed
bodies, the mixed form within tolerance with the same contacts, graph and
eager identical, and the contact flags as self_collision.detect defines them."""
import numpy as np
import pytest

from distance3d_gb300.robot import SelfCollisionBatch, SerialArm
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def arm():
    return SerialArm.synthetic(seed=4)


def test_fk_matches_numpy_chain(arm):
    rng = np.random.default_rng(0)
    q = rng.uniform(-np.pi, np.pi, (64, arm.dof))
    b = SelfCollisionBatch(arm, 64, precision="fp64", graph=False)
    b.run(q)
    got = b.poses.cpu().numpy().reshape(64, arm.n_bodies, 12)
    want = np.stack([arm.fk(qq) for qq in q])
    assert np.max(np.abs(got - want)) < 1e-12


@pytest.mark.parametrize("graph", [False, True])
def test_self_collision_forms(arm, graph):
    rng = np.random.default_rng(1)
    C = 512
    q = rng.uniform(-np.pi, np.pi, (C, arm.dof))
    f = SelfCollisionBatch(arm, C, precision="fp64", graph=graph)
    rf = {k: v.cpu().numpy() for k, v in f.run(q).items()}
    # the FP64 form is the reference's GJK on the posed bodies
    poses = f.poses.cpu().numpy()
    from distance3d_gb300.collider_set import ColliderSet
    n = C * arm.n_bodies
    posed = ColliderSet(np.tile(arm.body_type, C), poses, np.tile(arm.body_params, (C, 1)),
                        np.full(n, -1, dtype=np.int64), np.zeros(n, dtype=np.int32), np.zeros((0, 4)))
    ref = oracle.gjk_distance(posed, f.i1.cpu().numpy(), f.i2.cpu().numpy())
    assert np.array_equal(rf["dist"].reshape(-1), ref["dist"])
    # contacts: a body is in contact iff one of its listed pairs intersects
    table = arm.pair_table()
    hit = rf["dist"] == 0.0
    want = np.zeros((C, arm.n_bodies), dtype=bool)
    for p, (a, b) in enumerate(table):
        want[:, a] |= hit[:, p]
        want[:, b] |= hit[:, p]
    assert np.array_equal(rf["contacts"], want) and want.any() and not want.all()
    assert np.array_equal(rf["any"], want.any(axis=1))
    m = SelfCollisionBatch(arm, C, precision="mixed", graph=graph)
    rm = {k: v.cpu().numpy() for k, v in m.run(q).items()}
    df, dm = rf["dist"].reshape(-1), rm["dist"].reshape(-1)
    assert np.max(np.abs(dm - df) / np.maximum(1.0, df)) < 1e-5
    sep = df > 1e-6
    assert np.array_equal(dm[sep] > 0, df[sep] > 0)


def test_graph_equals_eager(arm):
    rng = np.random.default_rng(2)
    q = rng.uniform(-np.pi, np.pi, (256, arm.dof))
    a = SelfCollisionBatch(arm, 256, precision="mixed", graph=True)
    b = SelfCollisionBatch(arm, 256, precision="mixed", graph=False)
    for _ in range(2):
        ra, rb = a.run(q), b.run(q)
        for k in ra:
            assert np.array_equal(ra[k].cpu().numpy(), rb[k].cpu().numpy(), equal_nan=True), k
        q = rng.uniform(-np.pi, np.pi, (256, arm.dof))
