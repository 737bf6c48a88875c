"""EPA on the GPU (through the C ABI) against the golden vectors and the
oracle: status, MTV, face count and faces bit for bit."""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.collider_set import BOX, HULL
from distance3d_gb300.epa import epa_batch, epa_scratch_bytes
from distance3d_gb300.gjk import gjk_distance_batch
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu


def host(r):
    return {k: v.cpu().numpy() for k, v in r.items()}


@pytest.mark.parametrize("tag,kw", [("default", {}), ("large", dict(max_faces=256, max_loose_edges=128)),
                                    ("tight", dict(max_iter=20, max_faces=24, max_loose_edges=6)),
                                    ("short", dict(max_iter=6, max_faces=256, max_loose_edges=128)),
                                    ("edges", dict(max_faces=256, max_loose_edges=4)),
                                    ("eps", dict(max_faces=256, max_loose_edges=128, epsilon=1e-4))])
def test_epa_matches_reference_golden(golden, tag, kw):
    g, cs = golden("gjk_mixed6")
    e, _ = golden("epa_mixed6")
    p = e["pair"]
    r = host(epa_batch(ColliderStore(cs), g["i1"][p], g["i2"][p], g["simplex"][p], **kw))
    st = e[f"status_{tag}"]
    assert np.array_equal(r["status"], st)
    ok = (st == 0) | (st == 4)  # converged, or the closest face's MTV at the iteration bound
    assert np.array_equal(r["mtv"][ok], e[f"mtv_{tag}"][ok])
    assert np.array_equal(r["n_faces"][ok], e[f"n_faces_{tag}"][ok])


@pytest.mark.parametrize("max_faces,max_edges", [(64, 32), (256, 128)])
def test_epa_matches_oracle_with_faces(max_faces, max_edges):
    cs, i1, i2 = workloads.pairs_mixed_six(6000, seed=31, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero(g["dist"] == 0.0)
    assert len(hit) > 1000
    kw = dict(max_faces=max_faces, max_loose_edges=max_edges)
    r = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], return_faces=True, **kw))
    ref = oracle.epa(cs, i1[hit], i2[hit], g["simplex"][hit], want_faces=True, **kw)
    assert np.array_equal(r["status"], ref["status"])
    assert np.array_equal(r["n_faces"], ref["n_faces"])
    assert np.array_equal(r["mtv"], ref["mtv"], equal_nan=True)
    for k in range(len(hit)):
        nf = r["n_faces"][k]
        assert np.array_equal(r["faces"][k, :nf], ref["faces"][k, :nf])


@pytest.mark.parametrize("max_faces,max_edges", [(100, 40), (64, 128), (256, 128)])
def test_epa_polytope_sizes(max_faces, max_edges):
    """Polytope storage of other sizes than the defaults (the face and edge
    limits bind on different pairs) on the nine-type workload, against the
    oracle bit for bit."""
    cs, i1, i2 = workloads.pairs_all_types(6000, seed=33)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    kw = dict(max_faces=max_faces, max_loose_edges=max_edges)
    r = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], return_faces=True, **kw))
    ref = oracle.epa(cs, i1[hit], i2[hit], g["simplex"][hit], want_faces=True, **kw)
    assert np.array_equal(r["status"], ref["status"])
    assert np.array_equal(r["n_faces"], ref["n_faces"])
    assert np.array_equal(r["mtv"], ref["mtv"], equal_nan=True)
    for k in range(len(hit)):
        nf = r["n_faces"][k]
        assert np.array_equal(r["faces"][k, :nf], ref["faces"][k, :nf])
    if max_faces > 64:
        assert (ref["n_faces"] > 64).sum() > 10


@pytest.mark.parametrize("kw,with_faces", [(dict(max_iter=300, max_faces=256, max_loose_edges=128), True),
                                           (dict(max_faces=4096, max_loose_edges=512), False)])
def test_epa_beyond_warp_form(kw, with_faces):
    """Options the one-warp-per-pair kernel does not take (more than 251
    iterations: vertex ids beyond 8 bits; a polytope beyond the shared memory
    of a block) run in the thread-per-pair kernel, bit for bit the oracle's."""
    cs, i1, i2 = workloads.pairs_all_types(3000, seed=35)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    r = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], return_faces=with_faces, **kw))
    ref = oracle.epa(cs, i1[hit], i2[hit], g["simplex"][hit], want_faces=with_faces, **kw)
    assert np.array_equal(r["status"], ref["status"])
    assert np.array_equal(r["n_faces"], ref["n_faces"])
    assert np.array_equal(r["mtv"], ref["mtv"], equal_nan=True)
    if with_faces:
        for k in range(len(hit)):
            nf = r["n_faces"][k]
            assert np.array_equal(r["faces"][k, :nf], ref["faces"][k, :nf])


def test_epa_many_pairs_reuse_slots():
    """More pairs than scratch slots: every pair still gets its own answer."""
    cs, i1, i2 = workloads.pairs_mixed_six(200000, seed=32, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero(g["dist"] == 0.0)
    assert len(hit) > 40000
    r = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], max_faces=256, max_loose_edges=128))
    sample = np.random.default_rng(1).choice(len(hit), 3000, replace=False)
    ref = oracle.epa(cs, i1[hit][sample], i2[hit][sample], g["simplex"][hit][sample], max_faces=256,
                     max_loose_edges=128)
    assert np.array_equal(r["status"][sample], ref["status"])
    assert np.array_equal(r["mtv"][sample], ref["mtv"], equal_nan=True)
    assert epa_scratch_bytes(len(hit), max_faces=256, max_loose_edges=128) < 64 * len(hit) * 12 * 256 * 8


def test_epa_edge_cases():
    cs, i1, i2 = workloads.pairs_mixed_six(16, seed=2)
    st = ColliderStore(cs)
    r = epa_batch(st, [], [], np.zeros((0, 4, 3)))
    assert r["mtv"].shape == (0, 3)
    # zero iterations: the initial closest face, not converged
    s = np.random.default_rng(0).normal(size=(4, 4, 3))
    r = host(epa_batch(st, i1[:4], i2[:4], s, max_iter=0))
    ref = oracle.epa(cs, i1[:4], i2[:4], s, max_iter=0)
    assert np.array_equal(r["status"], ref["status"])
    assert np.array_equal(r["mtv"], ref["mtv"], equal_nan=True)
    # a degenerate (flat) simplex: whatever the reference does, the same status
    flat = np.zeros((4, 4, 3))
    flat[:, :, :2] = np.random.default_rng(1).normal(size=(4, 4, 2))
    r = host(epa_batch(st, i1[:4], i2[:4], flat))
    ref = oracle.epa(cs, i1[:4], i2[:4], flat)
    assert np.array_equal(r["status"], ref["status"])
    assert np.array_equal(r["mtv"], ref["mtv"], equal_nan=True)


def test_drop_in_epa():
    from distance3d_gb300 import colliders, epa, gjk
    from tests.test_known_answers import EPA_V1, EPA_V2
    c1, c2 = colliders.ConvexHullVertices(EPA_V1), colliders.ConvexHullVertices(EPA_V2)
    d, _, _, simplex = gjk.gjk(c1, c2)
    assert d == 0.0
    mtv, faces, success = epa.epa(simplex, c1, c2)
    assert success
    assert faces.shape[1:] == (4, 3)
    np.testing.assert_array_almost_equal(mtv, [-0.387287, 0.179576, -0.176204])


MIXED_DEPTH_TOL = 1e-5  # |depth_mixed - depth_fp64| / max(1, depth_fp64)


def check_mixed_depths(cs, i1, i2, m, ref):
    """Mixed EPA depths against the FP64 reference.

    Both forms return h(n) = n . (s1(n) - s2(-n)) for their final normal n,
    an upper bound on the true penetration depth for every n.  The mixed depth
    must never exceed the reference's by more than the tolerance; where the
    reference's exceeds the mixed one, h(n_mixed) -- recomputed here with the
    oracle's exact supports -- proves that the reference's depth is not the
    minimum (the reference's EPA keeps degenerate faces after its
    orientation fix, epa.py:139-146, and can stop on a wrong face)."""
    both = (m["status"] == 0) & (ref["status"] == 0)
    dm = np.linalg.norm(m["mtv"][both], axis=1)
    dr = np.linalg.norm(ref["mtv"][both], axis=1)
    tol = MIXED_DEPTH_TOL * np.maximum(1.0, dr)
    assert np.all(dm <= dr + tol), f"mixed deeper than the reference by {np.max(dm - dr)}"
    wrong = dr > dm + tol
    if wrong.any():
        n = m["mtv"][both][wrong] / dm[wrong, None]
        h = oracle.depth_upper_bound(cs, i1[both][wrong], i2[both][wrong], n)
        assert np.all(np.abs(h - dm[wrong]) <= 1e-7 * np.maximum(1.0, dm[wrong]))
        assert np.all(h < dr[wrong] - tol[wrong])
    assert wrong.mean() < 2e-3
    return both, wrong


@pytest.mark.parametrize("max_faces,max_edges", [(64, 32), (256, 128)])
def test_mixed_epa_within_tolerance(max_faces, max_edges):
    cs, i1, i2 = workloads.pairs_mixed_six(30000, seed=33, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero(g["dist"] == 0.0)
    kw = dict(max_faces=max_faces, max_loose_edges=max_edges)
    m = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], precision="mixed", **kw))
    ref = oracle.epa(cs, i1[hit], i2[hit], g["simplex"][hit], **kw)
    # exact topology (vertex ids) keeps the mixed search converging about as often
    assert (m["status"] == 0).sum() >= 0.99 * (ref["status"] == 0).sum()
    both, wrong = check_mixed_depths(cs, i1[hit], i2[hit], m, ref)
    assert both.sum() > 0.9 * (ref["status"] == 0).sum()
    dm = np.linalg.norm(m["mtv"][both], axis=1)
    dr = np.linalg.norm(ref["mtv"][both], axis=1)
    cosang = np.sum(m["mtv"][both] * ref["mtv"][both], axis=1) / np.maximum(dm * dr, 1e-300)
    # Polytope pairs (box, hull): the final face of the Minkowski difference
    # is the same face, so the directions agree to rounding.
    t1, t2 = cs.types[i1[hit][both]], cs.types[i2[hit][both]]
    poly = np.isin(t1, [BOX, HULL]) & np.isin(t2, [BOX, HULL]) & ~wrong & (dr > 1e-3)
    assert poly.sum() > 100
    assert np.all(cosang[poly] > 1 - 1e-9)
    # Curved pairs: the depth is flat in the direction near its minimum, and
    # both forms stop on a polytope face whose normal is within ~1e-3 rad of
    # the optimum.  The mixed direction is certified instead: the exact
    # support-function depth along it (the oracle's supports) equals the
    # reported depth and is within the tolerance of the reference's depth.
    n = m["mtv"][both] / dm[:, None]
    h = oracle.depth_upper_bound(cs, i1[hit][both], i2[hit][both], n)
    assert np.all(np.abs(h - dm) <= 1e-7 * np.maximum(1.0, dm))
    assert np.all(h <= dr + MIXED_DEPTH_TOL * np.maximum(1.0, dr))


def test_mixed_epa_status_agreement_and_the_pairs_it_settles():
    """Status agreement of the mixed EPA with the FP64 oracle at the bench's
    limits (256 faces, 128 loose edges, 64 iterations) on ~17k EPA pairs, and
    which answer is right where they differ.  The mixed search converges on
    pairs the reference leaves unconverged at the iteration bound (its
    face-winding defect, epa.py:142-146, slows its convergence); run with
    larger limits (2,000 iterations, 8,192 faces, 2,048 loose edges), the
    reference converges on most of them to the depth the mixed form reports,
    within the mixed form's tolerance."""
    cs, i1, i2 = workloads.pairs_mixed_six(60000, seed=77, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    g = host(gjk_distance_batch(st, i1, i2))
    hit = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    a, b, s = i1[hit], i2[hit], g["simplex"][hit]
    kw = dict(max_iter=64, max_loose_edges=128, max_faces=256, epsilon=1e-8)
    m = host(epa_batch(st, a, b, s, precision="mixed", **kw))
    f = oracle.epa(cs, a, b, s, **kw)
    assert len(hit) > 15000
    assert np.mean(m["status"] == f["status"]) > 0.95
    mo, fo = m["status"] == 0, f["status"] == 0
    assert mo.sum() > fo.sum()
    # the reference converges where the mixed form does not on a few pairs only
    assert (fo & ~mo).sum() < 0.005 * len(hit)
    sel = np.flatnonzero(mo & ~fo)
    big = oracle.epa(cs, a[sel], b[sel], s[sel], max_iter=2000, max_loose_edges=2048, max_faces=8192, epsilon=1e-8)
    ok = big["status"] == 0
    assert ok.mean() > 0.75
    dm = np.linalg.norm(m["mtv"][sel][ok], axis=1)
    dl = np.linalg.norm(big["mtv"][ok], axis=1)
    assert np.all(np.abs(dm - dl) <= MIXED_DEPTH_TOL * np.maximum(1.0, dl))
