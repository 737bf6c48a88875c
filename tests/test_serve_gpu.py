"""The device-count batch (d3d_collide), its CUDA graphs and the
continuous-batching server: same results as the separate calls, graph and
eager identical, and every request's result identical alone and in the mix."""
import numpy as np
import pytest

from distance3d_gb300 import workloads
from distance3d_gb300.epa import epa_batch
from distance3d_gb300.gjk import gjk_distance_batch
from distance3d_gb300.serve import CollisionBatch, CollisionServer, Request, request_sizes
from distance3d_gb300.store import ColliderStore
from oracle import oracle

pytestmark = pytest.mark.gpu

EPA_KW = dict(max_iter=64, max_loose_edges=128, max_faces=256, epsilon=1e-8)


def host(r):
    return {k: v.cpu().numpy() for k, v in r.items()}


@pytest.fixture(scope="module")
def scene():
    cs, i1, i2 = workloads.pairs_mixed_six(60000, seed=41, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    return cs, ColliderStore(cs), np.asarray(i1), np.asarray(i2)


def separate_calls(st, i1, i2, precision):
    g = host(gjk_distance_batch(st, i1, i2, precision=precision))
    hit = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    e = host(epa_batch(st, i1[hit], i2[hit], g["simplex"][hit], precision=precision, **EPA_KW))
    return g, hit, e


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_collide_equals_separate_calls(scene, precision):
    cs, st, i1, i2 = scene
    n = 20000
    b = CollisionBatch(st, 32768, precision=precision, epa_kw=EPA_KW, graphs=True)
    r = b.run(i1[:n], i2[:n])
    g, hit, e = separate_calls(st, i1[:n], i2[:n], precision)
    for k in ("dist", "cp1", "cp2", "simplex", "n_simplex", "status", "iterations"):
        assert np.array_equal(r[k], g[k], equal_nan=True), k
    assert np.array_equal(r["epa_status"][hit], e["status"])
    assert np.array_equal(r["mtv"][hit], e["mtv"], equal_nan=True)
    assert np.array_equal(r["n_faces"][hit], e["n_faces"])
    rest = np.setdiff1d(np.arange(n), hit)
    assert np.all(r["epa_status"][rest] == -1) and np.all(np.isnan(r["mtv"][rest]))
    if precision == "fp64":
        ref = oracle.gjk_distance(cs, i1[:n], i2[:n])
        assert np.array_equal(r["dist"], ref["dist"]) and np.array_equal(r["simplex"], ref["simplex"])


def test_graph_and_eager_identical_every_size(scene):
    _, st, i1, i2 = scene
    gb = CollisionBatch(st, 16384, precision="mixed", epa_kw=EPA_KW, graphs=True, classes=[1024, 16384])
    eb = CollisionBatch(st, 16384, precision="mixed", epa_kw=EPA_KW, graphs=False, classes=[1024, 16384])
    for n in (0, 1, 7, 1024, 1025, 9000, 16384):
        a, b = gb.run(i1[:n], i2[:n]), eb.run(i1[:n], i2[:n])
        for k in a:
            assert np.array_equal(a[k], b[k], equal_nan=True), (n, k)


def test_results_same_alone_and_in_the_mix(scene):
    _, st, i1, i2 = scene
    rng = np.random.default_rng(5)
    sizes = list(request_sizes(rng, 24)) + [1, 70000 % 60000, 45000]
    reqs, alone = [], []
    ref = CollisionBatch(st, 65536, precision="mixed", epa_kw=EPA_KW, graphs=False)
    for k, m in enumerate(sizes):
        sel = rng.integers(0, len(i1), int(m))
        reqs.append(Request(k, i1[sel].astype(np.int32), i2[sel].astype(np.int32), 0.0))
        alone.append(ref.run(i1[sel], i2[sel]))
    # small capacity: big requests are split over batches, batches overlap
    srv = CollisionServer(st, capacity=16384, slots=3, precision="mixed", epa_kw=EPA_KW)
    arrivals = np.sort(rng.uniform(0.0, 0.02, len(reqs)))
    srv.serve(reqs, arrivals)
    for r, a in zip(reqs, alone):
        assert r.finished is not None and r.finished >= r.arrival
        for k in a:
            assert np.array_equal(r.result[k], a[k], equal_nan=True), (r.rid, k)




def test_native_server_same_alone_and_in_the_mix(scene):
    from distance3d_gb300.serve import NativeCollisionServer
    _, st, i1, i2 = scene
    rng = np.random.default_rng(9)
    sizes = [int(m) for m in request_sizes(rng, 30)] + [1, 40000, 0]
    ref = CollisionBatch(st, 65536, precision="mixed", epa_kw=EPA_KW, graphs=False)
    srv = NativeCollisionServer(st, capacity=16384, slots=3, precision="mixed", epa_kw=EPA_KW)
    try:
        sels = [rng.integers(0, len(i1), m) for m in sizes]
        tickets = [srv.submit(i1[s], i2[s]) for s in sels]
        for s, t in zip(sels, tickets):
            out, lat = srv.result(t)
            alone = ref.run(i1[s], i2[s])
            assert lat >= 0.0
            for k in alone:
                assert np.array_equal(out[k], alone[k], equal_nan=True), (len(s), k)
        # replayed arrival trace: every request answered, latencies positive
        sz = request_sizes(rng, 50)
        sel = rng.integers(0, len(i1), int(sz.sum()))
        lat, span = srv.replay(sz, i1[sel], i2[sel], np.sort(rng.uniform(0, 0.05, len(sz))))
        assert np.all(lat > 0) and span > 0
    finally:
        srv.close()


def test_native_server_worker_priority(scene):
    """A worker asking for SCHED_FIFO answers as the default one; whether the
    process was allowed to raise it is reported, and out-of-range priorities
    are rejected."""
    from distance3d_gb300 import _lib
    from distance3d_gb300.serve import NativeCollisionServer
    _, st, i1, i2 = scene
    ref = CollisionBatch(st, 4096, precision="mixed", epa_kw=EPA_KW, graphs=False)
    srv = NativeCollisionServer(st, capacity=4096, slots=2, precision="mixed", epa_kw=EPA_KW, worker_priority=1)
    try:
        out, _ = srv.result(srv.submit(i1[:500], i2[:500]))
        alone = ref.run(i1[:500], i2[:500])
        for k in alone:
            assert np.array_equal(out[k], alone[k], equal_nan=True), k
        stats = srv.stats(reset=True)
        assert isinstance(stats["worker_realtime"], bool)
        assert srv.stats(reset=False)["worker_realtime"] == stats["worker_realtime"]  # survives a reset
    finally:
        srv.close()
    with pytest.raises(_lib.D3DError):
        NativeCollisionServer(st, capacity=4096, slots=1, precision="mixed", epa_kw=EPA_KW, worker_priority=100)


def test_native_server_rejects_bad_pairs(scene):
    from distance3d_gb300 import _lib
    from distance3d_gb300.serve import NativeCollisionServer
    _, st, i1, i2 = scene
    srv = NativeCollisionServer(st, capacity=4096, slots=1, precision="mixed", epa_kw=EPA_KW, graphs=False)
    try:
        with pytest.raises(_lib.D3DError):
            srv.submit([0, len(st)], [1, 2])
        out, _ = srv.result(srv.submit(i1[:10], i2[:10]))
        assert out["dist"].shape == (10,)
    finally:
        srv.close()


def test_store_update_keeps_graphs_valid():
    """ColliderStore.update packs new colliders of the same shape into the
    same device buffers: a CollisionBatch captured before the update gives
    what a fresh store gives for the new colliders."""
    from distance3d_gb300.store import PinnedColliderSet
    from distance3d_gb300.collider_set import ColliderSet
    a_cs, i1, i2 = workloads.pairs_mixed_six(5000, seed=61, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    # the second colliders of every pair moved by 0.05 along x: same shape, new distances
    poses, verts = a_cs.poses.copy(), a_cs.vertices.copy()
    poses[1::2, 9] += 0.05
    moved = np.zeros(len(verts), bool)
    for c in range(1, len(a_cs), 2):
        if a_cs.hull_offset[c] >= 0 and a_cs.types[c] == 5:
            moved[a_cs.hull_offset[c]:a_cs.hull_offset[c] + a_cs.hull_count[c]] = True
    verts[moved, 0] += 0.05
    b_cs = ColliderSet(a_cs.types, poses, a_cs.params, a_cs.hull_offset, a_cs.hull_count, verts)
    st = ColliderStore(PinnedColliderSet(a_cs))
    batch = CollisionBatch(st, 5000, precision="mixed", epa_kw=EPA_KW, graphs=True)
    ra = batch.run(i1, i2)
    st.update(PinnedColliderSet(b_cs))
    rb = batch.run(i1, i2)
    want = CollisionBatch(ColliderStore(b_cs), 5000, precision="mixed", epa_kw=EPA_KW, graphs=False).run(i1, i2)
    for k in ("dist", "simplex", "mtv", "epa_status"):
        assert np.array_equal(rb[k], want[k], equal_nan=True), k
    assert not np.array_equal(ra["dist"], rb["dist"])
    with pytest.raises(ValueError):
        st.update(PinnedColliderSet(workloads.pairs_mixed_six(100, seed=63)[0]))
