"""Host logic of the continuous-batching server, on a fake batch (no GPU):
admission within capacity and memory budget, splitting of large requests,
batches in flight at once, every pair answered exactly once and in place."""
import numpy as np

from distance3d_gb300.serve import PAIR_BYTES, CollisionServer, Request, latency_stats, request_sizes


class FakeBatch:
    """Answers pair k with (i1 + 1000 * i2) after `delay` polls."""

    def __init__(self, capacity, delay=2):
        self.capacity, self.delay, self.n, self.polls, self.launched = capacity, delay, 0, 0, []

    def submit(self, i1, i2):
        assert len(i1) <= self.capacity
        self.n = len(i1)
        self.polls = 0
        self.out = {"dist": (np.asarray(i1) + 1000.0 * np.asarray(i2)), "status": np.zeros(len(i1), np.int8)}
        self.launched.append(len(i1))

    def ready(self):
        self.polls += 1
        return self.polls > self.delay

    def results(self):
        return self.out


def make_requests(sizes, rng):
    return [Request(k, rng.integers(0, 900, m).astype(np.int32), rng.integers(0, 900, m).astype(np.int32), 0.0)
            for k, m in enumerate(sizes)]


def test_every_pair_answered_in_place_with_splitting():
    rng = np.random.default_rng(0)
    reqs = make_requests([5, 3000, 1, 12000, 700, 4096, 9000], rng)
    fakes = [FakeBatch(4096, delay=5) for _ in range(3)]
    srv = CollisionServer(None, capacity=4096, batches=fakes)
    srv.serve(reqs, np.zeros(len(reqs)))
    for r in reqs:
        assert np.array_equal(r.result["dist"], r.i1 + 1000.0 * r.i2)
        assert r.finished >= r.admitted >= r.arrival
    launched = sum(sum(f.launched) for f in fakes)
    assert launched == sum(len(r.i1) for r in reqs)
    assert max(max(f.launched) for f in fakes) <= 4096
    assert all(f.launched for f in fakes)  # every slot was used: batches overlapped


def test_memory_budget_limits_pairs_in_flight():
    rng = np.random.default_rng(1)
    reqs = make_requests([3000] * 6, rng)
    fakes = [FakeBatch(4096, delay=5) for _ in range(3)]
    budget = 5000 * PAIR_BYTES
    srv = CollisionServer(None, capacity=4096, batches=fakes, hbm_budget=budget)
    for r in reqs:
        srv.admit(r)
    peak = 0
    while not srv.idle():
        srv.step()
        peak = max(peak, sum(b.n for b, _ in srv.inflight))
    assert peak <= 5000
    for r in reqs:
        assert np.array_equal(r.result["dist"], r.i1 + 1000.0 * r.i2)


def test_request_sizes_and_stats():
    s = request_sizes(np.random.default_rng(0), 100000)
    assert s.min() >= 1 and s.max() <= 50000
    assert 1800 < np.median(s) < 2200
    r = Request(0, np.zeros(10, np.int32), np.zeros(10, np.int32), 1.0)
    r.finished = 1.002
    st = latency_stats([r])
    assert abs(st["p50_ms"] - 2.0) < 1e-6 and st["requests"] == 1
