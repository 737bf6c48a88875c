"""Batched GJK + EPA with the pair count on the device, CUDA graphs, and a
continuous-batching collision server.

* ``CollisionBatch`` runs ``d3d_collide`` (GJK distance, then EPA on the
  pairs GJK finds intersecting with a full simplex -- the reference's
  ``gjk()`` -> ``epa(simplex)`` composition, gjk/_gjk_jolt.py:138-221 and
  epa.py:9-78) on preallocated buffers.  Because the count lives on the
  device and every launch shape depends on the capacity only, one call per
  capacity class is captured as a CUDA graph and replayed for any batch that
  fits.
* ``CollisionServer`` serves collision queries (requests of 1 to 50,000
  pairs over one resident collider store) by continuous batching: requests
  that arrive while batches are on the GPU are admitted into the next batch
  as soon as a batch slot and its device memory are free, several batches are
  in flight on separate streams, and each request's latency is measured
  from its arrival to its results being in host memory.
"""
import ctypes
import time
from collections import deque

import numpy as np
import torch

from . import _lib
from .store import _ptr

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}

# per-pair outputs: name, dtype, trailing shape
_OUTPUTS = (("dist", torch.float64, ()), ("cp1", torch.float64, (3,)), ("cp2", torch.float64, (3,)),
            ("simplex", torch.float64, (4, 3)), ("n_simplex", torch.int8, ()), ("status", torch.int8, ()),
            ("iterations", torch.int32, ()), ("mtv", torch.float64, (3,)), ("epa_status", torch.int8, ()),
            ("n_faces", torch.int32, ()))

# bytes of device memory one pair slot holds (inputs, outputs, GJK scratch)
PAIR_BYTES = 8 + sum(torch.tensor([], dtype=d).element_size() * int(np.prod(s)) for _, d, s in _OUTPUTS) + 120


class CollisionBatch:
    """GJK + EPA on up to ``capacity`` pairs of ``store`` per call.

    ``precision`` applies to both GJK and EPA ("mixed" or "fp64"); ``epa_kw``
    sets max_iter / max_loose_edges / max_faces / epsilon as ``epa.epa``.
    With ``graphs=True`` each capacity class (``classes``, ascending, the
    last one equal to ``capacity``) is captured once as a CUDA graph; a call
    replays the smallest class that holds its pairs.
    """

    def __init__(self, store, capacity, *, precision="mixed", epa_kw=None, gjk_kw=None, graphs=True,
                 classes=None):
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
        self.store = store
        self.capacity = int(capacity)
        self.device = store.device
        ek = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
        ek.update(epa_kw or {})
        gk = dict(tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8, max_iterations=1024)
        gk.update(gjk_kw or {})
        self._gjk = _lib.GjkOptions(gk["tolerance"], gk["max_distance_squared"], gk["sanity_check"],
                                    int(gk["max_iterations"]), _PRECISIONS[precision])
        self._epa = _lib.EpaOptions(int(ek["max_iter"]), int(ek["max_loose_edges"]), int(ek["max_faces"]),
                                    _PRECISIONS[precision], float(ek["epsilon"]))
        self.classes = sorted(set(classes or [c for c in (4096, 16384, 65536) if c < self.capacity] +
                                  [self.capacity]))
        if self.classes[-1] != self.capacity:
            raise ValueError("the largest capacity class must equal capacity")
        lib = _lib.load()
        dev, cap = self.device, self.capacity
        with torch.cuda.device(dev):
            self.stream = torch.cuda.Stream(dev)
            self.i1 = torch.zeros(cap, dtype=torch.int32, device=dev)
            self.i2 = torch.zeros(cap, dtype=torch.int32, device=dev)
            self.n_dev = torch.zeros(1, dtype=torch.int64, device=dev)
            self.out = {k: torch.empty((cap,) + s, dtype=d, device=dev) for k, d, s in _OUTPUTS}
            nbytes = max(int(lib.d3d_collide_scratch_bytes(c, ctypes.byref(self._gjk), ctypes.byref(self._epa)))
                         for c in self.classes)
            self.scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            pin = dict(pin_memory=True)
            self.h_i1 = torch.zeros(cap, dtype=torch.int32, **pin)
            self.h_i2 = torch.zeros(cap, dtype=torch.int32, **pin)
            self.h_n = torch.zeros(1, dtype=torch.int64, **pin)
            self.h_out = {k: torch.empty((cap,) + s, dtype=d, **pin) for k, d, s in _OUTPUTS}
            self.done = torch.cuda.Event()
            self.graphs = {}
            if graphs:
                for c in self.classes:
                    # one eager call (first-use work such as kernel attributes), then the capture
                    with torch.cuda.stream(self.stream):
                        self._launch(c)
                    self.stream.synchronize()
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=self.stream):
                        self._launch(c)
                    self.graphs[c] = g
                self.stream.synchronize()
        self.n = 0

    def _launch(self, cap):
        o = self.out
        _lib.check(_lib.load().d3d_collide(
            self.store.view, _ptr(self.i1), _ptr(self.i2), cap, _ptr(self.n_dev), ctypes.byref(self._gjk),
            ctypes.byref(self._epa), _ptr(o["dist"]), _ptr(o["cp1"]), _ptr(o["cp2"]), _ptr(o["simplex"]),
            _ptr(o["n_simplex"]), _ptr(o["status"]), _ptr(o["iterations"]), _ptr(o["mtv"]), _ptr(o["epa_status"]),
            _ptr(o["n_faces"]), _ptr(self.scratch), self.scratch.numel(),
            ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def submit(self, i1, i2):
        """Start one batch: pairs (i1[k], i2[k]) from host arrays.  Copies in,
        runs and copies the results out on this batch's stream; ``ready()``
        and ``results()`` follow it."""
        n = len(i1)
        if n > self.capacity:
            raise ValueError(f"{n} pairs exceed the capacity {self.capacity}")
        # the previous batch's copies read and write the same page-locked buffers
        self.done.synchronize()
        self.n = n
        self.h_i1.numpy()[:n] = i1
        self.h_i2.numpy()[:n] = i2
        self.h_n.numpy()[0] = n
        with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
            if n:
                self.i1[:n].copy_(self.h_i1[:n], non_blocking=True)
                self.i2[:n].copy_(self.h_i2[:n], non_blocking=True)
            self.n_dev.copy_(self.h_n, non_blocking=True)
            cls = next(c for c in self.classes if c >= n)
            if self.graphs:
                self.graphs[cls].replay()
            else:
                self._launch(cls)
            for k in self.out:
                if n:
                    self.h_out[k][:n].copy_(self.out[k][:n], non_blocking=True)
            self.done.record(self.stream)

    def ready(self):
        return self.done.query()

    def results(self, lo=0, hi=None):
        """Host (NumPy) views of pairs lo..hi of the last batch (after ready())."""
        self.done.synchronize()
        hi = self.n if hi is None else hi
        return {k: v[lo:hi].numpy() for k, v in self.h_out.items()}

    def run(self, i1, i2):
        """Synchronous convenience: submit and return copies of the results."""
        self.submit(np.asarray(i1), np.asarray(i2))
        return {k: v.copy() for k, v in self.results().items()}


class Request:
    __slots__ = ("rid", "i1", "i2", "arrival", "admitted", "finished", "result")

    def __init__(self, rid, i1, i2, arrival):
        self.rid, self.i1, self.i2, self.arrival = rid, i1, i2, arrival
        self.admitted = self.finished = None
        self.result = None


class CollisionServer:
    """Continuous batching over ``slots`` CollisionBatch objects (each with
    its own stream and preallocated device memory).

    Admission: a request joins the batch being formed while the batch's
    pairs stay within its capacity and the device memory of all batches in
    flight stays within ``hbm_budget`` bytes; larger requests are split into
    pieces that ride consecutive batches.  A batch is launched as soon as a
    slot is free; requests arriving meanwhile wait for the next free slot,
    so batches overlap on the GPU.  Results are delivered per request when
    all its pieces are back in host memory.
    """

    def __init__(self, store, *, capacity=65536, slots=2, precision="mixed", epa_kw=None, graphs=True,
                 hbm_budget=None, batches=None):
        self.batches = batches if batches is not None else [
            CollisionBatch(store, capacity, precision=precision, epa_kw=epa_kw, graphs=graphs) for _ in range(slots)]
        self.capacity = capacity
        self.hbm_budget = hbm_budget if hbm_budget is not None else len(self.batches) * capacity * PAIR_BYTES
        self.pending = deque()   # (request, start, stop) pieces not yet in a batch
        self.inflight = []       # (batch, [(request, start, stop, offset), ...])
        self.remaining = {}      # request -> pieces still out

    def _form(self, batch):
        pieces, n = [], 0
        in_flight = sum(b.n for b, _ in self.inflight) * PAIR_BYTES
        room = min(self.capacity, max(0, (self.hbm_budget - in_flight) // PAIR_BYTES))
        while self.pending and n < room:
            req, lo, hi = self.pending[0]
            take = min(hi - lo, room - n)
            pieces.append((req, lo, lo + take, n))
            n += take
            if lo + take == hi:
                self.pending.popleft()
            else:
                self.pending[0] = (req, lo + take, hi)
                self.remaining[req] += 1
        if not pieces:
            return False
        i1 = np.concatenate([r.i1[lo:hi] for r, lo, hi, _ in pieces])
        i2 = np.concatenate([r.i2[lo:hi] for r, lo, hi, _ in pieces])
        now = time.perf_counter()
        for r, _, _, _ in pieces:
            if r.admitted is None:
                r.admitted = now
        batch.submit(i1, i2)
        self.inflight.append((batch, pieces))
        return True

    def _collect(self):
        done = []
        for entry in self.inflight:
            batch, pieces = entry
            if not batch.ready():
                continue
            out = batch.results()
            now = time.perf_counter()
            for r, lo, hi, off in pieces:
                part = {k: v[off:off + hi - lo].copy() for k, v in out.items()}
                if r.result is None:
                    r.result = {k: np.empty((len(r.i1),) + v.shape[1:], v.dtype) for k, v in part.items()}
                for k, v in part.items():
                    r.result[k][lo:hi] = v
                self.remaining[r] -= 1
                if self.remaining[r] == 0:
                    r.finished = now
                    del self.remaining[r]
            done.append(entry)
        for entry in done:
            self.inflight.remove(entry)

    def admit(self, req):
        self.pending.append((req, 0, len(req.i1)))
        self.remaining[req] = 1

    def step(self):
        """One turn of the loop: collect finished batches, launch a new one on
        a free slot.  Returns True if anything happened."""
        before = len(self.inflight)
        self._collect()
        busy = {id(b) for b, _ in self.inflight}
        launched = False
        for b in self.batches:
            if id(b) not in busy and self.pending:
                launched = self._form(b) or launched
                busy.add(id(b))
        return launched or len(self.inflight) != before

    def idle(self):
        return not self.pending and not self.inflight

    def serve(self, requests, arrivals):
        """Replay ``requests`` at wall-clock offsets ``arrivals`` (seconds from
        now, ascending) and run until all are answered.  Returns the
        requests with ``arrival``, ``admitted`` and ``finished`` set."""
        t0 = time.perf_counter()
        order = np.argsort(arrivals, kind="stable")
        k = 0
        while k < len(order) or not self.idle():
            now = time.perf_counter() - t0
            while k < len(order) and arrivals[order[k]] <= now:
                r = requests[order[k]]
                r.arrival = t0 + arrivals[order[k]]
                self.admit(r)
                k += 1
            self.step()
        return requests


def latency_stats(requests):
    lat = np.array([r.finished - r.arrival for r in requests])
    pairs = sum(len(r.i1) for r in requests)
    span = max(r.finished for r in requests) - min(r.arrival for r in requests)
    return dict(p50_ms=float(np.percentile(lat, 50) * 1e3), p99_ms=float(np.percentile(lat, 99) * 1e3),
                max_ms=float(lat.max() * 1e3), pairs_per_s=pairs / span, requests=len(requests))


def request_sizes(rng, n, median=2000, sigma=1.0, lo=1, hi=50000):
    """Pairs per request: lognormal with the given median, clipped to [lo, hi]."""
    return np.clip(np.round(rng.lognormal(np.log(median), sigma, n)), lo, hi).astype(np.int64)


class NativeCollisionServer:
    """The C++ continuous-batching server (``d3d_server_*``): the same
    admission and batching as ``CollisionServer``, run by a worker thread in
    the library with one CUDA graph per capacity class and slot.  ``submit``
    copies a request's host pairs and returns its id; ``result`` waits for it
    and returns host arrays plus its latency; ``replay`` submits a whole
    arrival trace from the library (so the arrival times are kept to the
    microsecond) and returns the per-request latencies.  ``worker_priority``
    > 0 asks for the worker thread under SCHED_FIFO at that priority (kept at
    the default policy where the process may not raise it; ``stats()`` says
    which)."""

    def __init__(self, store, *, capacity=65536, slots=2, precision="mixed", epa_kw=None, gjk_kw=None, graphs=True,
                 hbm_budget=0, worker_priority=0):
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
        ek = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
        ek.update(epa_kw or {})
        gk = dict(tolerance=1e-10, max_distance_squared=100000.0, sanity_check=1e-8, max_iterations=1024)
        gk.update(gjk_kw or {})
        self._gjk = _lib.GjkOptions(gk["tolerance"], gk["max_distance_squared"], gk["sanity_check"],
                                    int(gk["max_iterations"]), _PRECISIONS[precision])
        self._epa = _lib.EpaOptions(int(ek["max_iter"]), int(ek["max_loose_edges"]), int(ek["max_faces"]),
                                    _PRECISIONS[precision], float(ek["epsilon"]))
        self.store = store  # the server reads the store's device buffers
        self._lib = _lib.load()
        opt = _lib.ServerOptions(int(capacity), int(slots), 1 if graphs else 0, int(hbm_budget),
                                 int(worker_priority), 0)
        handle = ctypes.c_void_p()
        with torch.cuda.device(store.device):
            torch.cuda.synchronize(store.device)
            _lib.check(self._lib.d3d_server_create(store.view, ctypes.byref(self._gjk), ctypes.byref(self._epa),
                                                   ctypes.byref(opt), ctypes.byref(handle)))
        self._h = handle

    def close(self):
        if self._h:
            self._lib.d3d_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, i1, i2):
        a = np.ascontiguousarray(i1, dtype=np.int32)
        b = np.ascontiguousarray(i2, dtype=np.int32)
        rid = ctypes.c_int64()
        _lib.check(self._lib.d3d_server_submit(self._h, a.ctypes.data, b.ctypes.data, len(a), ctypes.byref(rid)))
        return rid.value, len(a)

    def result(self, ticket, timeout=60.0):
        rid, n = ticket
        _lib.check(self._lib.d3d_server_wait(self._h, rid, float(timeout)))
        out = {k: np.empty((n,) + tuple(s), dtype=torch.empty((), dtype=d).numpy().dtype) for k, d, s in _OUTPUTS}
        pr = _lib.PairResults(*[out[k].ctypes.data for k, _, _ in _OUTPUTS])
        lat = ctypes.c_double()
        _lib.check(self._lib.d3d_server_result(self._h, rid, ctypes.byref(pr), ctypes.byref(lat)))
        return out, lat.value

    def replay(self, sizes, i1, i2, offsets):
        """Requests of sizes[k] pairs (concatenated in i1/i2) arriving at
        offsets[k] seconds; returns (latencies in seconds, span in seconds)."""
        sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        offs = np.ascontiguousarray(offsets, dtype=np.float64)
        a = np.ascontiguousarray(i1, dtype=np.int32)
        b = np.ascontiguousarray(i2, dtype=np.int32)
        if a.size != sizes.sum() or b.size != a.size or offs.size != sizes.size:
            raise ValueError("sizes, offsets and pair arrays disagree")
        lat = np.empty(len(sizes))
        wait = np.empty(len(sizes))
        span = ctypes.c_double()
        _lib.check(self._lib.d3d_server_replay(self._h, len(sizes), offs.ctypes.data, sizes.ctypes.data,
                                               a.ctypes.data, b.ctypes.data, lat.ctypes.data, wait.ctypes.data,
                                               ctypes.byref(span)))
        self.last_wait = wait
        return lat, span.value

    def stats(self, reset=True):
        """The worker's counters since the last reset (d3d_server_stats_read):
        batches, and the longest batch (launch to results in host memory), the
        longest enqueue of one batch and the longest pass of the worker loop,
        in milliseconds."""
        st = _lib.ServerStats()
        _lib.check(self._lib.d3d_server_stats_read(self._h, ctypes.byref(st), 1 if reset else 0))
        return {"batches": st.batches, "max_batch_ms": 1e3 * st.max_batch_s,
                "max_enqueue_ms": 1e3 * st.max_enqueue_s, "max_loop_pass_ms": 1e3 * st.max_loop_gap_s,
                "worker_realtime": bool(st.worker_realtime)}
