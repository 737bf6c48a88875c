// server.cu -- continuous-batching collision server (host runtime).
//
// Serves collision queries over one resident collider store: each request is
// a list of pairs answered with d3d_collide's outputs (GJK distance, then EPA
// on the intersecting pairs -- the reference's gjk() -> epa() composition,
// gjk/_gjk_jolt.py:138-221 and epa.py:9-78).  A worker thread owns `slots`
// batch slots, each with its own stream, device buffers, page-locked staging
// and (optionally) one CUDA graph of d3d_collide per capacity class.  The
// worker loops:
//
//   collect  a slot whose event has completed: scatter its rows back into
//            the requests they came from; a request whose pieces are all
//            back is finished (timestamped, waiters woken)
//   launch   a free slot takes pending request pieces in arrival order while
//            the batch stays within its capacity and the pairs of all
//            batches in flight within the memory budget (larger requests are
//            split over batches); copies in, replays the graph of the
//            smallest class that holds the batch, copies out, records an
//            event
//
// so requests that arrive while batches are on the GPU join the next batch
// as soon as a slot and memory are free, and the batches of different slots
// overlap on the device.  Latency is measured from a request's arrival
// (submission) to its last piece being back in host memory.
#include <pthread.h>
#include <sched.h>

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "capi_util.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kOutputs = 10;
// per-pair bytes of each output of d3d_collide, in the order of d3d_pair_results
constexpr size_t kOutBytes[kOutputs] = {8, 24, 24, 96, 1, 1, 4, 24, 1, 4};
constexpr size_t kPairBytes = 8 + 187 + 120;  // pair ids, outputs, scratch (approximate)

struct Request {
    int64_t id;
    std::vector<int32_t> i1, i2;
    std::vector<unsigned char> out[kOutputs];  // empty if the results are not kept
    Clock::time_point arrival, launched, finish;
    int pieces_out = 0;
    bool keep = true;
    bool started = false;
    bool done = false;
};

struct Piece {
    std::shared_ptr<Request> req;
    int64_t lo, hi, off;  // rows lo..hi of the request at batch row off
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    int32_t *i1 = nullptr, *i2 = nullptr;
    int64_t* n_dev = nullptr;
    void* out[kOutputs] = {};
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int32_t *h_i1 = nullptr, *h_i2 = nullptr;
    int64_t* h_n = nullptr;
    void* h_out[kOutputs] = {};
    std::vector<std::pair<int64_t, cudaGraphExec_t>> graphs;  // capacity class -> graph
    std::vector<Piece> pieces;
    int64_t n = 0;
    bool busy = false;
    Clock::time_point launched_at;
};

}  // namespace

struct d3d_server {
    d3d_store store;
    d3d_gjk_options gjk;
    d3d_epa_options epa;
    d3d_server_options opt;
    int device = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Piece> pending;
    std::unordered_map<int64_t, std::shared_ptr<Request>> requests;
    int64_t next_id = 1;
    int64_t inflight_pairs = 0;
    int64_t events = 0;  // arrivals and finished batches, counted to wake the worker
    d3d_server_stats stats = {};
    bool stop = false;
    int error = D3D_SUCCESS;
    char error_msg[256] = {};
    std::thread worker;
};

namespace {

int cuda_fail(d3d_server* s, cudaError_t e, const char* what) {
    std::snprintf(s->error_msg, sizeof(s->error_msg), "d3d_server: %s: %s", what, cudaGetErrorString(e));
    s->error = D3D_ERR_CUDA;
    return D3D_ERR_CUDA;
}

int collide(d3d_server* s, Slot& sl, int64_t cap) {
    return d3d_collide(&s->store, sl.i1, sl.i2, cap, sl.n_dev, &s->gjk, &s->epa, (double*)sl.out[0],
                       (double*)sl.out[1], (double*)sl.out[2], (double*)sl.out[3], (int8_t*)sl.out[4],
                       (int8_t*)sl.out[5], (int32_t*)sl.out[6], (double*)sl.out[7], (int8_t*)sl.out[8],
                       (int32_t*)sl.out[9], sl.scratch, sl.scratch_bytes, sl.stream);
}

void free_slot(Slot& sl) {
    for (auto& g : sl.graphs) cudaGraphExecDestroy(g.second);
    sl.graphs.clear();
    cudaFree(sl.i1);
    cudaFree(sl.i2);
    cudaFree(sl.n_dev);
    cudaFree(sl.scratch);
    for (int k = 0; k < kOutputs; ++k) {
        cudaFree(sl.out[k]);
        cudaFreeHost(sl.h_out[k]);
    }
    cudaFreeHost(sl.h_i1);
    cudaFreeHost(sl.h_i2);
    cudaFreeHost(sl.h_n);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
}

int init_slot(d3d_server* s, Slot& sl) {
    const int64_t cap = s->opt.capacity;
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&sl.i1, sizeof(int32_t) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&sl.i2, sizeof(int32_t) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&sl.n_dev, sizeof(int64_t));
    for (int k = 0; k < kOutputs && e == cudaSuccess; ++k) {
        e = cudaMalloc(&sl.out[k], kOutBytes[k] * cap);
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_out[k], kOutBytes[k] * cap);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_i1, sizeof(int32_t) * cap);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_i2, sizeof(int32_t) * cap);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_n, sizeof(int64_t));
    if (e == cudaSuccess) {
        sl.scratch_bytes = d3d_collide_scratch_bytes(cap, &s->gjk, &s->epa);
        e = cudaMalloc(&sl.scratch, sl.scratch_bytes);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.i1, 0, sizeof(int32_t) * cap, sl.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.i2, 0, sizeof(int32_t) * cap, sl.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.n_dev, 0, sizeof(int64_t), sl.stream);
    if (e != cudaSuccess) return cuda_fail(s, e, "slot allocation");
    if (!s->opt.use_graphs) return cudaStreamSynchronize(sl.stream) == cudaSuccess ? D3D_SUCCESS : D3D_ERR_CUDA;
    // capacity classes: 4096, 16384, 65536, ... below the capacity, and the capacity
    std::vector<int64_t> classes;
    for (int64_t c = 4096; c < cap; c *= 4) classes.push_back(c);
    classes.push_back(cap);
    for (int64_t c : classes) {
        int rc = collide(s, sl, c);  // eager first use (kernel attributes, module loading)
        if (rc) return rc;
        e = cudaStreamSynchronize(sl.stream);
        if (e != cudaSuccess) return cuda_fail(s, e, "warm-up");
        cudaGraph_t g = nullptr;
        cudaGraphExec_t x = nullptr;
        e = cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(s, e, "graph capture");
        rc = collide(s, sl, c);
        cudaError_t e2 = cudaStreamEndCapture(sl.stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e2 != cudaSuccess) return cuda_fail(s, e2, "graph capture");
        e = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(s, e, "graph instantiation");
        sl.graphs.emplace_back(c, x);
        // upload the executable graph and launch it once on an empty batch (the device count is
        // still 0): the first launch of a graph pays for its upload, which had stalled the first
        // batches of a new size class by tens of milliseconds
        e = cudaGraphUpload(x, sl.stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(x, sl.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
        if (e != cudaSuccess) return cuda_fail(s, e, "graph upload");
    }
    return D3D_SUCCESS;
}

// Scatter a finished slot's rows back into their requests (worker thread).
void collect(d3d_server* s, Slot& sl, Clock::time_point now) {
    for (const Piece& p : sl.pieces) {
        Request& r = *p.req;
        if (!r.keep) continue;
        const int64_t len = p.hi - p.lo;
        for (int k = 0; k < kOutputs; ++k)
            std::memcpy(r.out[k].data() + p.lo * kOutBytes[k],
                        static_cast<unsigned char*>(sl.h_out[k]) + p.off * kOutBytes[k], len * kOutBytes[k]);
    }
    std::lock_guard<std::mutex> lock(s->mu);
    const double batch_s = std::chrono::duration<double>(now - sl.launched_at).count();
    if (batch_s > s->stats.max_batch_s) s->stats.max_batch_s = batch_s;
    for (const Piece& p : sl.pieces) {
        Request& r = *p.req;
        if (--r.pieces_out == 0) {
            r.finish = now;
            r.done = true;
        }
    }
    s->inflight_pairs -= sl.n;
    sl.pieces.clear();
    sl.busy = false;
    s->cv_done.notify_all();
}

// Host function queued after a batch's copies: wakes the worker, which then
// finds the slot's event complete.  It runs on a thread of the CUDA runtime
// and calls no CUDA function.
void CUDART_CB batch_done(void* arg) {
    d3d_server* s = static_cast<d3d_server*>(arg);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        ++s->events;
    }
    s->cv_work.notify_one();
}

// Form and launch a batch on a free slot; false if nothing was pending.
bool launch(d3d_server* s, Slot& sl) {
    const int64_t cap = s->opt.capacity;
    int64_t n = 0;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        int64_t room = s->opt.hbm_budget / (int64_t)kPairBytes - s->inflight_pairs;
        if (room > cap) room = cap;
        while (!s->pending.empty() && n < room) {
            Piece& front = s->pending.front();
            const int64_t take = std::min(front.hi - front.lo, room - n);
            sl.pieces.push_back(Piece{front.req, front.lo, front.lo + take, n});
            n += take;
            if (front.lo + take == front.hi) {
                s->pending.pop_front();
            } else {
                front.lo += take;
                ++front.req->pieces_out;
            }
        }
        if (n == 0) return false;
        s->inflight_pairs += n;
        const Clock::time_point now = Clock::now();
        for (const Piece& p : sl.pieces)
            if (!p.req->started) {
                p.req->started = true;
                p.req->launched = now;
            }
    }
    for (const Piece& p : sl.pieces) {
        std::memcpy(sl.h_i1 + p.off, p.req->i1.data() + p.lo, sizeof(int32_t) * (p.hi - p.lo));
        std::memcpy(sl.h_i2 + p.off, p.req->i2.data() + p.lo, sizeof(int32_t) * (p.hi - p.lo));
    }
    *sl.h_n = n;
    sl.n = n;
    sl.busy = true;
    sl.launched_at = Clock::now();
    cudaError_t e = cudaMemcpyAsync(sl.i1, sl.h_i1, sizeof(int32_t) * n, cudaMemcpyHostToDevice, sl.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.i2, sl.h_i2, sizeof(int32_t) * n, cudaMemcpyHostToDevice, sl.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.n_dev, sl.h_n, sizeof(int64_t), cudaMemcpyHostToDevice, sl.stream);
    int rc = D3D_SUCCESS;
    if (e == cudaSuccess) {
        if (sl.graphs.empty()) {
            rc = collide(s, sl, cap);
        } else {
            cudaGraphExec_t x = sl.graphs.back().second;
            for (auto& g : sl.graphs)
                if (g.first >= n) {
                    x = g.second;
                    break;
                }
            e = cudaGraphLaunch(x, sl.stream);
        }
    }
    for (int k = 0; k < kOutputs && e == cudaSuccess && !rc; ++k)
        e = cudaMemcpyAsync(sl.h_out[k], sl.out[k], kOutBytes[k] * n, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess && !rc) e = cudaEventRecord(sl.done, sl.stream);
    if (e == cudaSuccess && !rc) e = cudaLaunchHostFunc(sl.stream, batch_done, s);
    {
        const double enqueue_s = std::chrono::duration<double>(Clock::now() - sl.launched_at).count();
        std::lock_guard<std::mutex> lock(s->mu);
        ++s->stats.batches;
        if (enqueue_s > s->stats.max_enqueue_s) s->stats.max_enqueue_s = enqueue_s;
    }
    if (e != cudaSuccess || rc) {
        std::lock_guard<std::mutex> lock(s->mu);
        if (rc) {
            std::snprintf(s->error_msg, sizeof(s->error_msg), "d3d_server: batch launch failed (code %d)", rc);
            s->error = rc;
        } else {
            cuda_fail(s, e, "batch launch");
        }
        s->cv_done.notify_all();
    }
    return true;
}

// The worker sleeps until a request arrives or a batch finishes (the host
// function above), rather than polling the slots' events: a polling thread
// holds a host core for itself, and on a host whose cores are shared or
// rationed that can cost whole milliseconds of latency when the scheduler
// takes the core away.
void worker_main(d3d_server* s) {
    cudaSetDevice(s->device);
    if (s->opt.worker_priority > 0) {
        sched_param sp = {};
        sp.sched_priority = s->opt.worker_priority;
        const bool rt = pthread_setschedparam(pthread_self(), SCHED_FIFO, &sp) == 0;
        std::lock_guard<std::mutex> lock(s->mu);
        s->stats.worker_realtime = rt ? 1 : 0;
    }
    int64_t seen = 0;
    while (true) {
        const Clock::time_point pass = Clock::now();
        {
            std::lock_guard<std::mutex> lock(s->mu);
            if (s->stop || s->error) break;
            seen = s->events;
        }
        bool did = false;
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaSuccess) {
                collect(s, sl, Clock::now());
                did = true;
            } else if (e != cudaErrorNotReady) {
                std::lock_guard<std::mutex> lock(s->mu);
                cuda_fail(s, e, "batch");
                s->cv_done.notify_all();
            }
        }
        for (Slot& sl : s->slots)
            if (!sl.busy && launch(s, sl)) did = true;
        {
            const double pass_s = std::chrono::duration<double>(Clock::now() - pass).count();
            std::lock_guard<std::mutex> lock(s->mu);
            if (pass_s > s->stats.max_loop_gap_s) s->stats.max_loop_gap_s = pass_s;
        }
        if (!did) {
            // nothing to collect or launch: wait for the next arrival or finished batch (a bounded
            // wait, so that a lost wake-up costs at most that long)
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_work.wait_for(lock, std::chrono::milliseconds(2),
                                [&] { return s->stop || s->error || s->events != seen; });
        }
    }
}

int server_error(d3d_server* s) {
    d3d::set_error("%s", s->error_msg);
    return s->error;
}

}  // namespace

extern "C" int d3d_server_create(const d3d_store* store, const d3d_gjk_options* gjk, const d3d_epa_options* epa,
                                 const d3d_server_options* options, d3d_server** out) {
    int rc = d3d::check_store(store, "d3d_server_create");
    if (rc) return rc;
    D3D_REQUIRE(gjk && epa && options && out, "d3d_server_create: null argument");
    D3D_REQUIRE(options->capacity > 0 && options->capacity <= INT32_MAX && options->slots >= 1 &&
                    options->slots <= 64 && options->hbm_budget >= 0 && options->worker_priority >= 0 &&
                    options->worker_priority <= 99,
                "d3d_server_create: invalid options (capacity 1..2^31-1, slots 1..64, budget >= 0, "
                "worker_priority 0..99)");
    D3D_REQUIRE(d3d_collide_scratch_bytes(options->capacity, gjk, epa) > 0, "d3d_server_create: invalid options");
    auto* s = new d3d_server();
    s->store = *store;
    s->gjk = *gjk;
    s->epa = *epa;
    s->opt = *options;
    if (s->opt.hbm_budget == 0) s->opt.hbm_budget = (int64_t)s->opt.slots * s->opt.capacity * (int64_t)kPairBytes;
    if (s->opt.hbm_budget < (int64_t)kPairBytes) s->opt.hbm_budget = kPairBytes;
    cudaGetDevice(&s->device);
    s->slots.resize(s->opt.slots);
    for (Slot& sl : s->slots) {
        rc = init_slot(s, sl);
        if (rc) break;
    }
    if (rc) {
        if (s->error) server_error(s);
        for (Slot& sl : s->slots) free_slot(sl);
        delete s;
        return rc;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return D3D_SUCCESS;
}

extern "C" void d3d_server_destroy(d3d_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    // the streams' last host functions (batch_done) refer to the server: wait for them too
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        free_slot(sl);
    }
    delete s;
}

namespace {

int submit(d3d_server* s, const int32_t* i1, const int32_t* i2, int64_t n, int64_t* id, bool keep) {
    D3D_REQUIRE(s && id && n >= 0 && (n == 0 || (i1 && i2)), "d3d_server_submit: invalid argument");
    auto r = std::make_shared<Request>();
    r->keep = keep;
    r->i1.assign(i1, i1 + n);
    r->i2.assign(i2, i2 + n);
    if (keep)
        for (int k = 0; k < kOutputs; ++k) r->out[k].resize(kOutBytes[k] * n);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->error) return server_error(s);
    for (int64_t k = 0; k < n; ++k)
        if (r->i1[k] < 0 || r->i1[k] >= s->store.n_colliders || r->i2[k] < 0 || r->i2[k] >= s->store.n_colliders) {
            d3d::set_error("d3d_server_submit: pair %lld refers to a collider outside the store", (long long)k);
            return D3D_ERR_INVALID;
        }
    r->id = s->next_id++;
    r->arrival = Clock::now();
    if (n == 0) {
        r->finish = r->arrival;
        r->done = true;
    } else {
        r->pieces_out = 1;
        s->pending.push_back(Piece{r, 0, n, 0});
    }
    s->requests[r->id] = r;
    *id = r->id;
    ++s->events;
    s->cv_work.notify_one();
    return D3D_SUCCESS;
}

}  // namespace

extern "C" int d3d_server_submit(d3d_server* s, const int32_t* i1, const int32_t* i2, int64_t n, int64_t* id) {
    return submit(s, i1, i2, n, id, true);
}

extern "C" int d3d_server_wait(d3d_server* s, int64_t id, double timeout_s) {
    D3D_REQUIRE(s, "d3d_server_wait: null server");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) {
        d3d::set_error("d3d_server_wait: unknown request %lld", (long long)id);
        return D3D_ERR_INVALID;
    }
    std::shared_ptr<Request> r = it->second;
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (!r->done && !s->error) {
        if (s->cv_done.wait_until(lock, until) == std::cv_status::timeout && !r->done) {
            d3d::set_error("d3d_server_wait: request %lld not finished after %.3f s", (long long)id, timeout_s);
            return D3D_ERR_CAPACITY;
        }
    }
    if (s->error) return server_error(s);
    return D3D_SUCCESS;
}

extern "C" int d3d_server_result(d3d_server* s, int64_t id, const d3d_pair_results* out, double* latency_s) {
    D3D_REQUIRE(s, "d3d_server_result: null server");
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->requests.find(id);
        if (it == s->requests.end()) {
            d3d::set_error("d3d_server_result: unknown request %lld", (long long)id);
            return D3D_ERR_INVALID;
        }
        if (!it->second->done) {
            d3d::set_error("d3d_server_result: request %lld not finished", (long long)id);
            return D3D_ERR_INVALID;
        }
        r = it->second;
        s->requests.erase(it);
    }
    if (latency_s) *latency_s = std::chrono::duration<double>(r->finish - r->arrival).count();
    if (out && r->keep) {
        void* dst[kOutputs] = {out->dist, out->cp1, out->cp2, out->simplex, out->n_simplex,
                               out->status, out->iterations, out->mtv, out->epa_status, out->n_faces};
        for (int k = 0; k < kOutputs; ++k)
            if (dst[k]) std::memcpy(dst[k], r->out[k].data(), r->out[k].size());
    }
    return D3D_SUCCESS;
}

extern "C" int d3d_server_stats_read(d3d_server* s, d3d_server_stats* out, int reset) {
    D3D_REQUIRE(s && out, "d3d_server_stats_read: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    if (reset) {
        const int32_t rt = s->stats.worker_realtime;
        s->stats = d3d_server_stats{};
        s->stats.worker_realtime = rt;
    }
    return D3D_SUCCESS;
}

extern "C" int d3d_server_replay(d3d_server* s, int64_t n_requests, const double* offsets_s, const int64_t* sizes,
                                 const int32_t* i1, const int32_t* i2, double* latency_s, double* wait_s,
                                 double* span_s) {
    D3D_REQUIRE(s && n_requests >= 0 && (n_requests == 0 || (offsets_s && sizes && i1 && i2 && latency_s)),
                "d3d_server_replay: invalid argument");
    std::vector<int64_t> ids(n_requests);
    const auto t0 = Clock::now();
    int64_t base = 0;
    for (int64_t k = 0; k < n_requests; ++k) {
        const auto at = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(offsets_s[k]));
        // sleep to just before the arrival, then spin the last stretch for timing accuracy
        const auto wake = at - std::chrono::microseconds(200);
        if (Clock::now() < wake) std::this_thread::sleep_until(wake);
        while (Clock::now() < at) {
        }
        int rc = submit(s, i1 + base, i2 + base, sizes[k], &ids[k], false);
        if (rc) return rc;
        {
            // latency counts from the scheduled arrival, so a late submission is not hidden
            std::lock_guard<std::mutex> lock(s->mu);
            auto& r = s->requests[ids[k]];
            if (r->arrival > at) r->arrival = at;
        }
        base += sizes[k];
    }
    Clock::time_point last = t0;
    for (int64_t k = 0; k < n_requests; ++k) {
        int rc = d3d_server_wait(s, ids[k], 600.0);
        if (rc) return rc;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            const Request& r = *s->requests[ids[k]];
            if (r.finish > last) last = r.finish;
            if (wait_s) wait_s[k] = std::chrono::duration<double>((r.started ? r.launched : r.finish) - r.arrival).count();
        }
        rc = d3d_server_result(s, ids[k], nullptr, &latency_s[k]);
        if (rc) return rc;
    }
    if (span_s) *span_s = std::chrono::duration<double>(last - t0).count();
    return D3D_SUCCESS;
}
