// gjk_mixed.cu -- mixed-precision GJK distance.
//
// Four kernels over the type-sorted pair order:
//
// A  runs the Jolt loop in FP32 on the FP32 mirror of the store, with
//    thresholds scaled to single precision, hands each pair's outcome, final
//    closest point and the search direction of each final simplex row to B
//    (80 bytes/pair) and appends clipped and unconverged pairs to the
//    fallback list.
// B  walks the same type-sorted order (lanes of a warp then mostly hold
//    pairs of the same collider types) and refines A's separated and
//    touching pairs in FP64, one round per lane and iteration (pb_round): A's
//    final simplex rows are re-evaluated in FP64 along their FP32 directions,
//    all in the first round (polytope supports choose their vertex by an FP32
//    argmax and return the FP64 vertex); if that simplex encloses or touches
//    the origin the pair is done, otherwise the reference's loop continues
//    from it until the duality gap brackets the distance within 1e-6 of
//    itself or 1e-9 of the scene's scale.  A pair whose loop ends leaves its
//    simplex in the outputs and the rest of its state in an end record.
// E  (the end pass) computes the closest points and the checks of B's
//    finished pairs (pb_end), every lane on a finished pair.
// C  is the plain FP64 kernel over the fallback list (the reference's
//    arithmetic; CLIPPED and MAX_ITER keep their FP64 meaning).
//
// B keeps the simplex P/Q rows in shared memory and has one support call
// site, so that a warp's lanes share the support and simplex code whatever
// mode and simplex size each holds.  A pair goes to the fallback list only if
// its result fails the consistency check (closest points vs |v|) or the
// sanity check in E, or hits the iteration bound in B.
//
// On the six-type workloads A takes ~11 FP32 iterations and B replays ~3
// rows and runs ~2 FP64 iterations, against ~17-19 FP64 iterations for the
// plain form.  Compiled with -fmad=true: the tests bound its error against
// the FP64 oracle.
#include "capi_util.h"
#include "gjk_impl.h"
#include "gjk_mixed.cuh"
#include "gjk_out.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;


// Per-call counters (one 256-byte block): cursors of A, B and C, then the
// lengths of the fallback and finished lists.
enum { kCurA = 0, kCurB, kCurC, kNumFallback, kNumEnd, kCounters };

// B's state of a pair whose loop has ended, for the end pass (the simplex's
// Y rows and row count go to the outputs directly).
struct alignas(16) EndRecord {
    double pq[4][6];  // P and Q rows below n
    double dir[3];
    double vl;
    int it;  // A's and B's iterations
    int state;
    int status;
    int n;
};

struct Lists {
    int32_t* fallback;
    int32_t* ends;         // pairs whose FP64 loop ended in B, for the end pass
    EndRecord* records;    // their state, by pair
    unsigned long long* ctr;
};

// slots a warp claims from the type-sorted order at a time
constexpr int kChunk = 32;

// Phase A's register budget: at least 12 resident warps per SM (16 for
// 256-thread blocks), which ptxas would otherwise trade for a few more
// registers per thread.
template <int BLOCK>
constexpr int phase_a_min_blocks() { return BLOCK == 256 ? 2 : 384 / BLOCK; }

template <int BLOCK, bool MESH>
__global__ void __launch_bounds__(BLOCK, phase_a_min_blocks<BLOCK>()) k_gjk_mixed_a(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        const int64_t* __restrict__ n_dev, float tol_sq,
                                                        float max_d2, int max_iter, Handoff* __restrict__ hand,
                                                        DistanceOut out, Lists lists) {
    if (n_dev) n = *n_dev;
    PhaseALoop L;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true, bad = false;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // per-lane claims for the last slots: the pairs are short, and slots left in a busy warp's chunk
    // would hold up the end of the launch
    const long long split = n - 2LL * gridDim.x * blockDim.x;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(lists.ctr + kCurA, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            bad = !pair_ok(s, a, b);
            pa_begin(L);
            need = false;
        }
        // a pair with an out-of-range index ends at once; B skips it (its outcome is neither
        // separated nor touching) and it joins no list
        const int o = bad ? PA_BAD_INDEX : pa_step<MESH>(L, s, a, b, tol_sq, max_d2, max_iter);
        const bool done = o >= 0;
        if (done) {
            hand[pid] = pa_handoff(L, o);
            if (bad) store_bad_index(out, pid);
        }
        append_lanes(live, lists.fallback, lists.ctr + kNumFallback, done && (o == PA_CLIPPED || o == PA_FAILED),
                     (int32_t)pid);
        need = done;
    }
}

template <int BLOCK, bool MESH>
__global__ void __launch_bounds__(BLOCK) k_gjk_mixed_b(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        const int64_t* __restrict__ n_dev, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o, Lists lists) {
    __shared__ double rows[24 * BLOCK];
    if (n_dev) n = *n_dev;
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    PhaseB<SmemRows<double, BLOCK>> B;
    B.g.S.R.base = rows + threadIdx.x;
    int32_t pid = 0;
    int a = 0, b = 0;
    int it_a = 0;
    bool need = true;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // per-lane claims for the last slots: the pairs are short, and slots left in a busy warp's chunk
    // would hold up the end of the launch
    const long long split = n - 2LL * gridDim.x * blockDim.x;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(lists.ctr + kCurB, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            // the pairs in the collider-type order, A's separated and touching ones
            pid = order ? order[slot] : (int32_t)slot;
            const float4 v = hand[pid].v;
            const int outcome = __float_as_int(v.w) & 0xff;
            if (outcome != PA_SEPARATED && outcome != PA_TOUCHING) continue;
            a = i1[pid];
            b = i2[pid];
            it_a = handoff_iters(v);
            pb_begin(B, v);
            need = false;
        }
        if (B.mode == PB_FALLBACK || pb_round<MESH>(B, s, a, b, hand[pid].d, tol_sq, opt, E)) {
            if (B.mode != PB_FALLBACK) {
                // The closest points and checks of the pair (pb_end) run in
                // the end pass, where a warp's lanes all hold finished pairs;
                // here only a few lanes finish per round.
                const GjkLoop<double, SmemRows<double, BLOCK>>& g = B.g;
                EndRecord& e = lists.records[pid];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < g.S.n) {
                        const d3 pk = g.S.R.p(k), qk = g.S.R.q(k);
                        e.pq[k][0] = pk.x;
                        e.pq[k][1] = pk.y;
                        e.pq[k][2] = pk.z;
                        e.pq[k][3] = qk.x;
                        e.pq[k][4] = qk.y;
                        e.pq[k][5] = qk.z;
                    }
                }
                e.dir[0] = g.dir.x;
                e.dir[1] = g.dir.y;
                e.dir[2] = g.dir.z;
                e.vl = g.vl;
                e.it = g.it + it_a;
                e.state = g.state;
                e.status = g.status;
                e.n = g.S.n;
                double* sp = o.simplex + 12 * (int64_t)pid;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    sp[3 * j] = g.S.Y[j].x;
                    sp[3 * j + 1] = g.S.Y[j].y;
                    sp[3 * j + 2] = g.S.Y[j].z;
                }
                o.n_simplex[pid] = (int8_t)g.S.n;
                append_warp(lists.ends, lists.ctr + kNumEnd, true, pid);
            } else {
                lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
            }
            need = true;
        }
    }
}

// The end pass over B's finished pairs: closest points, sanity and
// consistency checks (pb_end) and the outputs; pairs failing a check go to
// the fallback list.
__global__ void __launch_bounds__(128) k_gjk_mixed_end(d3d_gjk_options opt, DistanceOut o, Lists lists) {
    const int64_t n = (int64_t)lists.ctr[kNumEnd];
    const JoltEps<double> E = reference_eps<double>();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t pid = lists.ends[k];
        const EndRecord& e = lists.records[pid];
        GjkLoop<double, RegRows<double>> g;
        g.S.n = e.n;
        const double* sp = o.simplex + 12 * (int64_t)pid;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            g.S.Y[j] = mk(sp[3 * j], sp[3 * j + 1], sp[3 * j + 2]);
            if (j < e.n)
                g.S.R.put(j, mk(e.pq[j][0], e.pq[j][1], e.pq[j][2]), mk(e.pq[j][3], e.pq[j][4], e.pq[j][5]));
        }
        g.dir = mk(e.dir[0], e.dir[1], e.dir[2]);
        g.vl = e.vl;
        g.prev = 0.0;
        g.it = e.it;
        g.state = e.state;
        g.status = e.status;
        GjkResult<double> r;
        if (pb_end(g, opt, E, r) == PB_DONE) {
            o.dist[pid] = r.dist;
            o.cp1[3 * (int64_t)pid] = r.a.x;
            o.cp1[3 * (int64_t)pid + 1] = r.a.y;
            o.cp1[3 * (int64_t)pid + 2] = r.a.z;
            o.cp2[3 * (int64_t)pid] = r.b.x;
            o.cp2[3 * (int64_t)pid + 1] = r.b.y;
            o.cp2[3 * (int64_t)pid + 2] = r.b.z;
            o.status[pid] = (int8_t)r.status;
            if (o.iterations) o.iterations[pid] = r.iters;
        } else {
            lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
        }
    }
}

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

namespace d3d {

size_t gjk_mixed_scratch_bytes(int64_t capacity) {
    return 256 + up(sizeof(int32_t) * (size_t)capacity) + pair_order_temp_bytes(capacity) +
           up(sizeof(Handoff) * (size_t)capacity) + 2 * up(sizeof(int32_t) * (size_t)capacity) +
           up(sizeof(EndRecord) * (size_t)capacity);
}

template <int BLOCK, bool MESH>
int launch_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                 const int64_t* n_dev, const d3d_gjk_options& opt, Handoff* hand, const DistanceOut& o,
                 const Lists& lists, int per_sm, cudaStream_t stream) {
    const float tol_sq = (float)(opt.tolerance * opt.tolerance);
    const void* ka = (const void*)k_gjk_mixed_a<BLOCK, MESH>;
    k_gjk_mixed_a<BLOCK, MESH><<<persistent_blocks(ka, BLOCK, n, per_sm), BLOCK, 0, stream>>>(
        store, i1, i2, order, n, n_dev, tol_sq, (float)opt.max_distance_squared, opt.max_iterations, hand, o,
        lists);
    int rc = check_launch("d3d_gjk_distance (mixed, FP32 phase)");
    if (rc) return rc;
    const void* kb = (const void*)k_gjk_mixed_b<BLOCK, MESH>;
    k_gjk_mixed_b<BLOCK, MESH><<<persistent_blocks(kb, BLOCK, n, per_sm), BLOCK, 0, stream>>>(
        store, i1, i2, order, n, n_dev, opt, hand, o, lists);
    rc = check_launch("d3d_gjk_distance (mixed, FP64 phase)");
    if (rc) return rc;
    k_gjk_mixed_end<<<persistent_blocks((const void*)k_gjk_mixed_end, 128, n), 128, 0, stream>>>(opt, o, lists);
    return check_launch("d3d_gjk_distance (mixed, end pass)");
}

// The kernels without the MeshGraph branch serve stores without meshes.
template <int BLOCK>
int launch_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                 const int64_t* n_dev, const d3d_gjk_options& opt, Handoff* hand, const DistanceOut& o,
                 const Lists& lists, int per_sm, cudaStream_t stream) {
    if (store.n_links > 0)
        return launch_mixed<BLOCK, true>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, per_sm, stream);
    return launch_mixed<BLOCK, false>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, per_sm, stream);
}

int gjk_mixed_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const int64_t* n_dev,
                  const d3d_gjk_options& opt, const DistanceOut& o, void* scratch, cudaStream_t stream) {
    const d3d_tuning t = tuning();
    const bool sched = n >= t.sort_min;
    const size_t order_bytes = up(sizeof(int32_t) * (size_t)n);
    const size_t temp_bytes = pair_order_temp_bytes(n);
    char* p = static_cast<char*>(scratch);
    Lists lists;
    lists.ctr = reinterpret_cast<unsigned long long*>(p);
    p += 256;
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p) : nullptr;
    p += order_bytes;
    void* temp = p;
    p += temp_bytes;
    Handoff* hand = reinterpret_cast<Handoff*>(p);
    p += up(sizeof(Handoff) * (size_t)n);
    lists.fallback = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)n);
    lists.ends = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)n);
    lists.records = reinterpret_cast<EndRecord*>(p);
    cudaError_t e = cudaMemsetAsync(lists.ctr, 0, kCounters * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) {
        set_error("d3d_gjk_distance (mixed): %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    int rc = sched ? pair_order(store, i1, i2, n, order, temp, temp_bytes, stream, n_dev) : D3D_SUCCESS;
    if (!rc) {
        if (t.gjk_block == 64)
            rc = launch_mixed<64>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, blocks_per_sm(t, 64), stream);
        else if (t.gjk_block == 256)
            rc = launch_mixed<256>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, blocks_per_sm(t, 256),
                                   stream);
        else
            rc = launch_mixed<128>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, blocks_per_sm(t, 128),
                                   stream);
    }
    if (!rc)
        rc = launch_gjk_f64(store, i1, i2, lists.fallback, n, lists.ctr + kNumFallback, lists.ctr + kCurC, opt, o,
                            stream);
    return rc;
}

int gjk_distance_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_gjk_options& opt, double* dist, double* cp1, double* cp2, double* simplex,
                       int8_t* n_simplex, int8_t* status, int32_t* iterations, cudaStream_t stream) {
    void* block = nullptr;
    int rc = scratch_alloc(&block, gjk_mixed_scratch_bytes(n), stream);
    if (rc) return rc;
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    rc = gjk_mixed_run(store, i1, i2, n, nullptr, opt, o, block, stream);
    scratch_free(block, stream);
    return rc;
}

}  // namespace d3d
