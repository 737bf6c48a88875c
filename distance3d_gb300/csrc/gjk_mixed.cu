// gjk_mixed.cu -- mixed-precision GJK distance.
//
// Four kernels over the type-sorted pair order:
//
// A  runs the Jolt loop in FP32 on the FP32 mirror of the store, with
//    thresholds scaled to single precision, hands each pair's outcome, final
//    closest point and per-row search directions to the FP64 kernels (80
//    bytes/pair) and sorts the pair into one of three lists: separated,
//    touching, or fallback (clipped / not converged).
// T  re-evaluates a touching pair's FP32 simplex rows in FP64 along the
//    directions that produced them; if that simplex encloses the origin the
//    pair is done, otherwise the FP64 loop resumes there (in T).
// B  refines a separated pair in FP64: the reference's loop restarted from
//    A's closest-point direction (polytope supports choose their vertex by an
//    FP32 argmax and return the FP64 vertex), stopped when the duality gap
//    |v|^2 - v.w falls below 1e-8 |v|^2, which bounds the relative distance
//    error.
// C  is the plain FP64 kernel over the fallback list (the reference's
//    arithmetic; CLIPPED and MAX_ITER keep their FP64 meaning).
//
// T and B keep the simplex P/Q rows in shared memory and run one support
// call site per kernel, so that a warp's lanes share the support and simplex
// code whatever simplex size each holds.  A pair leaves T or B for the
// fallback list only if its result fails the consistency check (closest
// points vs |v|), the sanity check or the iteration bound.
//
// On the six-type workloads A takes ~8-10 FP32 iterations and B ~4-6 FP64
// iterations, against ~17-19 FP64 iterations for the plain form.  Compiled
// with -fmad=true: the tests bound its error against the FP64 oracle.
#include "capi_util.h"
#include "gjk_impl.h"
#include "gjk_mixed.cuh"
#include "gjk_out.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 128;
constexpr int64_t kScheduleMin = 4096;

using Rows64 = SmemRows<double, kBlock>;

// Per-call counters (one 256-byte block): cursors of A, T, B and C, then the
// lengths of the separated, touching and fallback lists.
enum { kCurA = 0, kCurT, kCurB, kCurC, kNumSep, kNumTouch, kNumFallback, kCounters };

struct Lists {
    int32_t* sep;
    int32_t* touch;
    int32_t* fallback;
    unsigned long long* ctr;
};

__global__ void __launch_bounds__(kBlock) k_gjk_mixed_a(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n, float tol_sq,
                                                        float max_d2, int max_iter, Handoff* __restrict__ hand,
                                                        Lists lists) {
    PhaseALoop L;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(lists.ctr + kCurA, need);
        if (need) {
            if (slot >= n) break;
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            pa_begin(L);
            need = false;
        }
        const int o = pa_step(L, s, a, b, tol_sq, max_d2, max_iter);
        const bool done = o >= 0;
        if (done) hand[pid] = pa_handoff(L, o);
        if (__any_sync(__activemask(), done)) {
            append_warp(lists.sep, lists.ctr + kNumSep, o == PA_SEPARATED, (int32_t)pid);
            append_warp(lists.touch, lists.ctr + kNumTouch, o == PA_TOUCHING, (int32_t)pid);
            append_warp(lists.fallback, lists.ctr + kNumFallback, o >= PA_CLIPPED, (int32_t)pid);
        }
        need = done;
    }
}

__global__ void __launch_bounds__(kBlock) k_gjk_mixed_t(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o, Lists lists) {
    __shared__ double rows[24 * kBlock];
    const int64_t n = (int64_t)lists.ctr[kNumTouch];
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    GjkLoop<double, Rows64> g;
    g.S.R.base = rows + threadIdx.x;
    while (true) {
        const long long k = fetch_slot(lists.ctr + kCurT, true);
        if (k >= n) break;
        const int32_t pid = lists.touch[k];
        const int a = i1[pid], b = i2[pid];
        GjkResult<double> r;
        int mode = pt_replay(g, s, a, b, hand + pid, tol_sq, E, r);
        if (mode == PB_RUN) {
            while (!pb_step(g, s, a, b, tol_sq, opt, E)) {
            }
            mode = pb_end(g, opt, E, r);
        }
        if (mode == PB_DONE) {
            r.iters += handoff_iters(hand[pid].v);
            store_result(o, pid, r, g.S);
        } else {
            lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_gjk_mixed_b(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o, Lists lists) {
    __shared__ double rows[24 * kBlock];
    const int64_t n = (int64_t)lists.ctr[kNumSep];
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    GjkLoop<double, Rows64> g;
    g.S.R.base = rows + threadIdx.x;
    int32_t pid = 0;
    int a = 0, b = 0;
    int it_a = 0;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(lists.ctr + kCurB, need);
        if (need) {
            if (slot >= n) break;
            pid = lists.sep[slot];
            a = i1[pid];
            b = i2[pid];
            const float4 v = hand[pid].v;
            it_a = handoff_iters(v);
            pb_begin(g, v);
            need = false;
        }
        if (pb_step(g, s, a, b, tol_sq, opt, E)) {
            GjkResult<double> r;
            if (pb_end(g, opt, E, r) == PB_DONE) {
                r.iters += it_a;
                store_result(o, pid, r, g.S);
            } else {
                lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
            }
            need = true;
        }
    }
}

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

namespace d3d {

int gjk_distance_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_gjk_options& opt, double* dist, double* cp1, double* cp2, double* simplex,
                       int8_t* n_simplex, int8_t* status, int32_t* iterations, cudaStream_t stream) {
    const bool sched = n >= kScheduleMin;
    const size_t counters = 256;
    const size_t order_bytes = sched ? up(sizeof(int32_t) * (size_t)n) : 0;
    const size_t hand_bytes = up(sizeof(Handoff) * (size_t)n);
    const size_t list_bytes = up(sizeof(int32_t) * (size_t)n);
    const size_t temp_bytes = sched ? pair_order_temp_bytes(n) : 0;
    void* block = nullptr;
    int rc = scratch_alloc(&block, counters + order_bytes + hand_bytes + 3 * list_bytes + temp_bytes, stream);
    if (rc) return rc;
    char* p = static_cast<char*>(block);
    Lists lists;
    lists.ctr = reinterpret_cast<unsigned long long*>(p);
    p += counters;
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p) : nullptr;
    p += order_bytes;
    Handoff* hand = reinterpret_cast<Handoff*>(p);
    p += hand_bytes;
    lists.sep = reinterpret_cast<int32_t*>(p);
    lists.touch = reinterpret_cast<int32_t*>(p + list_bytes);
    lists.fallback = reinterpret_cast<int32_t*>(p + 2 * list_bytes);
    void* temp = p + 3 * list_bytes;
    cudaMemsetAsync(lists.ctr, 0, kCounters * sizeof(unsigned long long), stream);
    if (sched) rc = pair_order(store, i1, i2, n, order, temp, temp_bytes, stream);
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    if (!rc) {
        const float tol_sq = (float)(opt.tolerance * opt.tolerance);
        k_gjk_mixed_a<<<persistent_blocks((const void*)k_gjk_mixed_a, kBlock, n), kBlock, 0, stream>>>(
            store, i1, i2, order, n, tol_sq, (float)opt.max_distance_squared, opt.max_iterations, hand, lists);
        rc = check_launch("d3d_gjk_distance (mixed, FP32 phase)");
    }
    if (!rc) {
        k_gjk_mixed_t<<<persistent_blocks((const void*)k_gjk_mixed_t, kBlock, n), kBlock, 0, stream>>>(
            store, i1, i2, opt, hand, o, lists);
        rc = check_launch("d3d_gjk_distance (mixed, FP64 touching phase)");
    }
    if (!rc) {
        k_gjk_mixed_b<<<persistent_blocks((const void*)k_gjk_mixed_b, kBlock, n), kBlock, 0, stream>>>(
            store, i1, i2, opt, hand, o, lists);
        rc = check_launch("d3d_gjk_distance (mixed, FP64 phase)");
    }
    if (!rc)
        rc = launch_gjk_f64(store, i1, i2, lists.fallback, n, lists.ctr + kNumFallback, lists.ctr + kCurC, opt, o,
                            stream);
    scratch_free(block, stream);
    return rc;
}

}  // namespace d3d
