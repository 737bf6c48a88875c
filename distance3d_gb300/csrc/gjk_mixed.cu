// gjk_mixed.cu -- mixed-precision GJK distance.
//
// Three persistent kernels over the type-sorted pair order:
//
// A  runs the Jolt loop in FP32 on the FP32 mirror of the store, with
//    thresholds scaled to single precision, and hands each pair's outcome,
//    final closest point and per-row search directions to B (80 bytes/pair).
// B  refines in FP64.  A separated pair restarts the reference's loop from
//    A's closest-point direction (polytope supports choose their vertex by an
//    FP32 argmax and return the FP64 vertex) and stops when the duality gap
//    |v|^2 - v.w falls below 1e-9 |v|^2, which bounds the relative distance
//    error.  A touching pair re-evaluates A's simplex rows in FP64; if that
//    simplex encloses the origin the pair is done, otherwise the loop resumes
//    there.  Pairs whose result fails the consistency check (closest points
//    vs |v|), that A clipped or that did not converge are appended to a
//    fallback list.
// C  is the plain FP64 kernel over the fallback list (the reference's
//    arithmetic; CLIPPED and MAX_ITER keep their FP64 meaning).
//
// On the six-type workloads A takes ~8-10 FP32 iterations and B ~4-7 FP64
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

__global__ void __launch_bounds__(kBlock) k_gjk_mixed_a(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        unsigned long long* __restrict__ cursor, float tol_sq,
                                                        float max_d2, int max_iter, Handoff* __restrict__ hand) {
    PhaseALoop L;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(cursor, need);
        if (need) {
            if (slot >= n) break;
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            pa_begin(L);
            need = false;
        }
        Col<float> f1, f2;
        load_col(s, a, f1);
        load_col(s, b, f2);
        const int o = pa_step(L, f1, f2, s, tol_sq, max_d2, max_iter);
        if (o >= 0) {
            hand[pid] = pa_handoff(L, o);
            need = true;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_gjk_mixed_b(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        unsigned long long* __restrict__ cursor, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o,
                                                        int32_t* __restrict__ fallback,
                                                        unsigned long long* __restrict__ n_fallback) {
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    GjkLoop<double> g;
    GjkResult<double> r;
    int64_t pid = 0;
    int a = 0, b = 0;
    int it_a = 0;
    int mode = PB_DONE;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(cursor, need);
        Col<double> c1, c2;
        if (need) {
            if (slot >= n) break;
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            load_col(s, a, c1);
            load_col(s, b, c2);
            const Handoff h = hand[pid];
            it_a = handoff_iters(h);
            mode = pb_begin(h, c1, c2, s, tol_sq, E, g, r);
            need = false;
        }
        if (mode == PB_RUN) {
            load_col(s, a, c1);
            load_col(s, b, c2);
            if (pb_step(g, c1, c2, s, tol_sq, opt, E)) mode = pb_end(g, opt, E, r);
        }
        if (mode == PB_DONE) {
            r.iters += it_a;
            store_result(o, pid, r, g.S);
            need = true;
        } else if (mode == PB_FALLBACK) {
            fallback[atomicAdd(n_fallback, 1ull)] = (int32_t)pid;
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
    const size_t counters = 256;  // 3 cursors + fallback count
    const size_t order_bytes = sched ? up(sizeof(int32_t) * (size_t)n) : 0;
    const size_t hand_bytes = up(sizeof(Handoff) * (size_t)n);
    const size_t fb_bytes = up(sizeof(int32_t) * (size_t)n);
    const size_t temp_bytes = sched ? pair_order_temp_bytes(n) : 0;
    void* block = nullptr;
    int rc = scratch_alloc(&block, counters + order_bytes + hand_bytes + fb_bytes + temp_bytes, stream);
    if (rc) return rc;
    char* p = static_cast<char*>(block);
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(p);
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p + counters) : nullptr;
    Handoff* hand = reinterpret_cast<Handoff*>(p + counters + order_bytes);
    int32_t* fallback = reinterpret_cast<int32_t*>(p + counters + order_bytes + hand_bytes);
    void* temp = p + counters + order_bytes + hand_bytes + fb_bytes;
    cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), stream);
    if (sched) rc = pair_order(store, i1, i2, n, order, temp, temp_bytes, stream);
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    if (!rc) {
        const float tol_sq = (float)(opt.tolerance * opt.tolerance);
        k_gjk_mixed_a<<<persistent_blocks((const void*)k_gjk_mixed_a, kBlock, n), kBlock, 0, stream>>>(
            store, i1, i2, order, n, ctr + 0, tol_sq, (float)opt.max_distance_squared, opt.max_iterations, hand);
        rc = check_launch("d3d_gjk_distance (mixed, FP32 phase)");
    }
    if (!rc) {
        k_gjk_mixed_b<<<persistent_blocks((const void*)k_gjk_mixed_b, kBlock, n), kBlock, 0, stream>>>(
            store, i1, i2, order, n, ctr + 1, opt, hand, o, fallback, ctr + 3);
        rc = check_launch("d3d_gjk_distance (mixed, FP64 phase)");
    }
    if (!rc) rc = launch_gjk_f64(store, i1, i2, fallback, n, ctr + 3, ctr + 2, opt, o, stream);
    scratch_free(block, stream);
    return rc;
}

}  // namespace d3d
