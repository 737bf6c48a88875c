// mpr_mixed.cu -- the mixed-precision MPR (d3d_mpr with D3D_PRECISION_MIXED).
//
// A  the state machine of mpr.cuh in FP32 on the FP32 mirror (FastSupport),
//    one support evaluation per round, persistent lanes over the type-sorted
//    pairs.  Misses and intersection-only hits are final here.  A hit with
//    penetration hands over its outcome and the FP32 search directions of the
//    final portal's rows; a pair whose refinement reached `refine_limit` goes
//    to the FP64 kernel of mpr.cu.
// B  one lane per handed-over pair: the FP64 centers, the final portal's rows
//    evaluated in FP64 along their FP32 directions (RefineSupport: the FP32
//    discrete choices, FP64 points), then the reference's depth, direction and
//    contact position (mpr.py:337-393) in FP64.
//
// The FP32 search makes the reference's decisions wherever FP32 resolves them
// (everything but pairs within FP32 noise of touching, and near-ties between
// portal expansions); the collinear test of the portal discovery adds the
// FP32 noise of |v0 x v1|^2 to the reference's EPSILON so that the
// origin-on-segment case is found as in FP64.  Compiled with -fmad=true.
#include "capi_util.h"
#include "gjk_mixed.cuh"
#include "mpr.cuh"
#include "mpr_impl.h"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 128;

// Per-call counters (one 256-byte block): cursors of A, B and the FP64
// fallback, then the lengths of the handoff and fallback lists.
enum { kCurA = 0, kCurB, kCurC, kNumRefine, kNumFallback, kCounters };

struct Lists {
    int32_t* refine;
    int32_t* fallback;
    unsigned long long* ctr;
};

// A hit's final portal: the FP32 search directions of rows 1-3 (xyz) and
// the outcome (w of row 1, as int bits).
struct __align__(16) PortalHandoff {
    float4 d[3];
};

template <bool MESH>
__global__ void __launch_bounds__(kBlock) k_mpr_mixed_a(d3d_store st, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        d3d_mpr_options opt, PortalHandoff* __restrict__ hand, Lists lists,
                                                        mpr::Out o) {
    using PortalT = mpr::Portal<float, kBlock, false>;
    __shared__ float rows[PortalT::kWords * kBlock];
    const PortalT P{rows + threadIdx.x};
    mpr::Lane<float> L;
    int64_t pid = 0;
    int i = 0, j = 0;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(lists.ctr + kCurA, need);
        if (need) {
            if (slot >= n) break;
            pid = order ? order[slot] : slot;
            i = i1[pid];
            j = i2[pid];
            if (!pair_ok(st, i, j)) {
                const d3 nan3 = mk(double(NAN), double(NAN), double(NAN));
                mpr::store(o, pid, false, D3D_STATUS_BAD_INDEX, opt.penetration, NAN, nan3, nan3);
                continue;  // the lane fetches again
            }
            mpr::begin(P, L, mpr::collider_center<float>(st, i), mpr::collider_center<float>(st, j));
            need = false;
        }
        f3 pa, pb;
        pair_supports<float, FastSupportT<MESH>>(st, i, j, L.d, pa, pb);
        int status = D3D_STATUS_OK;
        const int r = mpr::round(P, L, pa, pb, opt, status);
        const bool done = r != mpr::kRunning;
        const bool fallback = done && status != D3D_STATUS_OK;
        const bool refine = done && !fallback && r != mpr::kMiss && opt.penetration;
        if (done && !fallback && !refine) {
            const d3 nan3 = mk(double(NAN), double(NAN), double(NAN));
            mpr::store(o, pid, r != mpr::kMiss, D3D_STATUS_OK, opt.penetration, NAN, nan3, nan3);
        }
        if (refine) {
            PortalHandoff h;
            for (int k = 0; k < 3; ++k) {
                const f3 d = P.dir(k + 1);
                h.d[k] = make_float4(d.x, d.y, d.z, 0.f);
            }
            h.d[0].w = __int_as_float(r);
            hand[pid] = h;
        }
        if (__any_sync(__activemask(), done)) {
            append_warp(lists.refine, lists.ctr + kNumRefine, refine, (int32_t)pid);
            append_warp(lists.fallback, lists.ctr + kNumFallback, fallback, (int32_t)pid);
        }
        need = done;
    }
}

// The final portal's FP64 rows, for mpr::penetration.
struct Rows {
    d3 vv[4], av[4], bv[4];
    __device__ d3 v(int k) const { return vv[k]; }
    __device__ d3 a(int k) const { return av[k]; }
    __device__ d3 b(int k) const { return bv[k]; }
};

template <bool MESH>
__global__ void __launch_bounds__(kBlock) k_mpr_mixed_b(d3d_store st, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const PortalHandoff* __restrict__ hand, Lists lists, mpr::Out o) {
    const int64_t n = (int64_t)lists.ctr[kNumRefine];
    for (int64_t s = (int64_t)blockIdx.x * kBlock + threadIdx.x; s < n; s += (int64_t)gridDim.x * kBlock) {
        const int32_t pid = lists.refine[s];
        const int i = i1[pid], j = i2[pid];
        const PortalHandoff h = hand[pid];
        const int outcome = __float_as_int(h.d[0].w);
        Rows R;
        R.av[0] = mpr::collider_center<double>(st, i);
        R.bv[0] = mpr::collider_center<double>(st, j);
        R.vv[0] = R.av[0] - R.bv[0];
        if (mpr::all_zero(R.vv[0])) R.vv[0].x += mpr::kEps * 10.0;
        const int rows = outcome == mpr::kHitPortal ? 3 : 1;
        for (int k = 0; k < 3; ++k) {
            if (k < rows) {
                const d3 d = mk((double)h.d[k].x, (double)h.d[k].y, (double)h.d[k].z);
                pair_supports<double, RefineSupportT<MESH>>(st, i, j, d, R.av[k + 1], R.bv[k + 1]);
                R.vv[k + 1] = R.av[k + 1] - R.bv[k + 1];
            } else {
                R.vv[k + 1] = R.av[k + 1] = R.bv[k + 1] = mk(0.0, 0.0, 0.0);
            }
        }
        double depth;
        d3 dir, pos;
        mpr::penetration(outcome, R, depth, dir, pos);
        mpr::store(o, pid, true, D3D_STATUS_OK, true, depth, dir, pos);
    }
}

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

template <bool MESH>
int launch_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                 const d3d_mpr_options& opt, PortalHandoff* hand, const Lists& lists, const mpr::Out& o,
                 cudaStream_t stream) {
    const void* ka = (const void*)k_mpr_mixed_a<MESH>;
    k_mpr_mixed_a<MESH><<<persistent_blocks(ka, kBlock, n), kBlock, 0, stream>>>(store, i1, i2, order, n, opt, hand,
                                                                                 lists, o);
    int rc = check_launch("d3d_mpr (mixed, FP32 search)");
    if (rc) return rc;
    const void* kb = (const void*)k_mpr_mixed_b<MESH>;
    k_mpr_mixed_b<MESH><<<persistent_blocks(kb, kBlock, n), kBlock, 0, stream>>>(store, i1, i2, hand, lists, o);
    return check_launch("d3d_mpr (mixed, FP64 portal)");
}

}  // namespace

namespace d3d {

size_t mpr_mixed_extra_bytes(int64_t n) {
    return 256 + up(sizeof(PortalHandoff) * (size_t)n) + 2 * up(sizeof(int32_t) * (size_t)n);
}

int mpr_mixed_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                  const d3d_mpr_options& opt, const mpr::Out& o, void* scratch, cudaStream_t stream) {
    const bool sched = n >= tuning().sort_min;
    char* p = static_cast<char*>(scratch) + 256;  // the FP64 form's cursor block stays unused
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p) : nullptr;
    p += up(sizeof(int32_t) * (size_t)n);
    void* temp = p;
    p += pair_order_temp_bytes(n);
    Lists lists;
    lists.ctr = reinterpret_cast<unsigned long long*>(p);
    p += 256;
    PortalHandoff* hand = reinterpret_cast<PortalHandoff*>(p);
    p += up(sizeof(PortalHandoff) * (size_t)n);
    lists.refine = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)n);
    lists.fallback = reinterpret_cast<int32_t*>(p);
    cudaError_t e = cudaMemsetAsync(lists.ctr, 0, kCounters * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) {
        set_error("d3d_mpr (mixed): %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    int rc = sched ? pair_order(store, i1, i2, n, order, temp, pair_order_temp_bytes(n), stream) : D3D_SUCCESS;
    if (!rc)
        rc = store.n_links > 0 ? launch_mixed<true>(store, i1, i2, order, n, opt, hand, lists, o, stream)
                               : launch_mixed<false>(store, i1, i2, order, n, opt, hand, lists, o, stream);
    if (!rc)
        rc = mpr_f64_launch(store, i1, i2, lists.fallback, n, lists.ctr + kNumFallback, lists.ctr + kCurC, opt, o,
                            stream);
    return rc;
}

}  // namespace d3d
