// mpr.cu -- Minkowski portal refinement (MPR), the plain FP64 drop-in for
// distance3d's mpr_intersection and mpr_penetration (mpr.py:21-110).
// Compiled with -fmad=false: every step is the reference's
// rounding sequence (NumPy orders as in d3d_device.cuh), so flags, depths,
// directions and contact positions are the reference's bit for bit.
//
// Each lane of the persistent kernel runs one pair as the state machine of
// mpr.cuh, one support evaluation per round (portal discovery, refinement,
// penetration search), and takes the next pair of the type-sorted order when
// its pair ends.  The portal (four Minkowski-difference vertices and the two
// colliders' support points behind each) lives in shared memory, one column
// per lane (stride kBlock), because the reference replaces its rows by
// data-dependent index.  The refinement loop of the reference has no bound;
// here it stops after `refine_limit` expansions with status
// D3D_STATUS_MAX_ITER.  d3d_mpr also dispatches the mixed form
// (mpr_mixed.cu).
#include "capi_util.h"
#include "mpr.cuh"
#include "mpr_impl.h"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 128;
constexpr int kChunk = 32;  // slots a warp claims from the type-sorted order at a time

// Persistent MPR: each lane runs one pair's MPR one support evaluation per
// round and fetches the next pair (in the type-sorted `order`) when its pair
// ends, so the support code runs once per round for the whole warp.  With
// n_dev, the pair count is read on the device (the mixed form's fallback
// list).
__global__ void __launch_bounds__(kBlock) k_mpr(d3d_store st, const int32_t* __restrict__ i1,
                                                const int32_t* __restrict__ i2, const int32_t* __restrict__ order,
                                                int64_t n, const unsigned long long* __restrict__ n_dev,
                                                unsigned long long* __restrict__ cursor, d3d_mpr_options opt,
                                                mpr::Out o) {
    using PortalT = mpr::Portal<double, kBlock, true>;
    __shared__ double rows[PortalT::kWords * kBlock];
    const PortalT P{rows + threadIdx.x};
    if (n_dev) n = (int64_t)*n_dev;
    mpr::Lane<double> L;
    int64_t pid = 0;
    int i = 0, j = 0;
    bool need = true;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // per-lane claims for the last slots: MPR pairs are short (whole chunks to the end held up the
    // end of a 131,072-pair launch by ~20%)
    const long long split = n - 2LL * gridDim.x * blockDim.x;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(cursor, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            pid = order ? order[slot] : slot;
            i = i1[pid];
            j = i2[pid];
            if (!pair_ok(st, i, j)) {
                const d3 nan3 = mk(double(NAN), double(NAN), double(NAN));
                mpr::store(o, pid, false, D3D_STATUS_BAD_INDEX, opt.penetration, NAN, nan3, nan3);
                continue;  // the lane fetches again
            }
            mpr::begin(P, L, mpr::collider_center<double>(st, i), mpr::collider_center<double>(st, j));
            need = false;
        }
        d3 pa, pb;
        pair_supports<double, ExactSupport>(st, i, j, L.d, pa, pb);
        int status = D3D_STATUS_OK;
        const int r = mpr::round(P, L, pa, pb, opt, status);
        if (r != mpr::kRunning) {
            double depth = NAN;
            d3 dir = mk(double(NAN), double(NAN), double(NAN)), pos = dir;
            if (r != mpr::kMiss && opt.penetration) mpr::penetration(r, P, depth, dir, pos);
            mpr::store(o, pid, r != mpr::kMiss, status, opt.penetration, depth, dir, pos);
            need = true;
        }
    }
}

}  // namespace

namespace d3d {

int mpr_f64_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const d3d_mpr_options& opt,
                   const mpr::Out& o, cudaStream_t stream) {
    const int blocks = persistent_blocks((const void*)k_mpr, kBlock, n);
    k_mpr<<<blocks, kBlock, 0, stream>>>(store, i1, i2, order, n, n_dev, cursor, opt, o);
    return check_launch("d3d_mpr");
}

}  // namespace d3d

extern "C" int d3d_mpr(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_mpr_options* opt, int8_t* hit, double* depth, double* dir, double* pos,
                       int8_t* status, void* stream) {
    int rc = d3d::check_store(store, "d3d_mpr");
    if (rc) return rc;
    D3D_REQUIRE(opt, "d3d_mpr: null options");
    D3D_REQUIRE(n >= 0, "d3d_mpr: n < 0");
    D3D_REQUIRE(opt->max_iterations >= 0 && opt->refine_limit >= 0, "d3d_mpr: negative iteration bound");
    D3D_REQUIRE(opt->tolerance >= 0.0, "d3d_mpr: negative tolerance");
    D3D_REQUIRE(opt->precision == D3D_PRECISION_FP64 || opt->precision == D3D_PRECISION_MIXED,
                "d3d_mpr: unknown precision %d", opt->precision);
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && hit && status, "d3d_mpr: null pointer");
    D3D_REQUIRE(n <= INT32_MAX, "d3d_mpr: more than 2^31 pairs");
    cudaStream_t st = d3d::as_stream(stream);
    const bool mixed = opt->precision == D3D_PRECISION_MIXED;
    void* scratch = nullptr;
    rc = d3d::scratch_alloc(&scratch, d3d::mpr_scratch_bytes(n, mixed), st);
    if (rc) return rc;
    d3d::mpr::Out o{hit, depth, dir, pos, status};
    rc = mixed ? d3d::mpr_mixed_run(*store, i1, i2, n, *opt, o, scratch, st)
               : d3d::mpr_f64_run(*store, i1, i2, n, *opt, o, scratch, st);
    d3d::scratch_free(scratch, st);
    return rc;
}

namespace d3d {

size_t mpr_scratch_bytes(int64_t n, bool mixed) {
    const size_t order = (sizeof(int32_t) * (size_t)n + 255) & ~size_t(255);
    size_t bytes = 256 + order + pair_order_temp_bytes(n);
    if (mixed) bytes += mpr_mixed_extra_bytes(n);
    return bytes;
}

int mpr_f64_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const d3d_mpr_options& opt,
                const mpr::Out& o, void* scratch, cudaStream_t st) {
    const bool sched = n >= tuning().sort_min;
    unsigned long long* cursor = static_cast<unsigned long long*>(scratch);
    const size_t order_bytes = (sizeof(int32_t) * (size_t)n + 255) & ~size_t(255);
    int32_t* order = sched ? reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + 256) : nullptr;
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) {
        set_error("d3d_mpr: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    int rc = D3D_SUCCESS;
    if (sched)
        rc = pair_order(store, i1, i2, n, order, static_cast<char*>(scratch) + 256 + order_bytes,
                        pair_order_temp_bytes(n), st);
    if (!rc) rc = mpr_f64_launch(store, i1, i2, order, n, nullptr, cursor, opt, o, st);
    return rc;
}

}  // namespace d3d
