// collide.cu -- one GJK + EPA batch whose pair count lives on the device.
//
// d3d_collide runs, for pairs k < *n_dev of buffers sized `capacity`, GJK
// distance (precision of the GJK options) and then EPA (precision of the EPA
// options) on the pairs GJK found intersecting with a full simplex -- the
// reference's composition, gjk() then epa() on the returned simplex
// (gjk/_gjk_jolt.py:138-221, epa.py:9-78).  The EPA pairs are found and
// listed on the device.  There is no host synchronisation and no allocation,
// and every launch shape depends on `capacity` only, so a CUDA graph can hold
// one call and replay it for any count up to the capacity.
#include "capi_util.h"
#include "epa_mixed.h"
#include "gjk_impl.h"
#include "gjk_out.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 256;
constexpr int64_t kF64Slots = 32768;      // FP64 EPA polytopes in flight (FP64 form)
constexpr int64_t kFallbackSlots = 2048;  // FP64 EPA polytopes for the mixed form's fallback pairs

// counters: EPA cursor, FP64 cursor, fallback count, EPA list length, FP64
// warp cursor, second fallback count
enum { kEpaCur = 0, kF64Cur, kNumFallback, kNumEpa, kW64Cur, kNumFallback2, kNumRefine, kCounters };

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

bool warp_form(const d3d_epa_options& o) { return o.precision == D3D_PRECISION_MIXED && epa_warp_supported(o); }

int64_t f64_slots(int64_t capacity, const d3d_epa_options& o) {
    int64_t s = warp_form(o) ? kFallbackSlots : kF64Slots;
    if (s > capacity) s = capacity;
    return ((s + 127) / 128) * 128;
}

size_t gjk_bytes(int64_t capacity, const d3d_gjk_options& g) {
    return g.precision == D3D_PRECISION_MIXED ? gjk_mixed_scratch_bytes(capacity) : gjk_f64_scratch_bytes(capacity);
}

// Every pair k < n gets "no EPA" (status -1, NaN mtv, no faces); those GJK
// left at distance 0 with a full simplex are appended to the EPA list.
__global__ void k_epa_select(int64_t cap, const int64_t* __restrict__ n_dev, const double* __restrict__ dist,
                             const int8_t* __restrict__ n_simplex, int32_t* __restrict__ list,
                             unsigned long long* __restrict__ count, double* __restrict__ mtv,
                             int8_t* __restrict__ status, int32_t* __restrict__ n_faces) {
    const int64_t n = *n_dev;
    for (int64_t k0 = (int64_t)blockIdx.x * blockDim.x; k0 < cap; k0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = k0 + threadIdx.x;
        bool take = false;
        if (k < n) {
            mtv[3 * k] = NAN;
            mtv[3 * k + 1] = NAN;
            mtv[3 * k + 2] = NAN;
            status[k] = -1;
            n_faces[k] = 0;
            take = dist[k] == 0.0 && n_simplex[k] == 4;
        }
        append_warp(list, count, take, (int32_t)k);
    }
}

}  // namespace

extern "C" size_t d3d_collide_scratch_bytes(int64_t capacity, const d3d_gjk_options* gjk,
                                            const d3d_epa_options* epa) {
    if (capacity <= 0 || !gjk || !epa || epa->max_faces < 4) return 0;
    return 256 + 4 * up(sizeof(int32_t) * (size_t)capacity) + up(gjk_bytes(capacity, *gjk)) +
           (size_t)(f64_slots(capacity, *epa) * epa_f64_slot_bytes(*epa));
}

extern "C" int d3d_collide(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t capacity,
                           const int64_t* n_dev, const d3d_gjk_options* gjk, const d3d_epa_options* epa,
                           double* dist, double* cp1, double* cp2, double* simplex, int8_t* n_simplex,
                           int8_t* status, int32_t* iterations, double* mtv, int8_t* epa_status, int32_t* n_faces,
                           void* scratch, size_t scratch_bytes, void* stream) {
    int rc = d3d::check_store(store, "d3d_collide");
    if (rc) return rc;
    D3D_REQUIRE(gjk && epa, "d3d_collide: null options");
    D3D_REQUIRE(capacity > 0 && capacity <= INT32_MAX, "d3d_collide: capacity %lld out of range",
                (long long)capacity);
    D3D_REQUIRE(gjk->max_iterations >= 1, "d3d_collide: max_iterations < 1");
    D3D_REQUIRE(gjk->precision == D3D_PRECISION_FP64 || gjk->precision == D3D_PRECISION_MIXED,
                "d3d_collide: unknown GJK precision %d", gjk->precision);
    D3D_REQUIRE(epa->max_iterations >= 0 && epa->max_faces >= 4 && epa->max_loose_edges >= 0 && epa->epsilon >= 0.0 &&
                    (epa->precision == D3D_PRECISION_FP64 || epa->precision == D3D_PRECISION_MIXED),
                "d3d_collide: invalid EPA options");
    D3D_REQUIRE(i1 && i2 && n_dev && dist && cp1 && cp2 && simplex && n_simplex && status && mtv && epa_status &&
                    n_faces && scratch,
                "d3d_collide: null pointer");
    const size_t need = d3d_collide_scratch_bytes(capacity, gjk, epa);
    if (scratch_bytes < need) {
        d3d::set_error("d3d_collide: scratch of %zu bytes < %zu needed", scratch_bytes, need);
        return D3D_ERR_CAPACITY;
    }
    cudaStream_t st = d3d::as_stream(stream);
    char* p = static_cast<char*>(scratch);
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(p);
    p += 256;
    int32_t* list = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)capacity);
    int32_t* fallback = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)capacity);
    int32_t* fallback2 = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)capacity);
    int32_t* refine = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * (size_t)capacity);
    void* gjk_scratch = p;
    p += up(gjk_bytes(capacity, *gjk));
    void* slots = p;

    cudaError_t e = cudaMemsetAsync(ctr, 0, kCounters * sizeof(unsigned long long), st);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_collide: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    rc = gjk->precision == D3D_PRECISION_MIXED
             ? d3d::gjk_mixed_run(*store, i1, i2, capacity, n_dev, *gjk, o, gjk_scratch, st)
             : d3d::gjk_f64_run(*store, i1, i2, capacity, n_dev, *gjk, o, gjk_scratch, st);
    if (rc) return rc;
    const int sel_blocks = d3d::persistent_blocks((const void*)k_epa_select, kBlock, capacity);
    k_epa_select<<<sel_blocks, kBlock, 0, st>>>(capacity, n_dev, dist, n_simplex, list, ctr + kNumEpa, mtv,
                                                epa_status, n_faces);
    rc = d3d::check_launch("d3d_collide (EPA pair selection)");
    if (rc) return rc;
    const int64_t nslots = f64_slots(capacity, *epa);
    if (warp_form(*epa)) {
        rc = d3d::epa_warp_launch(*store, i1, i2, list, capacity, ctr + kNumEpa, ctr + kEpaCur, simplex, *epa, mtv,
                                  epa_status, n_faces, nullptr, fallback, ctr + kNumFallback, st, false, refine,
                                  ctr + kNumRefine);
        const bool w64 = d3d::epa_warp_supported(*epa, true);
        if (!rc && w64)
            rc = d3d::epa_warp_launch(*store, i1, i2, fallback, capacity, ctr + kNumFallback, ctr + kW64Cur, simplex,
                                      *epa, mtv, epa_status, n_faces, nullptr, fallback2, ctr + kNumFallback2, st,
                                      true);
        if (!rc)
            rc = d3d::epa_f64_launch(*store, i1, i2, w64 ? fallback2 : fallback, capacity,
                                     ctr + (w64 ? kNumFallback2 : kNumFallback), ctr + kF64Cur, simplex, *epa, mtv,
                                     epa_status, n_faces, nullptr, slots, nslots, st);
    } else {
        rc = d3d::epa_f64_launch(*store, i1, i2, list, capacity, ctr + kNumEpa, ctr + kF64Cur, simplex, *epa, mtv,
                                 epa_status, n_faces, nullptr, slots, nslots, st);
    }
    return rc;
}
