// gjk_out.cuh -- per-pair output slots of d3d_gjk_distance.
#pragma once

#include "jolt.cuh"

namespace d3d {

struct DistanceOut {
    double* dist;
    double* cp1;
    double* cp2;
    double* simplex;
    int8_t* n_simplex;
    int8_t* status;
    int32_t* iterations;
};

// The slots of a pair whose collider indices are out of range.
__device__ __forceinline__ void store_bad_index(const DistanceOut& o, int64_t k) {
    o.dist[k] = NAN;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o.cp1[3 * k + j] = NAN;
        o.cp2[3 * k + j] = NAN;
    }
#pragma unroll
    for (int j = 0; j < 12; ++j) o.simplex[12 * k + j] = 0.0;
    o.n_simplex[k] = 0;
    o.status[k] = (int8_t)D3D_STATUS_BAD_INDEX;
    if (o.iterations) o.iterations[k] = 0;
}

template <typename Rows>
__device__ __forceinline__ void store_result(const DistanceOut& o, int64_t k, const GjkResult<double>& r,
                                             const Simplex<double, Rows>& S) {
    if (r.status == D3D_STATUS_CLIPPED) {
        o.dist[k] = DBL_MAX;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            o.cp1[3 * k + j] = NAN;
            o.cp2[3 * k + j] = NAN;
        }
    } else {
        o.dist[k] = r.dist;
        o.cp1[3 * k] = r.a.x;
        o.cp1[3 * k + 1] = r.a.y;
        o.cp1[3 * k + 2] = r.a.z;
        o.cp2[3 * k] = r.b.x;
        o.cp2[3 * k + 1] = r.b.y;
        o.cp2[3 * k + 2] = r.b.z;
    }
    double* sp = o.simplex + 12 * k;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        sp[3 * j] = S.Y[j].x;
        sp[3 * j + 1] = S.Y[j].y;
        sp[3 * j + 2] = S.Y[j].z;
    }
    o.n_simplex[k] = (int8_t)S.n;
    o.status[k] = (int8_t)r.status;
    if (o.iterations) o.iterations[k] = r.iters;
}

}  // namespace d3d
