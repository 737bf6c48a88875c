// capi_util.h -- host-side helpers of the C ABI: per-thread error message,
// argument checks, launch checks.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "d3d_gb300.h"

namespace d3d {

// defined in capi.cu
void set_error(const char* fmt, ...);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    return D3D_SUCCESS;
}

inline int check_store(const d3d_store* s, const char* what) {
    if (!s || !s->rec64 || !s->rec32 || !s->meta || s->n_colliders < 0 || s->n_vertices < 0 ||
        (s->n_vertices > 0 && (!s->verts64 || !s->verts32)) || s->n_links < 0 || (s->n_links > 0 && !s->links)) {
        set_error("%s: invalid d3d_store", what);
        return D3D_ERR_INVALID;
    }
    if (s->n_colliders >= (int64_t(1) << 31) || s->n_vertices >= (int64_t(1) << 31) ||
        s->n_links >= (int64_t(1) << 31)) {
        set_error("%s: store larger than 2^31 colliders, vertices or links", what);
        return D3D_ERR_INVALID;
    }
    return D3D_SUCCESS;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace d3d

#define D3D_REQUIRE(cond, ...)            \
    do {                                  \
        if (!(cond)) {                    \
            ::d3d::set_error(__VA_ARGS__); \
            return D3D_ERR_INVALID;       \
        }                                 \
    } while (0)
