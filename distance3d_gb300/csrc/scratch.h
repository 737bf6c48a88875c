// scratch.h -- library-internal temporaries and launch helpers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "d3d_gb300.h"

namespace d3d {

// Stream-ordered allocation from a per-device pool owned by the library
// (cudaMallocFromPoolAsync; memory stays cached in the pool up to 1 GiB).
// Returns D3D_SUCCESS or D3D_ERR_CUDA (message set).
int scratch_alloc(void** p, size_t bytes, cudaStream_t stream);
void scratch_free(void* p, cudaStream_t stream);

// Blocks for a persistent launch of `kernel` with `block` threads and
// `smem` bytes of dynamic shared memory: resident blocks per SM (at most
// max_per_sm if > 0) x SMs, capped by the work.
int persistent_blocks(const void* kernel, int block, int64_t work_items, int max_per_sm = 0, int smem = 0);

// The current launch parameters (d3d_set_tuning / d3d_autotune).
d3d_tuning tuning();

// blocks per SM for a GJK grid of `block` threads under tuning t (0: no cap)
inline int blocks_per_sm(const d3d_tuning& t, int block) {
    if (t.gjk_warps_per_sm <= 0) return 0;
    const int b = t.gjk_warps_per_sm / (block / 32);
    return b > 0 ? b : 1;
}

// Processing order of n pairs (i1[k], i2[k]): pair indices sorted by
// (type1, type2, hull-size class) so that a warp works on pairs that take the
// same support branches.  Writes order[n] (device).  `temp`/`temp_bytes`:
// see pair_order_temp_bytes.  With n_dev (device count <= n), the slots from
// *n_dev on are sorted to the end.
size_t pair_order_temp_bytes(int64_t n);
int pair_order(const d3d_store& s, const int32_t* i1, const int32_t* i2, int64_t n, int32_t* order, void* temp,
               size_t temp_bytes, cudaStream_t stream, const int64_t* n_dev = nullptr);

}  // namespace d3d
