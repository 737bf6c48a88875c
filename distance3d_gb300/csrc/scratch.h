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

// Blocks for a persistent launch of `kernel` with `block` threads:
// resident blocks per SM x SMs, capped by the work.
int persistent_blocks(const void* kernel, int block, int64_t work_items);

// Processing order of n pairs (i1[k], i2[k]): pair indices sorted by
// (type1, type2, hull-size class) so that a warp works on pairs that take the
// same support branches.  Writes order[n] (device).  `temp`/`temp_bytes`:
// see pair_order_temp_bytes.  With n_dev (device count <= n), the slots from
// *n_dev on are sorted to the end.
size_t pair_order_temp_bytes(int64_t n);
int pair_order(const d3d_store& s, const int32_t* i1, const int32_t* i2, int64_t n, int32_t* order, void* temp,
               size_t temp_bytes, cudaStream_t stream, const int64_t* n_dev = nullptr);

}  // namespace d3d
