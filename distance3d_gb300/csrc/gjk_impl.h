// gjk_impl.h -- internal entry points shared between the GJK translation units.
#pragma once

#include <cuda_runtime.h>

#include "d3d_gb300.h"

namespace d3d {

struct DistanceOut;

// persistent FP64 GJK distance over `order` (null: input order); n_dev, if
// not null, holds the pair count on the device; *cursor must be zero
int launch_gjk_f64(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const d3d_gjk_options& opt,
                   const DistanceOut& o, cudaStream_t stream);

// The mixed form on caller scratch (gjk_mixed_scratch_bytes(n)); with n_dev,
// the pair count is *n_dev <= n, read on the device, and the launches depend
// on n only (a CUDA graph can hold them).
size_t gjk_mixed_scratch_bytes(int64_t capacity);
int gjk_mixed_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const int64_t* n_dev,
                  const d3d_gjk_options& opt, const DistanceOut& o, void* scratch, cudaStream_t stream);

// the same on the FP64 kernel (gjk.cu)
size_t gjk_f64_scratch_bytes(int64_t capacity);
int gjk_f64_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const int64_t* n_dev,
                const d3d_gjk_options& opt, const DistanceOut& o, void* scratch, cudaStream_t stream);

// mixed-precision form of d3d_gjk_distance (gjk_mixed.cu)
int gjk_distance_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_gjk_options& opt, double* dist, double* cp1, double* cp2, double* simplex,
                       int8_t* n_simplex, int8_t* status, int32_t* iterations, cudaStream_t stream);

}  // namespace d3d
