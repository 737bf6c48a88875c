// mpr_impl.h -- library-internal entry points of the MPR forms (mpr.cu,
// mpr_mixed.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "d3d_gb300.h"
#include "mpr.cuh"

namespace d3d {

// scratch of d3d_mpr for n pairs (counters, type order, sort temporaries; the
// mixed form's handoff and lists)
size_t mpr_scratch_bytes(int64_t n, bool mixed);
size_t mpr_mixed_extra_bytes(int64_t n);

// the FP64 kernel over pairs order[slot] (or slot) for slot < n, or < *n_dev
int mpr_f64_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const d3d_mpr_options& opt,
                   const mpr::Out& o, cudaStream_t stream);
int mpr_f64_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const d3d_mpr_options& opt,
                const mpr::Out& o, void* scratch, cudaStream_t stream);
int mpr_mixed_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                  const d3d_mpr_options& opt, const mpr::Out& o, void* scratch, cudaStream_t stream);

}  // namespace d3d
