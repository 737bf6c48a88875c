// epa_mixed.h -- the mixed-precision EPA launcher (epa_mixed.cu), used by
// d3d_epa when options->precision is D3D_PRECISION_MIXED.
#pragma once

#include <cuda_runtime.h>

#include "d3d_gb300.h"

namespace d3d {

// bytes of one polytope slot: (max_iterations + 4) vertices and max_faces
// faces of 32 bytes, max_loose_edges edges of 8 bytes, a max_faces queue of
// 4 bytes (rounded up to 16)
int64_t epa_mixed_slot_bytes(const d3d_epa_options& o);

// persistent launch over `order` (null: input order); at most max_slots
// threads, each owning slot max_slots-aligned in `scratch`
// Pairs whose FP32 polytope fails validation are appended to fallback[]
// (count in *n_fallback) for the FP64 EPA.
int epa_mixed_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                     unsigned long long* cursor, const double* simplex, const d3d_epa_options& o, double* mtv,
                     int8_t* status, int32_t* n_faces, double* faces, void* scratch, int64_t max_slots,
                     int32_t* fallback, unsigned long long* n_fallback, cudaStream_t stream);

// The warp-per-pair form (epa_warp.cu): one warp per pair, its polytope in
// shared memory, FP32 (fp64 = false) or FP64 with the reference's supports
// (fp64 = true, for the FP32 form's fallback pairs); supported when
// max_iterations <= 250, max_loose_edges <= 255 and four polytopes fit in a
// block's shared memory.  Runs pairs list[k] (or k) for k < n, or
// k < *n_dev if n_dev is given (n then only sizes the launch); fallback pairs
// as above.  With `refine` (FP32 form only), each converged pair's FP32 face
// normal goes to mtv and the pair to refine[*n_refine ...] (the caller zeroes
// the count), and a second kernel then computes the pairs' FP64 depths along
// those normals, one pair per thread.
bool epa_warp_supported(const d3d_epa_options& o, bool fp64 = false);
int epa_warp_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                    const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                    const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                    int32_t* fallback, unsigned long long* n_fallback, cudaStream_t stream, bool fp64 = false,
                    int32_t* refine = nullptr, unsigned long long* n_refine = nullptr);

// The FP64 EPA (epa.cu) over list[k] (or k) for k < n or < *n_dev, on
// `slots` polytope slots of slot_bytes(o) in `scratch`.
int64_t epa_f64_slot_bytes(const d3d_epa_options& o);
int epa_f64_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                   const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                   void* scratch, int64_t slots, cudaStream_t stream);

}  // namespace d3d
