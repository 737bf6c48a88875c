// epa_mixed.cu -- mixed-precision EPA.
//
// The expanding-polytope search (epa.py:59-74) runs in FP32 on the FP32
// mirror of the store; only the converged face is refined in FP64.
//
// Polytope.  Each pair keeps a vertex table (Minkowski point y and the search
// direction that produced it; the four starting vertices remember their row of
// the FP64 input simplex instead) and faces as three vertex ids plus the unit
// normal and the plane offset.  Horizon edges are matched by vertex ids, so
// the matching is exact where the reference compares coordinates within
// epsilon (epa.py:189-191).  The starting tetrahedron is wound with every
// normal pointing away from the opposite vertex and each new face inherits
// the winding of its horizon edge, which keeps the normals outward without
// the reference's sign test against the origin (epa.py:139-146), unreliable
// when the origin lies near a face.
//
// Convergence.  FP32 stops when the new support point is less than
// max(epsilon, 8 FLT_EPSILON max|y|) beyond the closest face (the FP32 noise
// floor in place of the reference's 1e-8).  The FP64 refinement re-evaluates
// the closest face's three vertices (support along the recorded directions,
// polytope vertices chosen by FP32 argmax and read in FP64), takes that face's
// FP64 unit normal n, evaluates the FP64 support point w along n and returns
// mtv = n (n . w), the reference's expression at convergence (epa.py:69).
//
// Visibility.  The faces that see a new point by more than the reference's
// epsilon are grown by flood fill from the closest face across shared edges
// (vertex ids), so the visible set is always connected.
//
// Validation.  Every expansion is checked: the horizon must be one closed
// loop (the visible faces a disk), no new face may be degenerate in FP32 and
// the loose-edge list must not overflow.  A pair that fails any check is
// appended to a fallback list and recomputed by the FP64 EPA (the
// reference's arithmetic), so FP32 noise on near-coplanar faces (cylinder
// caps, box faces) never leaves the polytope with holes.
//
// Status codes are those of the FP64 EPA.  Compiled with -fmad=true; the
// tests bound the depth error against the FP64 oracle.
#include "capi_util.h"
#include "epa_mixed.h"
#include "epa_mixed.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 128;

__global__ void __launch_bounds__(kBlock) k_epa_mixed(d3d_store st, const int32_t* __restrict__ i1,
                                                      const int32_t* __restrict__ i2, const int32_t* __restrict__ order,
                                                      int64_t n, unsigned long long* __restrict__ cursor,
                                                      const double* __restrict__ simplex, d3d_epa_options o,
                                                      double* __restrict__ mtv, int8_t* __restrict__ status,
                                                      int32_t* __restrict__ n_faces, double* __restrict__ faces,
                                                      char* __restrict__ scratch, int64_t slot_bytes,
                                                      int32_t* __restrict__ fallback,
                                                      unsigned long long* __restrict__ n_fallback) {
    const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const Slot s = slot_at(scratch + slot * slot_bytes, o);
    MixedEpa L;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true;
    while (true) {
        const long long k = fetch_slot(cursor, need);
        if (need) {
            if (k >= n) break;
            pid = order ? order[k] : k;
            a = i1[pid];
            b = i2[pid];
            if (!pair_ok(st, a, b)) {
                epa_store_bad_index(mtv, status, n_faces, pid);
                continue;  // the thread fetches again
            }
            mepa_begin(L, s, simplex + 12 * pid);
            need = false;
        }
        Col<float> c1, c2;
        load_col(st, a, c1);
        load_col(st, b, c2);
        const int stt = mepa_step(L, s, c1, c2, st, o);
        if (stt == kEpaFallback) {
            fallback[atomicAdd(n_fallback, 1ull)] = (int32_t)pid;
            need = true;
        } else if (stt >= 0) {
            d3 m = mk(double(NAN), double(NAN), double(NAN));
            if (stt == D3D_STATUS_OK || stt == D3D_STATUS_EPA_NOT_CONVERGED)
                m = mepa_refine(L, s, st, a, b, simplex + 12 * pid);
            mtv[3 * pid] = m.x;
            mtv[3 * pid + 1] = m.y;
            mtv[3 * pid + 2] = m.z;
            status[pid] = (int8_t)stt;
            const int nf = stt == D3D_STATUS_EPA_DEGENERATE ? 0 : L.nf;
            n_faces[pid] = nf;
            if (faces) {
                double* out = faces + pid * 12 * (int64_t)o.max_faces;
                for (int f = 0; f < nf; ++f) {
                    const int4 fi = s.fi[f];
                    const float4 fn = s.fn[f];
                    const int v[3] = {fi.x, fi.y, fi.z};
                    for (int j = 0; j < 3; ++j) {
                        const float4 y = s.vy[v[j]];
                        out[12 * f + 3 * j] = y.x;
                        out[12 * f + 3 * j + 1] = y.y;
                        out[12 * f + 3 * j + 2] = y.z;
                    }
                    out[12 * f + 9] = fn.x;
                    out[12 * f + 10] = fn.y;
                    out[12 * f + 11] = fn.z;
                }
            }
            need = true;
        }
    }
}

}  // namespace

namespace d3d {

int64_t epa_mixed_slot_bytes(const d3d_epa_options& o) {
    const int64_t b = 32 * (int64_t)(o.max_iterations + 4) + 36 * (int64_t)o.max_faces + 8 * (int64_t)o.max_loose_edges;
    return (b + 15) & ~int64_t(15);
}

int epa_mixed_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                     unsigned long long* cursor, const double* simplex, const d3d_epa_options& o, double* mtv,
                     int8_t* status, int32_t* n_faces, double* faces, void* scratch, int64_t max_slots,
                     int32_t* fallback, unsigned long long* n_fallback, cudaStream_t stream) {
    int blocks = persistent_blocks((const void*)k_epa_mixed, kBlock, n);
    if (blocks > max_slots / kBlock) blocks = (int)(max_slots / kBlock);
    k_epa_mixed<<<blocks, kBlock, 0, stream>>>(store, i1, i2, order, n, cursor, simplex, o, mtv, status, n_faces,
                                               faces, static_cast<char*>(scratch), epa_mixed_slot_bytes(o), fallback,
                                               n_fallback);
    return check_launch("d3d_epa (mixed)");
}

}  // namespace d3d
