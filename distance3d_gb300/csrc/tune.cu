// tune.cu -- autotuner of the batch kernels' launch parameters.
//
// d3d_autotune times d3d_collide (GJK distance, EPA on the intersecting
// pairs) on the caller's sample pairs for candidate tunings and keeps the
// fastest:
//
//   stage 1  GJK threads per block {64, 128, 256} x resident warps per SM
//            {all that fit, 16} x type sorting {as set, never}, with the EPA
//            setting unchanged
//   stage 2  warp-EPA pairs per block {2, 4, 8} with the stage-1 winner
//
// Each candidate runs once untimed, then three timed samples of 1-16 runs
// (CUDA events on the caller's stream); the fastest sample counts.  The result is process
// state (d3d_set_tuning), read by every later launch.
#include <climits>
#include <cmath>
#include <vector>

#include "capi_util.h"
#include "scratch.h"

namespace {

struct Buffers {
    void* p[12] = {};
    size_t scratch_bytes = 0;
    ~Buffers() {
        for (void* q : p) cudaFree(q);
    }
};

int run(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n, const d3d_gjk_options* gjk,
        const d3d_epa_options* epa, Buffers& b, cudaStream_t st) {
    return d3d_collide(store, i1, i2, n, static_cast<int64_t*>(b.p[0]), gjk, epa, (double*)b.p[1], (double*)b.p[2],
                       (double*)b.p[3], (double*)b.p[4], (int8_t*)b.p[5], (int8_t*)b.p[6], (int32_t*)b.p[7],
                       (double*)b.p[8], (int8_t*)b.p[9], (int32_t*)b.p[10], b.p[11], b.scratch_bytes, st);
}

// milliseconds per run (the fastest of three timed samples, each sample
// repeating the run until it spans about 2 ms, so that small batches are not
// timed at the events' resolution), or a negative code
float time_tuning(const d3d_tuning& t, const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                  const d3d_gjk_options* gjk, const d3d_epa_options* epa, Buffers& b, cudaStream_t st,
                  cudaEvent_t e0, cudaEvent_t e1, int* rc) {
    *rc = d3d_set_tuning(&t);
    if (*rc) return -1.f;
    int reps = 1;
    float best = -1.f;
    for (int k = 0; k < 4 && !*rc; ++k) {  // sample 0: warm-up and estimate
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps && !*rc; ++r) *rc = run(store, i1, i2, n, gjk, epa, b, st);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            *rc = D3D_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (k == 0) {
            reps = ms > 0.f ? (int)ceilf(2.f / ms) : 16;
            reps = reps < 1 ? 1 : (reps > 16 ? 16 : reps);
            continue;
        }
        ms /= (float)reps;
        if (best < 0.f || ms < best) best = ms;
    }
    return best;
}

}  // namespace

extern "C" int d3d_autotune(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                            const d3d_gjk_options* gjk, const d3d_epa_options* epa, d3d_tuning* out, void* stream) {
    int rc = d3d::check_store(store, "d3d_autotune");
    if (rc) return rc;
    D3D_REQUIRE(gjk && epa && out && i1 && i2 && n > 0 && n <= INT32_MAX, "d3d_autotune: invalid argument");
    cudaStream_t st = d3d::as_stream(stream);
    const size_t bytes[11] = {8, 8, 24, 24, 96, 1, 1, 4, 24, 1, 4};
    Buffers b;
    b.scratch_bytes = d3d_collide_scratch_bytes(n, gjk, epa);
    D3D_REQUIRE(b.scratch_bytes > 0, "d3d_autotune: invalid options");
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 11 && e == cudaSuccess; ++k) e = cudaMalloc(&b.p[k], bytes[k] * (k == 0 ? 1 : (size_t)n));
    if (e == cudaSuccess) e = cudaMalloc(&b.p[11], b.scratch_bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.p[0], &n, sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_autotune: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const d3d_tuning start = d3d::tuning();
    d3d_tuning best = start;
    float best_ms = -1.f;
    // stage 1: the GJK kernels
    const int blocks[3] = {64, 128, 256};
    const int warps[2] = {0, 16};
    const int sorts[2] = {start.sort_min, INT_MAX};
    for (int bl : blocks)
        for (int w : warps)
            for (int so : sorts) {
                d3d_tuning t = start;
                t.gjk_block = bl;
                t.gjk_warps_per_sm = w;
                t.sort_min = so;
                const float ms = time_tuning(t, store, i1, i2, n, gjk, epa, b, st, e0, e1, &rc);
                if (rc) break;
                if (best_ms < 0.f || ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
    // stage 2: the warp EPA
    const int epa_warps[3] = {2, 4, 8};
    for (int k = 0; k < 3 && !rc; ++k) {
        d3d_tuning t = best;
        t.epa_warps = epa_warps[k];
        const float ms = time_tuning(t, store, i1, i2, n, gjk, epa, b, st, e0, e1, &rc);
        if (rc) break;
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        d3d_set_tuning(&start);
        return rc;
    }
    d3d_set_tuning(&best);
    *out = best;
    return D3D_SUCCESS;
}
