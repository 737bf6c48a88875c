// gjk.cu -- the plain FP64 GJK drop-in: batched distance and intersection,
// one thread per pair.  Compiled with -fmad=false so that the arithmetic is
// the reference's rounding sequence (see d3d_device.cuh); the results are the
// reference's bit for bit.
#include "capi_util.h"
#include "gjk_impl.h"
#include "gjk_out.cuh"
#include "persist.cuh"
#include "scratch.h"
#include "jolt.cuh"

namespace {

using namespace d3d;

// slots a warp claims from the type-sorted order at a time
constexpr int kChunk = 32;


// Persistent FP64 GJK distance: each lane runs the reference's loop for one
// pair at a time (one iteration per round) and fetches the next pair, in the
// type-sorted `order`, when its pair ends.  `n_dev` (if not null) holds the
// pair count on the device (fallback lists of the mixed form).
// The register budget of 12 resident warps per SM (at most 168 registers a
// thread), which ptxas would otherwise trade for a few more registers.
template <int BLOCK>
constexpr int f64_min_blocks() { return BLOCK >= 384 ? 1 : 384 / BLOCK; }

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, f64_min_blocks<BLOCK>()) k_gjk_distance_f64(d3d_store s, const int32_t* __restrict__ i1,
                                                            const int32_t* __restrict__ i2,
                                                            const int32_t* __restrict__ order, int64_t n,
                                                            const unsigned long long* __restrict__ n_dev,
                                                            unsigned long long* __restrict__ cursor,
                                                            d3d_gjk_options opt, DistanceOut o) {
    __shared__ double rows[24 * BLOCK];  // the simplex P/Q rows of each lane
    if (n_dev) n = (int64_t)*n_dev;
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    GjkLoop<double, SmemRows<double, BLOCK>> g;
    g.S.R.base = rows + threadIdx.x;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true, bad = false;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // whole chunks to the end of the order: with long pairs, the lanes' coherence outweighs the slots
    // left in busy warps' chunks at the end (per-lane claims for the last slots measured slower)
    const long long split = n;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(cursor, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            bad = !pair_ok(s, a, b);
            simplex_clear(g.S);
            const d3 dir = mk(1.0, 0.0, 0.0);
            gjk_begin(g, dir, dot(dir, dir), DBL_MAX);
            need = false;
        }
        __syncwarp(live);  // the round starts converged (gjk_step keeps it so through the solve)
        if (bad) {  // out-of-range index: reported at once, no record read
            store_bad_index(o, pid);
            need = true;
        } else if (gjk_step<double>(g, s, a, b, tol_sq, opt.max_distance_squared, opt.max_iterations, E)) {
            GjkResult<double> r;
            gjk_end(g, opt.sanity_check, E, r);
            store_result(o, pid, r, g.S);
            need = true;
        }
    }
}

// The same loop with the simplex solves of a block regrouped by simplex
// size.  The lanes of a warp hold simplices of different sizes, and each
// size takes its own branch of closest_to_origin, so a warp ran the segment,
// triangle and tetrahedron code one after the other with a few lanes each,
// while FP64 instructions cost the pipe the same however few lanes are
// active.  Here every round, after the supports (gjk_step_begin), each lane
// with a simplex to solve writes its rows to shared memory at a place sorted
// by size (tetrahedra, triangles, segments, points); thread t of the block
// then solves the t-th simplex of that order, and each lane reads its result
// back for gjk_step_end.  The solve reads only the rows, the row count and
// prev, so it is the same arithmetic wherever it runs.  The block runs its
// rounds in step (two barriers per round), to the end of its last pair.
// Capped at 128 registers (a few hundred bytes spilled) for 16 warps per SM,
// which hide more of the barrier waits than 12 without spills: 47.5 -> 45.4
// ms at 1M pairs.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 512 / BLOCK) k_gjk_distance_f64_grouped(
    d3d_store s, const int32_t* __restrict__ i1, const int32_t* __restrict__ i2, const int32_t* __restrict__ order,
    int64_t n, const unsigned long long* __restrict__ n_dev, unsigned long long* __restrict__ cursor,
    d3d_gjk_options opt, DistanceOut o) {
    constexpr int W = BLOCK / 32;
    static_assert((BLOCK & (BLOCK - 1)) == 0, "the solve rotation masks with BLOCK - 1");
    constexpr unsigned kAll = 0xffffffffu;
    __shared__ double rows[24 * BLOCK];  // the simplex P/Q rows of each lane
    __shared__ double ty[12 * BLOCK];    // task t: row r, coordinate c at [(3 r + c) BLOCK + t]
    __shared__ double tprev[BLOCK];
    __shared__ double rv[4 * BLOCK];     // result of the lane that owns a task: v (3), v.v
    __shared__ int tmeta[BLOCK];         // task t: row count | owner << 8
    __shared__ int rset[BLOCK];          // owner's result: set | closer << 8
    __shared__ int cnt[4 * W];           // simplices per size class and warp
    if (n_dev) n = (int64_t)*n_dev;
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
    GjkLoop<double, SmemRows<double, BLOCK>> g;
    g.S.R.base = rows + threadIdx.x;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool have = false, exhausted = false, bad = false;
    WarpChunk chunk;
    // the sorted solves go to the warps by a rotation that changes every round and differs
    // between the blocks of an SM, so that the tetrahedra do not always fall on the same warp
    // slot and with it on one sub-partition's FP64 pipe
    int rot = (int)(((unsigned)blockIdx.x * (unsigned)W) / gridDim.x) % W;
    while (true) {
        rot = rot + 1 == W ? 0 : rot + 1;
        __syncwarp();
        const bool want = !have && !exhausted;
        const long long slot = fetch_slot_chunked(cursor, want, chunk, kAll, kChunk, n);
        if (want) {
            if (slot >= n) {
                exhausted = true;
            } else {
                pid = order ? order[slot] : slot;
                a = i1[pid];
                b = i2[pid];
                bad = !pair_ok(s, a, b);
                simplex_clear(g.S);
                const d3 dir = mk(1.0, 0.0, 0.0);
                gjk_begin(g, dir, dot(dir, dir), DBL_MAX);
                have = true;
            }
        }
        if (!__syncthreads_or(have)) break;
        bool solve = false;
        if (have) {
            if (bad) {  // out-of-range index: reported at once, no record read
                store_bad_index(o, pid);
                have = false;
            } else if (gjk_step_begin<double>(g, s, a, b, opt.max_distance_squared, opt.max_iterations)) {
                GjkResult<double> r;
                gjk_end(g, opt.sanity_check, E, r);
                store_result(o, pid, r, g.S);
                have = false;
            } else {
                solve = true;
            }
        }
        // the solve's place: size class (0 tetrahedron .. 3 point), then warp, then lane
        const int cls = solve ? 4 - g.S.n : 4;
        int rank = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const unsigned m = __ballot_sync(kAll, cls == c);
            if (cls == c) rank = __popc(m & ((1u << ln) - 1u));
            if (ln == 0) cnt[c * W + wp] = __popc(m);
        }
        __syncthreads();
        int t = 0, ntask = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const int k = cnt[c * W + w];
                if (c < cls || (c == cls && w < wp)) t += k;
                ntask += k;
            }
        t += rank;
        if (solve) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                ty[(3 * r) * BLOCK + t] = g.S.Y[r].x;
                ty[(3 * r + 1) * BLOCK + t] = g.S.Y[r].y;
                ty[(3 * r + 2) * BLOCK + t] = g.S.Y[r].z;
            }
            tprev[t] = g.prev;
            tmeta[t] = g.S.n | ((int)threadIdx.x << 8);
        }
        __syncthreads();
        const int u = (threadIdx.x + 32 * rot) & (BLOCK - 1);
        if (u < ntask) {
            Simplex<double> S;
            const int meta = tmeta[u];
            S.n = meta & 0xff;
#pragma unroll
            for (int r = 0; r < 4; ++r)
                S.Y[r] = mk(ty[(3 * r) * BLOCK + u], ty[(3 * r + 1) * BLOCK + u], ty[(3 * r + 2) * BLOCK + u]);
            d3 nv = mk(0.0, 0.0, 0.0);
            double nl = 0.0;
            int set = 0;
            const bool closer = closest_to_origin(S, tprev[u], E, nv, nl, set);
            const int owner = meta >> 8;
            rv[owner] = nv.x;
            rv[BLOCK + owner] = nv.y;
            rv[2 * BLOCK + owner] = nv.z;
            rv[3 * BLOCK + owner] = nl;
            rset[owner] = (set & 0xff) | (closer ? 256 : 0);
        }
        __syncthreads();
        if (solve) {
            const int x = rset[threadIdx.x];
            const d3 nv = mk(rv[threadIdx.x], rv[BLOCK + threadIdx.x], rv[2 * BLOCK + threadIdx.x]);
            if (gjk_step_end(g, tol_sq, E, (x & 256) != 0, nv, rv[3 * BLOCK + threadIdx.x], x & 0xff)) {
                GjkResult<double> r;
                gjk_end(g, opt.sanity_check, E, r);
                store_result(o, pid, r, g.S);
                have = false;
            }
        }
    }
}

// The same loop with the reference's MeshGraph vertex caching: the mesh
// supports of pair k start from mesh_cache[2k] (collider i1[k]) and
// mesh_cache[2k+1] (collider i2[k]), -1 meaning the mesh's start vertex, and
// leave there the vertex their last call returned, as the reference's support
// object keeps it (mesh.py:84-85).  One thread per pair, in input order;
// entries of non-mesh colliders pass through unchanged.
__global__ void __launch_bounds__(128) k_gjk_distance_f64_cached(d3d_store s, const int32_t* __restrict__ i1,
                                                                 const int32_t* __restrict__ i2, int64_t n,
                                                                 d3d_gjk_options opt, DistanceOut o,
                                                                 int32_t* __restrict__ mesh_cache) {
    __shared__ double rows[24 * 128];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int a = i1[k], b = i2[k];
    if (!pair_ok(s, a, b)) {
        store_bad_index(o, k);
        return;
    }
    const JoltEps<double> E = reference_eps<double>();
    GjkLoop<double, SmemRows<double, 128>> g;
    g.S.R.base = rows + threadIdx.x;
    simplex_clear(g.S);
    const d3 dir = mk(1.0, 0.0, 0.0);
    gjk_begin(g, dir, dot(dir, dir), DBL_MAX);
    int cache[2] = {mesh_cache[2 * k], mesh_cache[2 * k + 1]};
    const double tol_sq = opt.tolerance * opt.tolerance;
    while (!gjk_step<double>(g, s, a, b, tol_sq, opt.max_distance_squared, opt.max_iterations, E, 0.0, 0.0, cache)) {
    }
    GjkResult<double> r;
    gjk_end(g, opt.sanity_check, E, r);
    store_result(o, k, r, g.S);
    mesh_cache[2 * k] = cache[0];
    mesh_cache[2 * k + 1] = cache[1];
}

__global__ void __launch_bounds__(128) k_gjk_intersection_f64(d3d_store s, const int32_t* __restrict__ i1,
                                                              const int32_t* __restrict__ i2, int64_t n,
                                                              double tol_sq, int max_iter, int8_t* __restrict__ hit,
                                                              int8_t* __restrict__ status) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    JoltEps<double> E = reference_eps<double>();
    const int a = i1[k], b = i2[k];
    if (!pair_ok(s, a, b)) {
        hit[k] = 0;
        status[k] = (int8_t)D3D_STATUS_BAD_INDEX;
        return;
    }
    int st;
    hit[k] = (int8_t)gjk_intersection_loop(s, a, b, tol_sq, max_iter, E, st);
    status[k] = (int8_t)st;
}

}  // namespace

extern "C" int d3d_gjk_distance(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                                const d3d_gjk_options* options, double* dist, double* cp1, double* cp2,
                                double* simplex, int8_t* n_simplex, int8_t* status, int32_t* iterations,
                                void* stream) {
    int rc = d3d::check_store(store, "d3d_gjk_distance");
    if (rc) return rc;
    D3D_REQUIRE(options, "d3d_gjk_distance: null options");
    D3D_REQUIRE(n >= 0, "d3d_gjk_distance: n < 0");
    D3D_REQUIRE(options->max_iterations >= 1, "d3d_gjk_distance: max_iterations < 1");
    D3D_REQUIRE(options->precision == D3D_PRECISION_FP64 || options->precision == D3D_PRECISION_MIXED,
                "d3d_gjk_distance: unknown precision %d", options->precision);
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && dist && cp1 && cp2 && simplex && n_simplex && status,
                "d3d_gjk_distance: null pointer");
    if (options->precision == D3D_PRECISION_MIXED)
        return d3d::gjk_distance_mixed(*store, i1, i2, n, *options, dist, cp1, cp2, simplex, n_simplex, status,
                                       iterations, d3d::as_stream(stream));
    cudaStream_t st = d3d::as_stream(stream);
    void* block = nullptr;
    rc = d3d::scratch_alloc(&block, d3d::gjk_f64_scratch_bytes(n), st);
    if (rc) return rc;
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    rc = d3d::gjk_f64_run(*store, i1, i2, n, nullptr, *options, o, block, st);
    d3d::scratch_free(block, st);
    return rc;
}

namespace d3d {

size_t gjk_f64_scratch_bytes(int64_t capacity) {
    return 256 + ((sizeof(int32_t) * (size_t)capacity + 255) & ~size_t(255)) + pair_order_temp_bytes(capacity);
}

int gjk_f64_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const int64_t* n_dev,
                const d3d_gjk_options& opt, const DistanceOut& o, void* scratch, cudaStream_t stream) {
    const bool sched = n >= tuning().sort_min;
    unsigned long long* cursor = static_cast<unsigned long long*>(scratch);
    int32_t* order = sched ? reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + 256) : nullptr;
    const size_t order_bytes = (sizeof(int32_t) * (size_t)n + 255) & ~size_t(255);
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) {
        set_error("d3d_gjk_distance: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    int rc = D3D_SUCCESS;
    if (sched)
        rc = pair_order(store, i1, i2, n, order, static_cast<char*>(scratch) + 256 + order_bytes,
                        pair_order_temp_bytes(n), stream, n_dev);
    if (!rc)
        rc = launch_gjk_f64(store, i1, i2, order, n, reinterpret_cast<const unsigned long long*>(n_dev), cursor,
                            opt, o, stream);
    return rc;
}

int launch_gjk_f64(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const d3d_gjk_options& opt,
                   const DistanceOut& o, cudaStream_t stream) {
    const d3d_tuning t = tuning();
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 32LL * sms) {
        // A small batch: one warp per block, so that the pairs spread over
        // as many SMs as they fill warps.  An FP64 instruction costs an SM's
        // FP64 pipe the same however few lanes are active, so fewer warps
        // per SM finish each round sooner (1,000 pairs: 32 SMs instead of 8).
        const int blocks = (int)((n + 31) / 32);
        k_gjk_distance_f64<32><<<blocks > 0 ? blocks : 1, 32, 0, stream>>>(store, i1, i2, order, n, n_dev, cursor,
                                                                           opt, o);
    } else if (t.gjk_block == 64) {
        const void* k = (const void*)k_gjk_distance_f64_grouped<64>;
        const int blocks = persistent_blocks(k, 64, n, blocks_per_sm(t, 64));
        k_gjk_distance_f64_grouped<64><<<blocks, 64, 0, stream>>>(store, i1, i2, order, n, n_dev, cursor, opt, o);
    } else {
        // 128-thread blocks for gjk_block 128 and 256: the block's solves regrouped by simplex size
        // pay more than the launch shape (at 1M pairs, 256-thread blocks without the regrouping took
        // 56.7 ms, 128-thread grouped blocks 44.8 ms), and an autotuning of the mixed form, which
        // may pick 256, applies to this kernel as well
        const void* k = (const void*)k_gjk_distance_f64_grouped<128>;
        const int blocks = persistent_blocks(k, 128, n, blocks_per_sm(t, 128));
        k_gjk_distance_f64_grouped<128><<<blocks, 128, 0, stream>>>(store, i1, i2, order, n, n_dev, cursor, opt, o);
    }
    return check_launch("d3d_gjk_distance");
}

}  // namespace d3d

extern "C" int d3d_gjk_distance_cached(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                                       const d3d_gjk_options* options, int32_t* mesh_cache, double* dist,
                                       double* cp1, double* cp2, double* simplex, int8_t* n_simplex, int8_t* status,
                                       int32_t* iterations, void* stream) {
    int rc = d3d::check_store(store, "d3d_gjk_distance_cached");
    if (rc) return rc;
    D3D_REQUIRE(options, "d3d_gjk_distance_cached: null options");
    D3D_REQUIRE(n >= 0, "d3d_gjk_distance_cached: n < 0");
    D3D_REQUIRE(options->max_iterations >= 1, "d3d_gjk_distance_cached: max_iterations < 1");
    D3D_REQUIRE(options->precision == D3D_PRECISION_FP64,
                "d3d_gjk_distance_cached: the vertex cache is the reference's; only the FP64 form takes it");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && mesh_cache && dist && cp1 && cp2 && simplex && n_simplex && status,
                "d3d_gjk_distance_cached: null pointer");
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    k_gjk_distance_f64_cached<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(*store, i1, i2, n,
                                                                                          *options, o, mesh_cache);
    return d3d::check_launch("d3d_gjk_distance_cached");
}

extern "C" int d3d_gjk_intersection(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                                    double tolerance, int32_t max_iterations, int8_t* hit, int8_t* status,
                                    void* stream) {
    int rc = d3d::check_store(store, "d3d_gjk_intersection");
    if (rc) return rc;
    D3D_REQUIRE(n >= 0, "d3d_gjk_intersection: n < 0");
    D3D_REQUIRE(max_iterations >= 1, "d3d_gjk_intersection: max_iterations < 1");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && hit && status, "d3d_gjk_intersection: null pointer");
    k_gjk_intersection_f64<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(
        *store, i1, i2, n, tolerance * tolerance, max_iterations, hit, status);
    return d3d::check_launch("d3d_gjk_intersection");
}
