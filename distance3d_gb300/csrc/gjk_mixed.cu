// gjk_mixed.cu -- mixed-precision GJK distance.
//
// Five kernels over the type-sorted pair order:
//
// A  runs the Jolt loop in FP32 on the FP32 mirror of the store, with
//    thresholds scaled to single precision, hands each pair's outcome, final
//    closest point and the search direction of each final simplex row on
//    (80 bytes/pair) and appends clipped and unconverged pairs to the
//    fallback list.
// R  (the refinement pass) takes one warp per 32 consecutive slots of the
//    type-sorted order, so that a warp's lanes evaluate the same supports.
//    Each lane re-evaluates its pair's final simplex rows in FP64 along their
//    FP32 directions (polytope supports choose their vertex by an FP32 argmax
//    and return the FP64 vertex) and, for a separated pair, one more support
//    pair along -v, the closest point A ended on.  A separated pair whose
//    origin projection lies inside its FP64 feature and whose duality gap
//    brackets the distance within 1e-6 of itself (or 1e-9 of the scene's
//    scale) is done there, closest points from the projection's barycentric
//    coordinates; so is a touching pair whose FP64 tetrahedron encloses the
//    origin.  Every other separated or touching pair is flagged, its FP64 rows
//    in its record, and a stable compaction (CUB) lists the flagged pairs in
//    the type-sorted order.
// B  continues the reference's loop in FP64 for the listed pairs, one round
//    per lane and iteration (pb_round): the first round solves the handed
//    rows, later rounds add a support pair along -v, until the duality gap
//    closes as in R.  A pair whose loop ends leaves its simplex in the outputs
//    and the rest of its state in its record.
// E  (the end pass) computes the closest points and the checks of B's
//    finished pairs (pb_end), every lane on a finished pair.
// C  is the plain FP64 kernel over the fallback list (the reference's
//    arithmetic; CLIPPED and MAX_ITER keep their FP64 meaning).
//
// FP64 instructions cost the GB300's FP64 pipe the same however few lanes of
// a warp are active, so the FP64 work sits where lanes are busy: R runs the
// same support code on every lane of a warp and a short per-lane solve, and
// only the pairs R cannot finish (those whose gap or feature check fails)
// pay for B's divergent per-lane loop.  B keeps the simplex P/Q rows in
// shared memory and has one support call site.  A pair goes to the fallback
// list only if its result fails the consistency check (closest points vs |v|)
// or the sanity check in E, or hits the iteration bound in B.
//
// On the six-type workloads A takes ~11 FP32 iterations and R evaluates ~3
// rows plus the gap row, against ~17-19 FP64 iterations for the plain form.
// Compiled with -fmad=true: the tests bound its error against the FP64
// oracle.
#include <cub/cub.cuh>

#include "capi_util.h"
#include "gjk_impl.h"
#include "gjk_mixed.cuh"
#include "gjk_out.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;


// Per-call counters (one 256-byte block): cursors of A, B and C, then the
// lengths of the fallback, finished and run lists.
enum { kCurA = 0, kCurB, kCurC, kNumFallback, kNumEnd, kNumRun, kCounters };

struct Lists {
    int32_t* fallback;
    int32_t* ends;         // pairs whose FP64 loop ended in B, for the end pass
    EndRecord* records;    // by pair: R's FP64 rows for B, B's end state for E
    int8_t* run_flag;      // by slot of the order: R left the pair to B
    int32_t* run_pid;      // by slot of the order: the pair
    int32_t* run;          // the flagged pairs in the order (B's work list)
    unsigned long long* ctr;
};

// slots a warp claims from the type-sorted order at a time
constexpr int kChunk = 32;

// Phase A's register budget: 16 resident warps per SM (128 registers), its
// simplex P/Q rows in shared memory (ARows).  At 1M pairs: 3.9 ms for the
// mixed GJK, against 4.2 with 12 warps and the rows in registers, 4.2 with 20
// warps and 4.9 with 24 (more spilled registers).
template <int BLOCK>
constexpr int phase_a_min_blocks() { return 512 / BLOCK; }

template <int BLOCK, bool MESH>
__global__ void __launch_bounds__(BLOCK, phase_a_min_blocks<BLOCK>()) k_gjk_mixed_a(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t n,
                                                        const int64_t* __restrict__ n_dev, float tol_sq,
                                                        float max_d2, int max_iter, Handoff* __restrict__ hand,
                                                        DistanceOut out, Lists lists) {
    if (n_dev) n = *n_dev;
    __shared__ float4 arows[4 * BLOCK];
    PhaseALoop<ARows<BLOCK>> L;
    L.S.R.base = arows + threadIdx.x;
    int64_t pid = 0;
    int a = 0, b = 0;
    bool need = true, bad = false;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // per-lane claims for the last slots: the pairs are short, and slots left in a busy warp's chunk
    // would hold up the end of the launch
    const long long split = n - 2LL * gridDim.x * blockDim.x;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(lists.ctr + kCurA, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            pid = order ? order[slot] : slot;
            a = i1[pid];
            b = i2[pid];
            bad = !pair_ok(s, a, b);
            pa_begin(L);
            need = false;
        }
        __syncwarp(live);  // the round starts converged (pa_step keeps it so through the solve)
        // a pair with an out-of-range index ends at once; R skips it (its outcome is neither
        // separated nor touching) and it joins no list
        const int o = bad ? PA_BAD_INDEX : pa_step<MESH>(L, s, a, b, tol_sq, max_d2, max_iter);
        const bool done = o >= 0;
        if (done) {
            hand[pid] = pa_handoff(L, o);
            if (bad) store_bad_index(out, pid);
        }
        append_lanes(live, lists.fallback, lists.ctr + kNumFallback, done && (o == PA_CLIPPED || o == PA_FAILED),
                     (int32_t)pid);
        need = done;
    }
}

// R's checks and outputs for one pair, its FP64 rows at my[(6 j + e) BLOCK]
// (the rows of separated pairs end with the gap row).  Run by the thread the
// block's regrouping gave the pair, which may not be the one that read it.
template <int BLOCK>
__device__ __forceinline__ void r_finish(const double* my, int nr, bool sep, bool touch, float4 v, int it_a,
                                         int32_t pid, int64_t slot, const d3d_gjk_options& opt, const DistanceOut& o,
                                         const Lists& lists) {
    const bool rows_ok = sep || touch;
    auto row_p = [&](int j) { return mk(my[(6 * j) * BLOCK], my[(6 * j + 1) * BLOCK], my[(6 * j + 2) * BLOCK]); };
    auto row_q = [&](int j) {
        return mk(my[(6 * j + 3) * BLOCK], my[(6 * j + 4) * BLOCK], my[(6 * j + 5) * BLOCK]);
    };
    bool done = false;
    d3 cp1 = mk(0.0, 0.0, 0.0), cp2 = cp1;
    double dist = 0.0;
    d3 w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = (j < nr && rows_ok) ? row_p(j) - row_q(j) : mk(0.0, 0.0, 0.0);
    if (sep) {
        d3 vv;
        double lam[3];
        const bool inside = feature_point(w, nr, vv, lam);
        const double vl = dot(vv, vv);
        const d3 wg = row_p(nr) - row_q(nr);
        const d3 u = mk((double)v.x, (double)v.y, (double)v.z);
        // distance in [u.wg / |u|, |vv|] (wg is the support of the Minkowski difference along -u)
        const double upper = sqrt(vl);
        const double lower = dot(u, wg) / sqrt(dot(u, u));
        const double gap = upper - lower;
        double ymax = dot(w[0], w[0]);
#pragma unroll
        for (int j = 1; j < 3; ++j)
            if (j < nr) ymax = maxf2(ymax, dot(w[j], w[j]));
        const double tol_sq = opt.tolerance * opt.tolerance;
        // touching in FP64 (pb_round's test) is B's to decide
        const bool apart = vl > tol_sq && vl > DBL_EPSILON * ymax;
        const bool closed = gap <= kMixedRelGap * upper || gap * gap <= kMixedAbsGap2 * maxf2(1.0, dot(wg, wg));
        if (inside && apart && closed) {
            cp1 = row_p(0) * lam[0];
            cp2 = row_q(0) * lam[0];
#pragma unroll
            for (int j = 1; j < 3; ++j) {
                if (j < nr) {
                    cp1 = cp1 + row_p(j) * lam[j];
                    cp2 = cp2 + row_q(j) * lam[j];
                }
            }
            dist = upper;
            const d3 ab = cp1 - cp2;
            // pb_end's consistency check
            done = abs_t(sqrt(dot(ab, ab)) - dist) <= 1e-10 * maxf2(dist, 1.0);
        }
    } else if (touch) {
        if (outside_planes(w[0], w[1], w[2], w[3], reference_eps<double>()) == 0) {
            // the origin inside the FP64 tetrahedron: closest points as gjk_end takes them
            // (bary_tetra, then merged at distance 0)
            double o4[4];
            bary_tetra(w[0], w[1], w[2], w[3], o4);
            const d3 pa = ((row_p(0) * o4[0] + row_p(1) * o4[1]) + row_p(2) * o4[2]) + row_p(3) * o4[3];
            const d3 pb = ((row_q(0) * o4[0] + row_q(1) * o4[1]) + row_q(2) * o4[2]) + row_q(3) * o4[3];
            cp1 = cp2 = (pa + pb) * 0.5;
            done = true;
        }
    }
    if (done) {
        o.dist[pid] = dist;
        o.cp1[3 * (int64_t)pid] = cp1.x;
        o.cp1[3 * (int64_t)pid + 1] = cp1.y;
        o.cp1[3 * (int64_t)pid + 2] = cp1.z;
        o.cp2[3 * (int64_t)pid] = cp2.x;
        o.cp2[3 * (int64_t)pid + 1] = cp2.y;
        o.cp2[3 * (int64_t)pid + 2] = cp2.z;
        double* sp = o.simplex + 12 * (int64_t)pid;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sp[3 * j] = w[j].x;
            sp[3 * j + 1] = w[j].y;
            sp[3 * j + 2] = w[j].z;
        }
        o.n_simplex[pid] = (int8_t)nr;
        o.status[pid] = (int8_t)D3D_STATUS_OK;
        // the gap row counts as the FP64 iteration that closed the bracket
        if (o.iterations) o.iterations[pid] = it_a + (sep ? 1 : 0);
    } else {
        EndRecord& e = lists.records[pid];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j < nr && rows_ok) {
                const d3 p = row_p(j), q = row_q(j);
                e.pq[j][0] = p.x;
                e.pq[j][1] = p.y;
                e.pq[j][2] = p.z;
                e.pq[j][3] = q.x;
                e.pq[j][4] = q.y;
                e.pq[j][5] = q.z;
            }
        }
        e.n = rows_ok ? nr : 0;
    }
    lists.run_flag[slot] = (int8_t)(!done);
    lists.run_pid[slot] = pid;
}

// R, one lane per slot of the order (see the top of this file).  The grid
// covers the capacity; slots at and beyond the pair count are flagged 0.
// Each lane evaluates its pair's FP64 rows; the checks that follow run in
// different branches for touching pairs and for separated pairs of one, two
// and three rows, so the block regroups them: the pairs are sorted by that
// class (counting sort over the block, the rows staying where they are in
// shared memory) and thread t runs the t-th pair's checks (r_finish).
template <int BLOCK, bool MESH>
__global__ void __launch_bounds__(BLOCK) k_gjk_mixed_r(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2,
                                                        const int32_t* __restrict__ order, int64_t cap,
                                                        const int64_t* __restrict__ n_dev, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o, Lists lists) {
    constexpr int W = BLOCK / 32;
    constexpr unsigned kAll = 0xffffffffu;
    // p and q of up to five rows per lane: element e of row j at [(6 j + e) BLOCK]
    __shared__ double rows[30 * BLOCK];
    __shared__ float4 tv[BLOCK];       // the handoff's v of each lane's pair
    __shared__ int tpid[BLOCK], tita[BLOCK], tcls[BLOCK];
    __shared__ unsigned short tperm[BLOCK];
    __shared__ int cnt[4 * W];
    const int64_t n = n_dev ? *n_dev : cap;
    const int64_t slot = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
    const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
    int32_t pid = 0;
    int outcome = PA_FAILED, nr = 0, it_a = 0;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (slot < n && slot < cap) {
        pid = order ? order[slot] : (int32_t)slot;
        v = hand[pid].v;
        outcome = __float_as_int(v.w) & 0xff;
        nr = (__float_as_int(v.w) >> 8) & 0xff;
        it_a = handoff_iters(v);
    }
    const bool mine = outcome == PA_SEPARATED || outcome == PA_TOUCHING;  // R or B finishes it
    const bool rows_ok = mine && nr >= 1 && nr <= 4;
    const bool sep = rows_ok && outcome == PA_SEPARATED && nr <= 3;
    const bool touch = rows_ok && outcome == PA_TOUCHING && nr == 4;
    int a = 0, b = 0;
    if (rows_ok) {
        a = i1[pid];
        b = i2[pid];
    }
    // the rows in FP64, then the gap row of a separated pair along -v
    const int count = rows_ok ? nr + (sep ? 1 : 0) : 0;
    double* my = rows + threadIdx.x;
#pragma unroll 1
    for (int j = 0; j < 5; ++j) {
        if (j < count) {
            d3 d;
            float4 f = make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));  // the gap row: no vertices known
            if (j < nr) {
                f = hand[pid].d[j];
                d = mk((double)f.x, (double)f.y, (double)f.z);
            } else {
                d = mk(-(double)v.x, -(double)v.y, -(double)v.z);
            }
            // the polytope vertices phase A took along this row's direction are read, not searched again
            d3 p, q;
#pragma unroll 1
            for (int k = 0; k < 2; ++k) {
                Col<double> c;
                load_col(s, k ? b : a, c);
                const d3 x = RefineSupportT<MESH>::eval_at(c, s, k ? -d : d, handoff_vertex(f, k));
                if (k)
                    q = x;
                else
                    p = x;
            }
            my[(6 * j + 0) * BLOCK] = p.x;
            my[(6 * j + 1) * BLOCK] = p.y;
            my[(6 * j + 2) * BLOCK] = p.z;
            my[(6 * j + 3) * BLOCK] = q.x;
            my[(6 * j + 4) * BLOCK] = q.y;
            my[(6 * j + 5) * BLOCK] = q.z;
        }
    }
    // class of the checks: 0 touching (four rows), 1-3 separated with that many rows, 4 none
    const int cls = touch ? 0 : (sep ? nr : 4);
    if (cls == 4 && slot < cap) {
        // a pair R does not check goes to B as it is (rows of a pair of another shape are kept), or
        // is not R's at all
        if (mine) {
            EndRecord& e = lists.records[pid];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j < nr && rows_ok) {
                    e.pq[j][0] = my[(6 * j) * BLOCK];
                    e.pq[j][1] = my[(6 * j + 1) * BLOCK];
                    e.pq[j][2] = my[(6 * j + 2) * BLOCK];
                    e.pq[j][3] = my[(6 * j + 3) * BLOCK];
                    e.pq[j][4] = my[(6 * j + 4) * BLOCK];
                    e.pq[j][5] = my[(6 * j + 5) * BLOCK];
                }
            }
            e.n = rows_ok ? nr : 0;
        }
        lists.run_flag[slot] = (int8_t)mine;
        lists.run_pid[slot] = pid;
    }
    tv[threadIdx.x] = v;
    tpid[threadIdx.x] = pid;
    tita[threadIdx.x] = it_a;
    tcls[threadIdx.x] = cls | (nr << 8);
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
    if (cls < 4) tperm[t + rank] = (unsigned short)threadIdx.x;
    __syncthreads();
    if ((int)threadIdx.x < ntask) {
        const int owner = tperm[threadIdx.x];
        const int x = tcls[owner];
        const int c = x & 0xff, rn = x >> 8;
        r_finish<BLOCK>(rows + owner, rn, c >= 1, c == 0, tv[owner], tita[owner], tpid[owner],
                        (int64_t)blockIdx.x * BLOCK + owner, opt, o, lists);
    }
}

// B over R's run list, in the type-sorted order.
template <int BLOCK, bool MESH>
__global__ void __launch_bounds__(BLOCK) k_gjk_mixed_b(d3d_store s, const int32_t* __restrict__ i1,
                                                        const int32_t* __restrict__ i2, d3d_gjk_options opt,
                                                        const Handoff* __restrict__ hand, DistanceOut o, Lists lists) {
    __shared__ double rows[24 * BLOCK];
    const int64_t n = (int64_t)lists.ctr[kNumRun];
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    PhaseB<SmemRows<double, BLOCK>> B;
    B.g.S.R.base = rows + threadIdx.x;
    int32_t pid = 0;
    int a = 0, b = 0;
    int it_a = 0;
    bool need = true;
    unsigned live = __activemask();  // the warp's lanes still in the loop
    WarpChunk chunk;
    // per-lane claims for the last slots: the pairs are short, and slots left in a busy warp's chunk
    // would hold up the end of the launch
    const long long split = n - 2LL * gridDim.x * blockDim.x;
    while (true) {
        __syncwarp(live);
        const long long slot = fetch_slot_chunked(lists.ctr + kCurB, need, chunk, live, kChunk, split);
        const bool quit = need && slot >= n;
        live = __ballot_sync(live, !quit);
        if (quit) break;
        if (need) {
            pid = lists.run[slot];
            a = i1[pid];
            b = i2[pid];
            it_a = handoff_iters(hand[pid].v);
            pb_begin(B, lists.records[pid]);
            need = false;
        }
        __syncwarp(live);  // the round starts converged (pb_round keeps it so through the solve)
        if (B.mode == PB_FALLBACK || pb_round<MESH>(B, s, a, b, tol_sq, opt, E)) {
            if (B.mode != PB_FALLBACK) {
                // The closest points and checks of the pair (pb_end) run in
                // the end pass, where a warp's lanes all hold finished pairs;
                // here only a few lanes finish per round.
                const GjkLoop<double, SmemRows<double, BLOCK>>& g = B.g;
                EndRecord& e = lists.records[pid];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < g.S.n) {
                        const d3 pk = g.S.R.p(k), qk = g.S.R.q(k);
                        e.pq[k][0] = pk.x;
                        e.pq[k][1] = pk.y;
                        e.pq[k][2] = pk.z;
                        e.pq[k][3] = qk.x;
                        e.pq[k][4] = qk.y;
                        e.pq[k][5] = qk.z;
                    }
                }
                e.dir[0] = g.dir.x;
                e.dir[1] = g.dir.y;
                e.dir[2] = g.dir.z;
                e.vl = g.vl;
                e.it = g.it + it_a;
                e.state = g.state;
                e.status = g.status;
                e.n = g.S.n;
                double* sp = o.simplex + 12 * (int64_t)pid;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    sp[3 * j] = g.S.Y[j].x;
                    sp[3 * j + 1] = g.S.Y[j].y;
                    sp[3 * j + 2] = g.S.Y[j].z;
                }
                o.n_simplex[pid] = (int8_t)g.S.n;
                append_warp(lists.ends, lists.ctr + kNumEnd, true, pid);
            } else {
                lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
            }
            need = true;
        }
    }
}

// The end pass over B's finished pairs: closest points, sanity and
// consistency checks (pb_end) and the outputs; pairs failing a check go to
// the fallback list.
__global__ void __launch_bounds__(128) k_gjk_mixed_end(d3d_gjk_options opt, DistanceOut o, Lists lists) {
    const int64_t n = (int64_t)lists.ctr[kNumEnd];
    const JoltEps<double> E = reference_eps<double>();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t pid = lists.ends[k];
        const EndRecord& e = lists.records[pid];
        GjkLoop<double, RegRows<double>> g;
        g.S.n = e.n;
        const double* sp = o.simplex + 12 * (int64_t)pid;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            g.S.Y[j] = mk(sp[3 * j], sp[3 * j + 1], sp[3 * j + 2]);
            if (j < e.n)
                g.S.R.put(j, mk(e.pq[j][0], e.pq[j][1], e.pq[j][2]), mk(e.pq[j][3], e.pq[j][4], e.pq[j][5]));
        }
        g.dir = mk(e.dir[0], e.dir[1], e.dir[2]);
        g.vl = e.vl;
        g.prev = 0.0;
        g.it = e.it;
        g.state = e.state;
        g.status = e.status;
        GjkResult<double> r;
        if (pb_end(g, opt, E, r) == PB_DONE) {
            o.dist[pid] = r.dist;
            o.cp1[3 * (int64_t)pid] = r.a.x;
            o.cp1[3 * (int64_t)pid + 1] = r.a.y;
            o.cp1[3 * (int64_t)pid + 2] = r.a.z;
            o.cp2[3 * (int64_t)pid] = r.b.x;
            o.cp2[3 * (int64_t)pid + 1] = r.b.y;
            o.cp2[3 * (int64_t)pid + 2] = r.b.z;
            o.status[pid] = (int8_t)r.status;
            if (o.iterations) o.iterations[pid] = r.iters;
        } else {
            lists.fallback[atomicAdd(lists.ctr + kNumFallback, 1ull)] = pid;
        }
    }
}

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

namespace d3d {

// temporary storage of the run list's stable compaction (CUB) over n slots
size_t select_temp_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceSelect::Flagged(nullptr, b, static_cast<const int32_t*>(nullptr), static_cast<const int8_t*>(nullptr),
                               static_cast<int32_t*>(nullptr), static_cast<unsigned long long*>(nullptr), (int)n);
    return up(b);
}

size_t gjk_mixed_scratch_bytes(int64_t capacity) {
    const size_t c = (size_t)capacity;
    return 256 + up(sizeof(int32_t) * c) + pair_order_temp_bytes(capacity) + up(sizeof(Handoff) * c) +
           2 * up(sizeof(int32_t) * c) + up(sizeof(EndRecord) * c) + up(c) + 2 * up(sizeof(int32_t) * c) +
           select_temp_bytes(capacity);
}

// R's block: 30 doubles of shared memory per lane
constexpr int kRefineBlock = 128;

template <int BLOCK, bool MESH>
int launch_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                 const int64_t* n_dev, const d3d_gjk_options& opt, Handoff* hand, const DistanceOut& o,
                 const Lists& lists, void* select_temp, size_t select_bytes, int per_sm, cudaStream_t stream) {
    const float tol_sq = (float)(opt.tolerance * opt.tolerance);
    const void* ka = (const void*)k_gjk_mixed_a<BLOCK, MESH>;
    k_gjk_mixed_a<BLOCK, MESH><<<persistent_blocks(ka, BLOCK, n, per_sm), BLOCK, 0, stream>>>(
        store, i1, i2, order, n, n_dev, tol_sq, (float)opt.max_distance_squared, opt.max_iterations, hand, o,
        lists);
    int rc = check_launch("d3d_gjk_distance (mixed, FP32 phase)");
    if (rc) return rc;
    k_gjk_mixed_r<kRefineBlock, MESH><<<grid_for(n, kRefineBlock), kRefineBlock, 0, stream>>>(
        store, i1, i2, order, n, n_dev, opt, hand, o, lists);
    rc = check_launch("d3d_gjk_distance (mixed, refinement pass)");
    if (rc) return rc;
    // the flagged pairs, in the order of the slots
    cudaError_t e = cub::DeviceSelect::Flagged(select_temp, select_bytes, lists.run_pid, lists.run_flag, lists.run,
                                               lists.ctr + kNumRun, (int)n, stream);
    if (e != cudaSuccess) {
        set_error("d3d_gjk_distance (mixed, run list): %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    const void* kb = (const void*)k_gjk_mixed_b<BLOCK, MESH>;
    k_gjk_mixed_b<BLOCK, MESH><<<persistent_blocks(kb, BLOCK, n, per_sm), BLOCK, 0, stream>>>(store, i1, i2, opt,
                                                                                             hand, o, lists);
    rc = check_launch("d3d_gjk_distance (mixed, FP64 loop)");
    if (rc) return rc;
    k_gjk_mixed_end<<<persistent_blocks((const void*)k_gjk_mixed_end, 128, n), 128, 0, stream>>>(opt, o, lists);
    return check_launch("d3d_gjk_distance (mixed, end pass)");
}

// The kernels without the MeshGraph branch serve stores without meshes.
template <int BLOCK>
int launch_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* order, int64_t n,
                 const int64_t* n_dev, const d3d_gjk_options& opt, Handoff* hand, const DistanceOut& o,
                 const Lists& lists, void* select_temp, size_t select_bytes, int per_sm, cudaStream_t stream) {
    if (store.n_links > 0)
        return launch_mixed<BLOCK, true>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, select_temp,
                                         select_bytes, per_sm, stream);
    return launch_mixed<BLOCK, false>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, select_temp, select_bytes,
                                      per_sm, stream);
}

int gjk_mixed_run(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n, const int64_t* n_dev,
                  const d3d_gjk_options& opt, const DistanceOut& o, void* scratch, cudaStream_t stream) {
    const d3d_tuning t = tuning();
    const bool sched = n >= t.sort_min;
    const size_t c = (size_t)n;
    const size_t order_bytes = up(sizeof(int32_t) * c);
    const size_t temp_bytes = pair_order_temp_bytes(n);
    char* p = static_cast<char*>(scratch);
    Lists lists;
    lists.ctr = reinterpret_cast<unsigned long long*>(p);
    p += 256;
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p) : nullptr;
    p += order_bytes;
    void* temp = p;
    p += temp_bytes;
    Handoff* hand = reinterpret_cast<Handoff*>(p);
    p += up(sizeof(Handoff) * c);
    lists.fallback = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * c);
    lists.ends = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * c);
    lists.records = reinterpret_cast<EndRecord*>(p);
    p += up(sizeof(EndRecord) * c);
    lists.run_flag = reinterpret_cast<int8_t*>(p);
    p += up(c);
    lists.run_pid = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * c);
    lists.run = reinterpret_cast<int32_t*>(p);
    p += up(sizeof(int32_t) * c);
    void* select_temp = p;
    const size_t select_bytes = select_temp_bytes(n);
    cudaError_t e = cudaMemsetAsync(lists.ctr, 0, kCounters * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) {
        set_error("d3d_gjk_distance (mixed): %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    int rc = sched ? pair_order(store, i1, i2, n, order, temp, temp_bytes, stream, n_dev) : D3D_SUCCESS;
    if (!rc) {
        if (t.gjk_block == 64)
            rc = launch_mixed<64>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, select_temp, select_bytes,
                                  blocks_per_sm(t, 64), stream);
        else if (t.gjk_block == 256)
            rc = launch_mixed<256>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, select_temp, select_bytes,
                                   blocks_per_sm(t, 256), stream);
        else
            rc = launch_mixed<128>(store, i1, i2, order, n, n_dev, opt, hand, o, lists, select_temp, select_bytes,
                                   blocks_per_sm(t, 128), stream);
    }
    if (!rc)
        rc = launch_gjk_f64(store, i1, i2, lists.fallback, n, lists.ctr + kNumFallback, lists.ctr + kCurC, opt, o,
                            stream);
    return rc;
}

int gjk_distance_mixed(const d3d_store& store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_gjk_options& opt, double* dist, double* cp1, double* cp2, double* simplex,
                       int8_t* n_simplex, int8_t* status, int32_t* iterations, cudaStream_t stream) {
    void* block = nullptr;
    int rc = scratch_alloc(&block, gjk_mixed_scratch_bytes(n), stream);
    if (rc) return rc;
    DistanceOut o{dist, cp1, cp2, simplex, n_simplex, status, iterations};
    rc = gjk_mixed_run(store, i1, i2, n, nullptr, opt, o, block, stream);
    scratch_free(block, stream);
    return rc;
}

}  // namespace d3d
