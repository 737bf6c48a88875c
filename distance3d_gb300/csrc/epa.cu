// epa.cu -- batched FP64 EPA (expanding polytope): one warp per pair
// (k_epa_exact_warp, the polytope in shared memory) for every option set of up
// to 251 iterations whose polytope fits a block's shared memory, one thread
// per pair (k_epa, the polytope in caller scratch) for the others.
//
// Restates distance3d epa.py (Kevin Moran's formulation): the polytope is an
// unordered array of faces (3 vertices + unit normal), the face closest to the
// origin is found by a linear scan with first-minimum tie-breaking, faces
// visible from the new support point are removed by moving the last face into
// their slot and re-testing that slot, and the horizon ("loose") edges are
// matched by coordinates within epsilon.  Every order-dependent step keeps the
// reference's order, so faces, normals and the MTV are the reference's bit for
// bit (-fmad=false; see d3d_device.cuh).
//
// Where the reference raises (face buffer full, epa.py:128; np.argmin on an
// empty polytope) the pair gets a status code instead.
//
// Thread form scheduling: pairs are sorted by collider types, and a
// persistent grid runs one EPA iteration per round per lane; a lane whose pair
// ends fetches the next one.  Each thread owns one scratch slot of max_faces
// faces and max_loose_edges edges (d3d_epa_scratch_bytes), reused across its
// pairs, so the scratch is bounded by the slot count, not by n.
#include <cmath>
#include <cstring>
#include <mutex>

#include "capi_util.h"
#include "d3d_device.cuh"
#include "epa_mixed.h"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int64_t kMaxSlots = 32768;  // scratch slots (threads) per launch
constexpr int kBlock = 128;
constexpr int64_t kScheduleMin = 4096;

__device__ __forceinline__ d3 ld(const double* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ void st(double* p, d3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// utils.py:12-30 norm_vector
__device__ __forceinline__ d3 norm_vec(d3 v) {
    double n = sqrt(dot(v, v));
    if (n == 0.0) return v;
    return mk(v.x / n, v.y / n, v.z / n);
}

// epa.py:99-102; a face is 12 doubles: v0, v1, v2, n
__device__ __forceinline__ void face_normal(double* f) {
    d3 v0 = ld(f), v1 = ld(f + 3), v2 = ld(f + 6);
    st(f + 9, norm_vec(cross(v1 - v0, v2 - v0)));
}

// The smallest x >= 0 with sqrt(x) >= e.  IEEE sqrt is correctly rounded on
// the host and on the device, hence monotonic, so for every x >= 0 and NaN
//     sqrt(x) < e   <=>   x < sqrt_less_bound(e),
// which lets the kernels compare squared lengths with the reference's
// sqrt(...) < e tests, bit for bit.
double sqrt_less_bound(double e) {
    if (!(e > 0.0)) return 0.0;
    if (e == INFINITY) return INFINITY;
    uint64_t lo = 0, hi = 0x7ff0000000000000ull;  // sqrt(+inf) >= e
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        double x;
        memcpy(&x, &mid, sizeof x);
        if (std::sqrt(x) >= e)
            hi = mid;
        else
            lo = mid + 1;
    }
    double t;
    memcpy(&t, &hi, sizeof t);
    return t;
}

// squared-length bounds of epa.py's two length tests
struct LengthBounds {
    double edge;  // epa.py:189-191: norm(edge end difference) < epsilon
    double keep;  // epa.py:134: norm(face normal) < 0.5
};

LengthBounds length_bounds(double epsilon) { return LengthBounds{sqrt_less_bound(epsilon), sqrt_less_bound(0.5)}; }

__device__ __forceinline__ void copy12(double* dst, const double* src) {
#pragma unroll
    for (int j = 0; j < 12; ++j) dst[j] = src[j];
}

// One pair's EPA between iterations.  F (faces) and E (loose edges) live in
// the thread's scratch slot.
struct EpaLoop {
    int nf;       // faces in the polytope
    int closest;  // face chosen by the last iteration's scan
    int it;
};

// epa.py:56-57, 89-97: the initial faces ABC, ACD, ADB, BDC
__device__ __forceinline__ void epa_begin(EpaLoop& L, const double* simplex, double* F) {
    const int init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) st(F + 12 * i + 3 * j, ld(simplex + 3 * init[i][j]));
        face_normal(F + 12 * i);
    }
    L.nf = 4;
    L.closest = 0;
    L.it = 0;
}

// One iteration of epa.py:59-74.  Returns -1 while running, else the status
// (mtv written).
__device__ __forceinline__ int epa_step(EpaLoop& L, const Col<double>& c1, const Col<double>& c2,
                                        const d3d_store& store, const d3d_epa_options& o, double* F,
                                        double* E, d3& mtv) {
    const double eps = o.epsilon;
    if (L.it >= o.max_iterations) {
        // epa.py:77: closest_face is a view, read after the last iteration's edits
        const double* f = F + 12 * L.closest;
        d3 n = ld(f + 9);
        mtv = n * dot(ld(f), n);
        return D3D_STATUS_EPA_NOT_CONVERGED;
    }
    ++L.it;
    int nf = L.nf;
    if (nf == 0) {
        mtv = mk(double(NAN), double(NAN), double(NAN));
        return D3D_STATUS_EPA_DEGENERATE;
    }
    // epa.py:104-109: np.sum(v0 * n, axis=1), np.argmin (first minimum)
    double md = 0.0;
    int closest = 0;
    for (int i = 0; i < nf; ++i) {
        const double* f = F + 12 * i;
        double d = (f[0] * f[9] + f[1] * f[10]) + f[2] * f[11];
        if (i == 0 || d < md) {
            md = d;
            closest = i;
        }
    }
    L.closest = closest;
    d3 sd = ld(F + 12 * closest + 9);
    d3 np_ = support(c1, store, sd) - support(c2, store, -sd);
    double pd = dot(np_, sd);
    if (pd - md < eps) {  // epa.py:67-70
        mtv = sd * pd;
        return D3D_STATUS_OK;
    }
    // epa.py:157-165 remove visible faces, collect horizon edges
    int ne = 0;
    int i = 0;
    while (i < nf) {
        double* f = F + 12 * i;
        if (dot(ld(f + 9), np_ - ld(f)) > eps) {  // epa.py:122-124
            for (int j = 0; j < 3; ++j) {         // epa.py:167-187
                d3 e0 = ld(f + 3 * j), e1 = ld(f + 3 * ((j + 1) % 3));
                bool found = false;
                for (int k = 0; k < ne; ++k) {
                    double* e = E + 6 * k;
                    d3 d1 = ld(e + 3) - e0, d0 = ld(e) - e1;
                    if (sqrt(dot(d1, d1)) < eps && sqrt(dot(d0, d0)) < eps) {
                        const double* last = E + 6 * (ne - 1);
#pragma unroll
                        for (int q = 0; q < 6; ++q) e[q] = last[q];
                        --ne;
                        found = true;
                        break;
                    }
                }
                if (!found) {
                    if (ne >= o.max_loose_edges) break;  // epa.py:193-198
                    st(E + 6 * ne, e0);
                    st(E + 6 * ne + 3, e1);
                    ++ne;
                }
            }
            copy12(f, F + 12 * (nf - 1));  // epa.py:118-120
            --nf;
            continue;
        }
        ++i;
    }
    // epa.py:126-137 extend_with_point
    for (int k = 0; k < ne; ++k) {
        if (!(nf < o.max_faces)) {
            L.nf = nf;
            mtv = mk(double(NAN), double(NAN), double(NAN));
            return D3D_STATUS_EPA_FACE_OVERFLOW;
        }
        double* f = F + 12 * nf;
        st(f, ld(E + 6 * k));
        st(f + 3, ld(E + 6 * k + 3));
        st(f + 6, np_);
        face_normal(f);
        d3 n = ld(f + 9);
        if (sqrt(dot(n, n)) < 0.5) continue;
        // epa.py:139-146: the reference swaps through a NumPy view of row
        // 0, so the net effect is v0 := v1 (v1 unchanged), n := -n
        if (dot(ld(f), n) + 1e-6 < 0.0) {
            st(f, ld(f + 3));
            st(f + 9, -n);
        }
        ++nf;
    }
    L.nf = nf;
    return -1;
}

__global__ void __launch_bounds__(kBlock) k_epa(d3d_store s, const int32_t* __restrict__ i1,
                                                const int32_t* __restrict__ i2, const int32_t* __restrict__ order,
                                                int64_t n, const unsigned long long* __restrict__ n_dev,
                                                unsigned long long* __restrict__ cursor,
                                                const double* __restrict__ simplex, d3d_epa_options o,
                                                double* __restrict__ mtv, int8_t* __restrict__ status,
                                                int32_t* __restrict__ n_faces, double* __restrict__ faces,
                                                double* __restrict__ scratch, int64_t slot_doubles) {
    if (n_dev) n = (int64_t)*n_dev;
    const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double* F = scratch + slot * slot_doubles;
    double* E = F + 12 * (int64_t)o.max_faces;
    EpaLoop L;
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
            if (!pair_ok(s, a, b)) {
                epa_store_bad_index(mtv, status, n_faces, pid);
                continue;  // the thread fetches again
            }
            epa_begin(L, simplex + 12 * pid, F);
            need = false;
        }
        Col<double> c1, c2;
        load_col(s, a, c1);
        load_col(s, b, c2);
        d3 m;
        const int stt = epa_step(L, c1, c2, s, o, F, E, m);
        if (stt >= 0) {
            mtv[3 * pid] = m.x;
            mtv[3 * pid + 1] = m.y;
            mtv[3 * pid + 2] = m.z;
            status[pid] = (int8_t)stt;
            const int nf = stt == D3D_STATUS_EPA_DEGENERATE ? 0 : L.nf;
            n_faces[pid] = nf;
            if (faces) {
                double* out = faces + pid * 12 * (int64_t)o.max_faces;
                for (int j = 0; j < 12 * nf; ++j) out[j] = F[j];
            }
            need = true;
        }
    }
}

// ---------------------------------------------------------------------------
// The same EPA with one warp per pair.  The polytope (faces as corner ids
// and normals, see WarpPoly) and the loose edges live in the warp's shared
// memory; the steps whose
// order does not matter run across the lanes -- the closest-face scan (on
// integer keys of the face distances), the visibility of every face, the
// normals of the new faces, the closeness of a new vertex to the others --
// and the order-dependent bookkeeping keeps the reference's order exactly:
// faces are removed by moving the last face into the first visible slot and
// testing that slot again, each removed face's edges are matched against the
// loose list in list order (the first match is overwritten by the last
// edge), and new faces are appended in loose-edge order.  Results are those
// of k_epa (and of the reference) bit for bit.

constexpr unsigned kWarpAll = 0xffffffffu;

__device__ __forceinline__ int lane_of() { return threadIdx.x & 31; }

// Storage of one warp's polytope, for cap_f faces, cap_e loose edges and
// nvc vertices (see WarpPoly).
__host__ __device__ inline int pm_words(int nvc) { return (nvc + 31) / 32; }
__host__ __device__ inline int exact_warp_bytes(int cap_f, int cap_e, int nvc) {
    const int e = cap_e > 0 ? cap_e : 1;
    return (32 * cap_f + 24 * nvc + 4 * nvc * pm_words(nvc) + 4 * cap_f + 2 * e + cap_f + 15) & ~15;
}
__host__ __device__ inline int exact_warp_bytes(const d3d_epa_options& o) {
    return exact_warp_bytes(o.max_faces, o.max_loose_edges, o.max_iterations + 4);
}

// One warp's polytope in shared memory.  Every point of the polytope is one
// of its vertices: the simplex's four points and one support point per
// iteration (at most nvc = max_iterations + 4).  A face is the ids of its
// three corners in V and its unit normal; a loose edge the ids of its ends.
// The reference's faces and loose edges hold copies of the corner points
// (epa.py:86, 131-133, 169, 196); the ids name exactly those points, so every
// product below reads the same doubles.  pm holds the reference's closeness
// test between two points (norm(x - y) < epsilon, epa.py:189-191) for every
// pair of vertices, so that matching loose edges needs no arithmetic.  (Ids
// instead of copies: about a third of the shared memory per polytope, so
// about three times the warps per SM on the FP64 pipe.)
struct WarpPoly {
    double* N;              // faces' unit normals (3 doubles)
    unsigned long long* K;  // ordering key of each face's distance
    double* V;              // vertices (3 doubles)
    unsigned* pm;           // bit y of row x (words x * W ...): vertices x and y are close
    unsigned* fid;          // vertex ids of each face's corners v0, v1, v2, 8 bits each
    unsigned short* eid;    // vertex ids of each loose edge's ends (a | b << 8)
    unsigned char* vis;     // visibility flags of the faces
    int W;                  // words per row of pm

    __device__ static WarpPoly at(unsigned char* base, int cap_f, int cap_e, int nvc) {
        const int e = cap_e > 0 ? cap_e : 1;
        WarpPoly P;
        P.N = reinterpret_cast<double*>(base);
        P.K = reinterpret_cast<unsigned long long*>(P.N + 3 * (int64_t)cap_f);
        P.V = reinterpret_cast<double*>(P.K + cap_f);
        P.W = pm_words(nvc);
        P.pm = reinterpret_cast<unsigned*>(P.V + 3 * nvc);
        P.fid = P.pm + nvc * P.W;
        P.eid = reinterpret_cast<unsigned short*>(P.fid + cap_f);
        P.vis = reinterpret_cast<unsigned char*>(P.eid + e);
        return P;
    }
    __device__ bool close(int x, int y) const { return (pm[x * W + (y >> 5)] >> (y & 31)) & 1u; }
    __device__ d3 vert(int v) const { return ld(V + 3 * v); }
    __device__ d3 corner(int f, int j) const { return vert((fid[f] >> (8 * j)) & 0xff); }
    __device__ d3 normal(int f) const { return ld(N + 3 * f); }
    // epa.py:104-106, np.sum(v0 * n) over the face's row
    __device__ double dist(int f) const {
        const d3 v = corner(f, 0), n = normal(f);
        return (v.x * n.x + v.y * n.y) + v.z * n.z;
    }
};

// Ordering key of a face distance: unsigned order equals the order of the
// doubles (-0 as +0); NaN sorts last.
__device__ __forceinline__ unsigned long long dist_key(double d) {
    if (d != d) return ~0ull;
    if (d == 0.0) d = 0.0;
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// The warp's smallest (key, index): the smallest key, then the smallest index
// holding it, by REDUX on the keys' 32-bit halves (no shuffle rounds).
__device__ __forceinline__ void warp_min_key(unsigned long long& k, int& i) {
    const unsigned hi = __reduce_min_sync(kWarpAll, (unsigned)(k >> 32));
    const unsigned lo = __reduce_min_sync(kWarpAll, (unsigned)(k >> 32) == hi ? (unsigned)k : 0xffffffffu);
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    i = (int)__reduce_min_sync(kWarpAll, k == m ? (unsigned)i : 0xffffffffu);
    k = m;
}

// Ordering key of a support product for the first-maximum scans: unsigned
// order equals the order of the doubles (-0 as +0); a NaN is 0, below every
// number, so that it never beats a number.  Integer work only, which keeps the
// scans off the FP64 pipe.
__device__ __forceinline__ unsigned long long max_key(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if ((u << 1) > 0xffe0000000000000ull) return 0ull;
    if ((u << 1) == 0ull) return 0x8000000000000000ull;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// First maximum of V . d over a box's or hull's vertices by the 16 lanes of
// this half warp (np.argmax): a NaN at vertex 0 wins, later NaNs never do.
__device__ __forceinline__ int half_first_max(const d3d_store& st, const Col<double>& c, d3 dd, unsigned half) {
    const int h = lane_of() & 15;
    unsigned long long bk = 0ull;
    int bj = 0x7fffffff;
    bool nan0 = false;
    for (int k = h; k < c.nv; k += 16) {
        const d3 v = load_vertex(st.verts64, c.off + k);
        const unsigned long long key = max_key(dot102(v.x, v.y, v.z, dd.x, dd.y, dd.z));
        if (k == 0 && key == 0ull) nan0 = true;
        if (key > bk) {
            bk = key;
            bj = k;
        }
    }
    for (int m = 8; m; m >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(half, bk, m);
        const int oi = __shfl_xor_sync(half, bj, m);
        if (ok > bk || (ok == bk && oi < bj)) {
            bk = ok;
            bj = oi;
        }
    }
    const bool any_nan0 = __ballot_sync(half, nan0) != 0u;
    return (c.nv == 1 || any_nan0 || bj >= c.nv) ? 0 : bj;
}

// w = s_a(d) - s_b(-d) with the reference's supports: lanes 0-15 evaluate
// collider a, lanes 16-31 collider b; a box or hull's first-maximum vertex is
// found by the 16 lanes of its half (np.argmax).  Every lane returns w.
__device__ d3 minkowski_exact_warp(const d3d_store& st, int a, int b, d3 d) {
    const int ln = lane_of();
    const bool up = ln & 16;
    // the two halves may take different branches: the shuffles and votes
    // below stay within this half
    const unsigned half = up ? 0xffff0000u : 0x0000ffffu;
    Col<double> c;
    load_col(st, up ? b : a, c);
    const d3 dd = up ? -d : d;
    d3 s;
    if (c.type == D3D_BOX || c.type == D3D_HULL) {
        if (c.nv < 1) {
            s = mk(double(NAN), double(NAN), double(NAN));
        } else {
            // (The FP32 filter of hull_argmax_filtered does not pay here: with 16 lanes a typical
            // hull takes a few FP64 rounds, about what its FP32 passes and reductions cost.)
            s = add_margin(c, load_vertex(st.verts64, c.off + half_first_max(st, c, dd, half)), dd);
        }
    } else {
        s = support(c, st, dd);
    }
    const d3 o = mk(__shfl_xor_sync(kWarpAll, s.x, 16), __shfl_xor_sync(kWarpAll, s.y, 16),
                    __shfl_xor_sync(kWarpAll, s.z, 16));
    return up ? o - s : s - o;
}

// One pair's EPA by one warp (epa.py:9-78).  Returns the status; mtv and nf
// (faces left) as k_epa sets them.  The polytope of max_faces faces and
// max_loose_edges loose edges lives in the warp's shared memory (WarpPoly).
__device__ int epa_pair_warp(const d3d_store& store, int a, int b, const double* simplex,
                             const d3d_epa_options& o, LengthBounds lb, const WarpPoly& P, d3& mtv, int& nf_out) {
    unsigned long long* const K = P.K;
    unsigned char* const vis = P.vis;
    const int ln = lane_of();
    const double eps = o.epsilon;
    // vertices 0-3: the simplex's rows, and their closeness
    if (ln < 12) P.V[ln] = simplex[ln];
    __syncwarp();
    {
        const d3 d = ld(P.V + 3 * ((ln >> 2) & 3)) - ld(P.V + 3 * (ln & 3));
        const unsigned m = __ballot_sync(kWarpAll, ln < 16 && dot(d, d) < lb.edge);
        if (ln < 4) P.pm[ln * P.W] = (m >> (4 * ln)) & 0xfu;
    }
    // epa.py:56-57, 89-97: faces ABC, ACD, ADB, BDC
    if (ln < 4) {
        const int init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
        const d3 v0 = P.vert(init[ln][0]), v1 = P.vert(init[ln][1]), v2 = P.vert(init[ln][2]);
        const d3 n = norm_vec(cross(v1 - v0, v2 - v0));  // epa.py:99-102
        st(P.N + 3 * ln, n);
        K[ln] = dist_key((v0.x * n.x + v0.y * n.y) + v0.z * n.z);
        P.fid[ln] = (unsigned)init[ln][0] | ((unsigned)init[ln][1] << 8) | ((unsigned)init[ln][2] << 16);
    }
    __syncwarp();
    int nf = 4, closest = 0, nv = 4;
    for (int it = 0;; ++it) {
        if (it >= o.max_iterations) {
            // epa.py:77: closest_face is a view, read after the last iteration's edits
            const d3 n = P.normal(closest);
            mtv = n * dot(P.corner(closest, 0), n);
            nf_out = nf;
            return D3D_STATUS_EPA_NOT_CONVERGED;
        }
        if (nf == 0) {
            mtv = mk(double(NAN), double(NAN), double(NAN));
            nf_out = nf;
            return D3D_STATUS_EPA_DEGENERATE;
        }
        // epa.py:104-109: np.sum(v0 * n, axis=1), first minimum (k_epa's
        // scan: a NaN at face 0 wins, later NaNs never do), on the faces'
        // ordering keys
        unsigned long long bk = ~0ull;
        int bi = 0x7fffffff;
        for (int i = ln; i < nf; i += 32) {
            const unsigned long long k = K[i];
            if (k < bk) {
                bk = k;
                bi = i;
            }
        }
        warp_min_key(bk, bi);
        closest = (K[0] == ~0ull || bk == ~0ull) ? 0 : bi;
        const double md = P.dist(closest);
        const d3 sd = P.normal(closest);
        const d3 w = minkowski_exact_warp(store, a, b, sd);
        const double pd = dot(w, sd);
        if (pd - md < eps) {  // epa.py:67-70
            mtv = sd * pd;
            nf_out = nf;
            return D3D_STATUS_OK;
        }
        // w becomes vertex wv: its closeness to every vertex (itself
        // included) fills row wv and column wv of pm
        const int wv = nv++;
        if (ln < 3) P.V[3 * wv + ln] = ln == 0 ? w.x : (ln == 1 ? w.y : w.z);
        for (int kb = 0; kb <= wv; kb += 32) {
            const int k = kb + ln;
            bool c = false;
            if (k <= wv) {
                const d3 d = (k == wv ? w : ld(P.V + 3 * k)) - w;
                c = dot(d, d) < lb.edge;
            }
            const unsigned m = __ballot_sync(kWarpAll, c);
            if (ln == 0) P.pm[wv * P.W + (kb >> 5)] = m;
            if (k < wv) {
                unsigned& word = P.pm[k * P.W + (wv >> 5)];
                const unsigned bit = (c ? 1u : 0u) << (wv & 31);
                word = (wv & 31) == 0 ? bit : (word | bit);
            }
        }
        // epa.py:157-165: visibility of every face (epa.py:122-124)
        for (int i = ln; i < nf; i += 32) vis[i] = dot(P.normal(i), w - P.corner(i, 0)) > eps ? 1 : 0;
        __syncwarp();
        // remove visible faces in the reference's order, collecting edges
        int ne = 0, i = 0;
        while (true) {
            int p = -1;
            for (int base = i; base < nf; base += 32) {
                const int j = base + ln;
                const unsigned m = __ballot_sync(kWarpAll, j < nf && vis[j]);
                if (m) {
                    p = base + __ffs(m) - 1;
                    break;
                }
            }
            if (p < 0) break;
            const unsigned fv = P.fid[p];
            // epa.py:167-187: edge j = (v_j, v_j+1) of the face matches loose
            // edge (a, b) when b is close to v_j and a to v_j+1
            // (epa.py:189-191); the first match leaves the list by a swap with
            // its last edge, no match appends the edge
            for (int j = 0; j < 3; ++j) {
                const int x0 = (fv >> (8 * j)) & 0xff, x1 = (fv >> (8 * ((j + 1) % 3))) & 0xff;
                int found = -1;
                for (int kb = 0; kb < ne; kb += 32) {
                    const int k = kb + ln;
                    bool match = false;
                    if (k < ne) {
                        const unsigned e = P.eid[k];
                        match = P.close(e >> 8, x0) && P.close(e & 0xff, x1);
                    }
                    const unsigned m = __ballot_sync(kWarpAll, match);
                    if (m) {
                        found = kb + __ffs(m) - 1;
                        break;
                    }
                }
                if (found >= 0) {
                    if (ln == 0) P.eid[found] = P.eid[ne - 1];
                    --ne;
                } else {
                    if (ne >= o.max_loose_edges) break;  // epa.py:193-198
                    if (ln == 0) P.eid[ne] = (unsigned short)(x0 | (x1 << 8));
                    ++ne;
                }
                __syncwarp();
            }
            // epa.py:118-120: the last face moves into slot p, which is tested again
            if (ln < 3) P.N[3 * p + ln] = P.N[3 * (nf - 1) + ln];
            if (ln == 0) {
                vis[p] = vis[nf - 1];
                K[p] = K[nf - 1];
                P.fid[p] = P.fid[nf - 1];
            }
            --nf;
            i = p;
            __syncwarp();
        }
        // epa.py:126-137 extend_with_point, in loose-edge order
        int kept = 0;
        for (int kb = 0; kb < ne; kb += 32) {
            const int k = kb + ln;
            d3 v0 = mk(0.0, 0.0, 0.0), nrm = v0;
            bool keep = false;
            unsigned ids = 0;
            if (k < ne) {
                // the face (a, b, w) of loose edge k (epa.py:131-133)
                const unsigned ev = P.eid[k];
                ids = (ev & 0xffu) | (ev & 0xff00u) | ((unsigned)wv << 16);
                const d3 e0 = P.vert(ev & 0xffu), e1 = P.vert((ev >> 8) & 0xffu);
                v0 = e0;
                nrm = norm_vec(cross(e1 - e0, w - e0));
                keep = !(dot(nrm, nrm) < lb.keep);
                // epa.py:139-146: the reference swaps through a NumPy view of
                // row 0, so the net effect is v0 := v1 (v1 unchanged), n := -n
                if (keep && dot(v0, nrm) + 1e-6 < 0.0) {
                    v0 = e1;
                    nrm = -nrm;
                    ids = (ids & ~0xffu) | ((ids >> 8) & 0xffu);
                }
            }
            const unsigned km = __ballot_sync(kWarpAll, keep);
            const int before = __popc(km & ((1u << ln) - 1u));
            // epa.py:128: the face buffer is checked before every loose edge
            const bool over = k < ne && nf + kept + before >= o.max_faces;
            const unsigned om = __ballot_sync(kWarpAll, over);
            const int limit = om ? __ffs(om) - 1 : 32;  // edges of this chunk written before the overflow
            if (keep && ln < limit) {
                const int idx = nf + kept + before;
                st(P.N + 3 * idx, nrm);
                K[idx] = dist_key((v0.x * nrm.x + v0.y * nrm.y) + v0.z * nrm.z);
                P.fid[idx] = ids;
            }
            if (om) {
                nf += kept + __popc(km & ((1u << limit) - 1u));
                __syncwarp();
                mtv = mk(double(NAN), double(NAN), double(NAN));
                nf_out = nf;
                return D3D_STATUS_EPA_FACE_OVERFLOW;
            }
            // epa.py:131-135 writes each new face into slot n_faces before testing it, so a degenerate
            // face stays in the slot past the live faces until the next face takes that slot: after the
            // loop the slot holds the last loose edge's face if that one was not kept.  An unconverged
            // pair's MTV can read it (closest_face is a view into the faces, epa.py:77).
            if (k == ne - 1 && !keep) {
                const int idx = nf + kept + before;
                st(P.N + 3 * idx, nrm);
                P.fid[idx] = ids;
            }
            kept += __popc(km);
        }
        nf += kept;
        __syncwarp();
    }
}

// One warp per block; each warp takes pairs from the cursor and holds its
// polytope in the block's dynamic shared memory.
__global__ void k_epa_exact_warp(d3d_store s, const int32_t* __restrict__ i1, const int32_t* __restrict__ i2,
                                 const int32_t* __restrict__ list, int64_t n,
                                 const unsigned long long* __restrict__ n_dev,
                                 unsigned long long* __restrict__ cursor, const double* __restrict__ simplex,
                                 d3d_epa_options o, LengthBounds lb, double* __restrict__ mtv,
                                 int8_t* __restrict__ status, int32_t* __restrict__ n_faces,
                                 double* __restrict__ faces) {
    extern __shared__ __align__(16) unsigned char smem_epa[];
    const int ln = lane_of();
    const WarpPoly P = WarpPoly::at(smem_epa, o.max_faces, o.max_loose_edges, o.max_iterations + 4);
    if (n_dev) n = (int64_t)*n_dev;
    while (true) {
        long long slot = 0;
        if (ln == 0) slot = (long long)atomicAdd(cursor, 1ull);
        slot = __shfl_sync(kWarpAll, slot, 0);
        if (slot >= n) break;
        const int64_t pid = list ? list[slot] : slot;
        const int a = i1[pid], b = i2[pid];
        if (!pair_ok(s, a, b)) {  // the same for every lane
            if (ln == 0) epa_store_bad_index(mtv, status, n_faces, pid);
            __syncwarp();
            continue;
        }
        d3 m;
        int nf = 0;
        const int stt = epa_pair_warp(s, a, b, simplex + 12 * pid, o, lb, P, m, nf);
        if (ln == 0) {
            mtv[3 * pid] = m.x;
            mtv[3 * pid + 1] = m.y;
            mtv[3 * pid + 2] = m.z;
            status[pid] = (int8_t)stt;
            n_faces[pid] = stt == D3D_STATUS_EPA_DEGENERATE ? 0 : nf;
        }
        if (faces && stt != D3D_STATUS_EPA_DEGENERATE) {
            // the reference's rows: v0, v1, v2, n
            double* out = faces + pid * 12 * (int64_t)o.max_faces;
            for (int f = ln; f < nf; f += 32) {
#pragma unroll
                for (int j = 0; j < 3; ++j) st(out + 12 * f + 3 * j, P.corner(f, j));
                st(out + 12 * f + 9, P.normal(f));
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// The same EPA with W pairs per block in lock step (k_epa_exact_block).  Two
// steps of an iteration cost the FP64 pipe per pair, not per lane: the
// support of an analytic collider (16 lanes of a half warp evaluate the same
// FP64 expressions, and the two halves of a pair of different types run one
// after the other) and the normals of the new faces (one lane per loose edge,
// ~8 of 32 lanes active).  Here each round every warp runs one iteration of
// its pair up to the support, posts the supports of its analytic colliders
// (a box or hull keeps its 16-lane FP64 argmax in the owning warp), and the
// posted supports are evaluated one per lane, the supports of collider type t
// by warp t % W (so that the warps run different types' paths side by side,
// 61.8 -> 59.1 ms against warp 0 for all); after the visible faces are
// removed every warp posts its loose edges (up to 32) and all lanes of the
// block compute the new faces' normals, one per lane; each warp then commits
// its new faces in loose-edge order.  Every value is computed by the same
// expressions as in epa_pair_warp, so the results are the same bit for bit.
// A warp whose pair ends (or that has none) sits out the rest of the round.

constexpr int kFaceTaskPerWarp = 32;  // loose edges a warp posts per round; more are computed in place

struct BlockTasks {
    double* sres;            // support results, 3 doubles per task (task 2 w + side)
    double* sdir;            // support directions of the posted tasks
    int* scol;               // collider of each posted task, -1 if none
    int* stype;              // its collider type
    double* fn;              // new faces: normal (3 doubles) per task
    unsigned long long* fk;  // their distance keys (kept faces)
    unsigned* fid;           // ids | 1 << 31 if kept
    unsigned* ftask;         // task: warp | edge << 8
    int* wv;                 // the new vertex of each warp this round
    int* nface;              // face tasks posted this round
};

__host__ __device__ inline int block_task_bytes(int W) {
    const int st = 2 * W;
    const int ft = W * kFaceTaskPerWarp;
    return ((st * 48 + st * 8 + ft * (24 + 8 + 4 + 4) + W * 4 + 16) + 15) & ~15;
}

template <int W>
__device__ __forceinline__ BlockTasks block_tasks_at(unsigned char* base) {
    constexpr int ST = 2 * W, FT = W * kFaceTaskPerWarp;
    BlockTasks T;
    T.sres = reinterpret_cast<double*>(base);
    T.sdir = T.sres + 3 * ST;
    T.fn = T.sdir + 3 * ST;
    T.fk = reinterpret_cast<unsigned long long*>(T.fn + 3 * FT);
    T.scol = reinterpret_cast<int*>(T.fk + FT);
    T.stype = T.scol + ST;
    T.fid = reinterpret_cast<unsigned*>(T.stype + ST);
    T.ftask = T.fid + FT;
    T.wv = reinterpret_cast<int*>(T.ftask + FT);
    T.nface = T.wv + W;
    return T;
}

// epa.py:131-146 for loose edge k of polytope P with new vertex wv: the
// face's unit normal and first corner after the reference's winding fix,
// whether it is kept (norm >= 0.5), and its vertex ids.
__device__ __forceinline__ void new_face(const WarpPoly& P, int k, int wv, LengthBounds lb, d3& v0, d3& nrm, bool& keep,
                                         unsigned& ids) {
    const unsigned ev = P.eid[k];
    ids = (ev & 0xffu) | (ev & 0xff00u) | ((unsigned)wv << 16);
    const d3 e0 = P.vert(ev & 0xffu), e1 = P.vert((ev >> 8) & 0xffu), w = P.vert(wv);
    v0 = e0;
    nrm = norm_vec(cross(e1 - e0, w - e0));
    keep = !(dot(nrm, nrm) < lb.keep);
    // epa.py:139-146: the reference swaps through a NumPy view of row 0, so
    // the net effect is v0 := v1 (v1 unchanged), n := -n
    if (keep && dot(v0, nrm) + 1e-6 < 0.0) {
        v0 = e1;
        nrm = -nrm;
        ids = (ids & ~0xffu) | ((ids >> 8) & 0xffu);
    }
}

template <int W>
__global__ void __launch_bounds__(32 * W, 16 / W) k_epa_exact_block(d3d_store s, const int32_t* __restrict__ i1,
                                                            const int32_t* __restrict__ i2,
                                                            const int32_t* __restrict__ list, int64_t n,
                                                            const unsigned long long* __restrict__ n_dev,
                                                            unsigned long long* __restrict__ cursor,
                                                            const double* __restrict__ simplex, d3d_epa_options o,
                                                            LengthBounds lb, double* __restrict__ mtv_out,
                                                            int8_t* __restrict__ status_out,
                                                            int32_t* __restrict__ n_faces_out,
                                                            double* __restrict__ faces) {
    extern __shared__ __align__(16) unsigned char smem_blk[];
    const int ln = lane_of(), wp = threadIdx.x >> 5;
    const int pbytes = exact_warp_bytes(o);
    const WarpPoly P = WarpPoly::at(smem_blk + wp * pbytes, o.max_faces, o.max_loose_edges, o.max_iterations + 4);
    const BlockTasks T = block_tasks_at<W>(smem_blk + W * pbytes);
    unsigned long long* const K = P.K;
    unsigned char* const vis = P.vis;
    const double eps = o.epsilon;
    if (n_dev) n = (int64_t)*n_dev;
    int64_t pid = 0;
    int a = 0, b = 0, nf = 0, closest = 0, nv = 0, it = 0, stt = 0;
    bool have = false, exhausted = false;
    d3 mtv = mk(0.0, 0.0, 0.0);
    // The block's shared work (posted supports, new faces) goes to warps by a rotation that
    // changes every round and differs between the blocks of an SM, so that it does not always
    // fall on the same warp slot and with it on one sub-partition's FP64 pipe.
    int rot = (int)(((unsigned)blockIdx.x * (unsigned)W) / gridDim.x) % W;
    while (true) {
        rot = rot + 1 == W ? 0 : rot + 1;
        // a warp without a pair takes the next one
        bool fresh = false;
        if (!have && !exhausted) {
            long long slot = 0;
            if (ln == 0) slot = (long long)atomicAdd(cursor, 1ull);
            slot = __shfl_sync(kWarpAll, slot, 0);
            if (slot >= n) {
                exhausted = true;
            } else {
                pid = list ? list[slot] : slot;
                a = i1[pid];
                b = i2[pid];
                if (pair_ok(s, a, b)) {
                    have = true;
                    fresh = true;
                } else if (ln == 0) {
                    epa_store_bad_index(mtv_out, status_out, n_faces_out, pid);
                }
            }
        }
        if (!__syncthreads_or(have || (!exhausted && ln == 0))) break;
        if (threadIdx.x == 0) *T.nface = 0;
        bool run = have;  // this warp iterates this round
        if (fresh) {
            // vertices 0-3: the simplex's rows, and their closeness; faces ABC, ACD, ADB, BDC
            const double* sx = simplex + 12 * pid;
            if (ln < 12) P.V[ln] = sx[ln];
            __syncwarp();
            {
                const d3 d = ld(P.V + 3 * ((ln >> 2) & 3)) - ld(P.V + 3 * (ln & 3));
                const unsigned m = __ballot_sync(kWarpAll, ln < 16 && dot(d, d) < lb.edge);
                if (ln < 4) P.pm[ln * P.W] = (m >> (4 * ln)) & 0xfu;
            }
            if (ln < 4) {
                const int init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
                const d3 v0 = P.vert(init[ln][0]), v1 = P.vert(init[ln][1]), v2 = P.vert(init[ln][2]);
                const d3 nn = norm_vec(cross(v1 - v0, v2 - v0));  // epa.py:99-102
                st(P.N + 3 * ln, nn);
                K[ln] = dist_key((v0.x * nn.x + v0.y * nn.y) + v0.z * nn.z);
                P.fid[ln] = (unsigned)init[ln][0] | ((unsigned)init[ln][1] << 8) | ((unsigned)init[ln][2] << 16);
            }
            __syncwarp();
            nf = 4;
            closest = 0;
            nv = 4;
            it = 0;
        }
        // the iteration up to the support
        d3 sd = mk(0.0, 0.0, 0.0);
        double md = 0.0;
        if (run) {
            if (it >= o.max_iterations) {
                // epa.py:77: closest_face is a view, read after the last iteration's edits
                const d3 nn = P.normal(closest);
                mtv = nn * dot(P.corner(closest, 0), nn);
                stt = D3D_STATUS_EPA_NOT_CONVERGED;
                run = false;
            } else if (nf == 0) {
                mtv = mk(double(NAN), double(NAN), double(NAN));
                stt = D3D_STATUS_EPA_DEGENERATE;
                run = false;
            }
        }
        if (run) {
            unsigned long long bk = ~0ull;
            int bi = 0x7fffffff;
            for (int i = ln; i < nf; i += 32) {
                const unsigned long long k = K[i];
                if (k < bk) {
                    bk = k;
                    bi = i;
                }
            }
            warp_min_key(bk, bi);
            closest = (K[0] == ~0ull || bk == ~0ull) ? 0 : bi;
            md = P.dist(closest);
            sd = P.normal(closest);
            // supports: a box or hull by its half warp here (first maximum of V . d, a NaN at vertex
            // 0 wins, later NaNs never do); the other types are posted for warp 0
            const bool up = ln & 16;
            const unsigned half = up ? 0xffff0000u : 0x0000ffffu;
            const int side = up ? 1 : 0;
            Col<double> c;
            load_col(s, up ? b : a, c);
            const d3 dd = up ? -sd : sd;
            if (c.type == D3D_BOX || c.type == D3D_HULL) {
                d3 r;
                if (c.nv < 1) {
                    r = mk(double(NAN), double(NAN), double(NAN));
                } else {
                    r = add_margin(c, load_vertex(s.verts64, c.off + half_first_max(s, c, dd, half)), dd);
                }
                if ((ln & 15) == 0) {
                    st(T.sres + 3 * (2 * wp + side), r);
                    T.scol[2 * wp + side] = -1;
                }
            } else if ((ln & 15) == 0) {
                st(T.sdir + 3 * (2 * wp + side), dd);
                T.scol[2 * wp + side] = up ? b : a;
                T.stype[2 * wp + side] = c.type;
            }
        } else if (ln < 2) {
            T.scol[2 * wp + ln] = -1;
        }
        __syncthreads();
        // the posted supports, one per lane, each collider type on its own warp where W allows
        // (the analytic types numbered 0-7, rotated), so that the warps run different types'
        // FP64 paths side by side
        if (ln < 2 * W) {
            const int ci = T.scol[ln];
            const int ty = T.stype[ln];
            if (ci >= 0 && (ty - (ty > D3D_BOX) - (ty > D3D_HULL) + rot) % W == wp) {
                Col<double> c;
                load_col(s, ci, c);
                st(T.sres + 3 * ln, support(c, s, ld(T.sdir + 3 * ln)));
            }
        }
        __syncthreads();
        int ne = 0, wv = 0;
        d3 w = mk(0.0, 0.0, 0.0);
        if (run) {
            w = ld(T.sres + 3 * (2 * wp)) - ld(T.sres + 3 * (2 * wp + 1));
            const double pd = dot(w, sd);
            if (pd - md < eps) {  // epa.py:67-70
                mtv = sd * pd;
                stt = D3D_STATUS_OK;
                run = false;
            }
        }
        if (run) {
            ++it;
            // w becomes vertex wv: its closeness to every vertex (itself
            // included) fills row wv and column wv of pm
            wv = nv++;
            if (ln < 3) P.V[3 * wv + ln] = ln == 0 ? w.x : (ln == 1 ? w.y : w.z);
            for (int kb = 0; kb <= wv; kb += 32) {
                const int k = kb + ln;
                bool c = false;
                if (k <= wv) {
                    const d3 d = (k == wv ? w : ld(P.V + 3 * k)) - w;
                    c = dot(d, d) < lb.edge;
                }
                const unsigned m = __ballot_sync(kWarpAll, c);
                if (ln == 0) P.pm[wv * P.W + (kb >> 5)] = m;
                if (k < wv) {
                    unsigned& word = P.pm[k * P.W + (wv >> 5)];
                    const unsigned bit = (c ? 1u : 0u) << (wv & 31);
                    word = (wv & 31) == 0 ? bit : (word | bit);
                }
            }
            // epa.py:157-165: visibility of every face (epa.py:122-124)
            for (int i = ln; i < nf; i += 32) vis[i] = dot(P.normal(i), w - P.corner(i, 0)) > eps ? 1 : 0;
            __syncwarp();
            // remove visible faces in the reference's order, collecting edges
            int i = 0;
            while (true) {
                int p = -1;
                for (int base = i; base < nf; base += 32) {
                    const int j = base + ln;
                    const unsigned m = __ballot_sync(kWarpAll, j < nf && vis[j]);
                    if (m) {
                        p = base + __ffs(m) - 1;
                        break;
                    }
                }
                if (p < 0) break;
                const unsigned fv = P.fid[p];
                for (int j = 0; j < 3; ++j) {
                    const int x0 = (fv >> (8 * j)) & 0xff, x1 = (fv >> (8 * ((j + 1) % 3))) & 0xff;
                    int found = -1;
                    for (int kb = 0; kb < ne; kb += 32) {
                        const int k = kb + ln;
                        bool match = false;
                        if (k < ne) {
                            const unsigned e = P.eid[k];
                            match = P.close(e >> 8, x0) && P.close(e & 0xff, x1);
                        }
                        const unsigned m = __ballot_sync(kWarpAll, match);
                        if (m) {
                            found = kb + __ffs(m) - 1;
                            break;
                        }
                    }
                    if (found >= 0) {
                        if (ln == 0) P.eid[found] = P.eid[ne - 1];
                        --ne;
                    } else {
                        if (ne >= o.max_loose_edges) break;  // epa.py:193-198
                        if (ln == 0) P.eid[ne] = (unsigned short)(x0 | (x1 << 8));
                        ++ne;
                    }
                    __syncwarp();
                }
                // epa.py:118-120: the last face moves into slot p, which is tested again
                if (ln < 3) P.N[3 * p + ln] = P.N[3 * (nf - 1) + ln];
                if (ln == 0) {
                    vis[p] = vis[nf - 1];
                    K[p] = K[nf - 1];
                    P.fid[p] = P.fid[nf - 1];
                }
                --nf;
                i = p;
                __syncwarp();
            }
        }
        // the new faces of up to 32 loose edges per warp go to the block
        const bool post = run && ne <= kFaceTaskPerWarp;
        int fbase = 0;
        if (post && ln == 0) {
            fbase = atomicAdd(T.nface, ne);
            T.wv[wp] = wv;
        }
        fbase = __shfl_sync(kWarpAll, fbase, 0);
        if (post && ln < ne) T.ftask[fbase + ln] = (unsigned)wp | ((unsigned)ln << 8);
        __syncthreads();
        // chunk c of 32 tasks on warp (c + rot) % W
        for (int t = 32 * ((wp - rot + W) % W) + ln; t < *T.nface; t += 32 * W) {
            const unsigned task = T.ftask[t];
            const int q = task & 0xff, k = task >> 8;
            const WarpPoly Q = WarpPoly::at(smem_blk + q * pbytes, o.max_faces, o.max_loose_edges,
                                            o.max_iterations + 4);
            d3 v0, nrm;
            bool keep;
            unsigned ids;
            new_face(Q, k, T.wv[q], lb, v0, nrm, keep, ids);
            st(T.fn + 3 * t, nrm);
            if (keep) T.fk[t] = dist_key((v0.x * nrm.x + v0.y * nrm.y) + v0.z * nrm.z);
            T.fid[t] = ids | (keep ? 0x80000000u : 0u);
        }
        __syncthreads();
        if (run) {
            // epa.py:126-137 extend_with_point, in loose-edge order
            int kept = 0;
            for (int kb = 0; kb < ne; kb += 32) {
                const int k = kb + ln;
                d3 v0 = mk(0.0, 0.0, 0.0), nrm = v0;
                bool keep = false;
                unsigned ids = 0;
                unsigned long long key = 0;
                if (k < ne) {
                    if (post) {
                        const int t = fbase + k;
                        nrm = ld(T.fn + 3 * t);
                        ids = T.fid[t];
                        keep = (ids >> 31) != 0;
                        ids &= 0x7fffffffu;
                        if (keep) key = T.fk[t];
                    } else {
                        new_face(P, k, wv, lb, v0, nrm, keep, ids);
                        if (keep) key = dist_key((v0.x * nrm.x + v0.y * nrm.y) + v0.z * nrm.z);
                    }
                }
                const unsigned km = __ballot_sync(kWarpAll, keep);
                const int before = __popc(km & ((1u << ln) - 1u));
                // epa.py:128: the face buffer is checked before every loose edge
                const bool over = k < ne && nf + kept + before >= o.max_faces;
                const unsigned om = __ballot_sync(kWarpAll, over);
                const int limit = om ? __ffs(om) - 1 : 32;  // edges of this chunk written before the overflow
                if (keep && ln < limit) {
                    const int idx = nf + kept + before;
                    st(P.N + 3 * idx, nrm);
                    K[idx] = key;
                    P.fid[idx] = ids;
                }
                if (om) {
                    nf += kept + __popc(km & ((1u << limit) - 1u));
                    mtv = mk(double(NAN), double(NAN), double(NAN));
                    stt = D3D_STATUS_EPA_FACE_OVERFLOW;
                    run = false;
                    break;
                }
                // epa.py:131-135: a face that is not kept stays in the slot past the live faces
                // (see epa_pair_warp)
                if (k == ne - 1 && !keep) {
                    const int idx = nf + kept + before;
                    st(P.N + 3 * idx, nrm);
                    P.fid[idx] = ids;
                }
                kept += __popc(km);
            }
            if (run) nf += kept;
            __syncwarp();
        }
        // a pair that ended this round
        if (have && !run) {
            if (ln == 0) {
                mtv_out[3 * pid] = mtv.x;
                mtv_out[3 * pid + 1] = mtv.y;
                mtv_out[3 * pid + 2] = mtv.z;
                status_out[pid] = (int8_t)stt;
                n_faces_out[pid] = stt == D3D_STATUS_EPA_DEGENERATE ? 0 : nf;
            }
            if (faces && stt != D3D_STATUS_EPA_DEGENERATE) {
                double* out = faces + pid * 12 * (int64_t)o.max_faces;
                for (int f = ln; f < nf; f += 32) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) st(out + 12 * f + 3 * j, P.corner(f, j));
                    st(out + 12 * f + 9, P.normal(f));
                }
            }
            have = false;
            __syncwarp();
        }
    }
}

constexpr int64_t kExactSmemPerBlock = 227 * 1024;

bool exact_warp_supported(const d3d_epa_options& o) {
    // vertex ids fit in 8 bits
    return o.max_iterations <= 251 && o.max_faces <= 65536 && o.max_loose_edges <= 65536 &&
           (int64_t)exact_warp_bytes(o) <= kExactSmemPerBlock;
}

// W pairs per block in lock step (k_epa_exact_block), W = 4 or 2 as shared
// memory allows; 0 if neither fits.  (At the bench's options, 310k pairs:
// W = 4 61.7 ms, W = 2 70.0 ms, W = 8 69.3 ms, W = 16 78.4 ms, one warp per
// block 84.1 ms: wider blocks share more supports and normals but wait longer
// at their barriers, narrower ones share less.  With the shared work rotated
// over the warps: W = 4 55.2 ms, W = 8 56.6 ms.)
int exact_block_warps(const d3d_epa_options& o) {
    if (!exact_warp_supported(o)) return 0;
    for (int w = 4; w >= 2; w /= 2)
        if ((int64_t)w * exact_warp_bytes(o) + block_task_bytes(w) <= kExactSmemPerBlock) return w;
    return 0;
}

template <int W>
int exact_block_launch_w(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                         const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                         const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                         cudaStream_t stream) {
    const int smem = W * exact_warp_bytes(o) + block_task_bytes(W);
    const void* fn = (const void*)k_epa_exact_block<W>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) {
        set_error("d3d_epa: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    const int blocks = persistent_blocks(fn, 32 * W, n * 32, 0, smem);
    k_epa_exact_block<W><<<blocks, 32 * W, smem, stream>>>(store, i1, i2, list, n, n_dev, cursor, simplex, o,
                                                           length_bounds(o.epsilon), mtv, status, n_faces, faces);
    return check_launch("d3d_epa");
}

// The FP64 EPA with the polytopes in shared memory: W pairs per block in lock
// step where W polytopes fit a block (k_epa_exact_block), else one warp per
// block, each block holding one polytope, as many per SM as shared memory and
// registers allow (k_epa_exact_warp).
int exact_warp_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                      const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                      const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                      cudaStream_t stream) {
    // the block form where its polytopes fit
    const int bw = exact_block_warps(o);
    if (bw == 4)
        return exact_block_launch_w<4>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces, faces,
                                       stream);
    if (bw == 2)
        return exact_block_launch_w<2>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces, faces,
                                       stream);
    const int smem = exact_warp_bytes(o);
    const void* fn = (const void*)k_epa_exact_warp;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) {
        set_error("d3d_epa: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    const int blocks = persistent_blocks(fn, 32, n, 0, smem);
    k_epa_exact_warp<<<blocks, 32, smem, stream>>>(store, i1, i2, list, n, n_dev, cursor, simplex, o,
                                                   length_bounds(o.epsilon), mtv, status, n_faces, faces);
    return check_launch("d3d_epa");
}

int64_t slot_doubles(const d3d_epa_options& o) {
    return 12 * (int64_t)o.max_faces + 6 * (int64_t)o.max_loose_edges;
}

// the mixed form also runs the FP64 kernel on its fallback pairs
int64_t slot_bytes_for(const d3d_epa_options& o) {
    const int64_t f64 = slot_doubles(o) * (int64_t)sizeof(double);
    if (o.precision != D3D_PRECISION_MIXED) return f64;
    const int64_t mixed = d3d::epa_mixed_slot_bytes(o);
    return mixed > f64 ? mixed : f64;
}

int64_t slots_for(int64_t n) {
    int64_t s = n < kMaxSlots ? n : kMaxSlots;
    return ((s + kBlock - 1) / kBlock) * kBlock;
}

bool valid(const d3d_epa_options* o) {
    return o && o->max_iterations >= 0 && o->max_faces >= 4 && o->max_loose_edges >= 0 && o->epsilon >= 0.0 &&
           (o->precision == D3D_PRECISION_FP64 || o->precision == D3D_PRECISION_MIXED);
}

}  // namespace

namespace d3d {

int64_t epa_f64_slot_bytes(const d3d_epa_options& o) { return slot_doubles(o) * (int64_t)sizeof(double); }

int epa_f64_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                   const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                   const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                   void* scratch, int64_t slots, cudaStream_t stream) {
    if (exact_warp_supported(o))  // the polytopes in shared memory: no slot scratch
        return exact_warp_launch(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces, faces,
                                 stream);
    int blocks = persistent_blocks((const void*)k_epa, kBlock, n);
    if (blocks > slots / kBlock) blocks = (int)(slots / kBlock);
    if (blocks < 1) {
        set_error("d3d_epa: fewer than %d polytope slots", kBlock);
        return D3D_ERR_CAPACITY;
    }
    k_epa<<<blocks, kBlock, 0, stream>>>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces,
                                         faces, static_cast<double*>(scratch), slot_doubles(o));
    return check_launch("d3d_epa");
}

}  // namespace d3d

extern "C" size_t d3d_epa_scratch_bytes(int64_t n, const d3d_epa_options* options) {
    if (!valid(options) || n <= 0) return 0;
    return (size_t)(slots_for(n) * slot_bytes_for(*options));
}

extern "C" int d3d_epa(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n, const double* simplex,
                       const d3d_epa_options* options, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                       void* scratch, size_t scratch_bytes, void* stream) {
    int rc = d3d::check_store(store, "d3d_epa");
    if (rc) return rc;
    D3D_REQUIRE(valid(options), "d3d_epa: invalid options (need max_faces >= 4, limits >= 0, epsilon >= 0)");
    D3D_REQUIRE(n >= 0, "d3d_epa: n < 0");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && simplex && mtv && status && n_faces, "d3d_epa: null pointer");
    size_t need = d3d_epa_scratch_bytes(n, options);
    if (!scratch || scratch_bytes < need) {
        d3d::set_error("d3d_epa: scratch of %zu bytes < %zu needed", scratch_bytes, need);
        return D3D_ERR_CAPACITY;
    }
    cudaStream_t st = d3d::as_stream(stream);
    const bool mixed = options->precision == D3D_PRECISION_MIXED;
    const bool warp = mixed && d3d::epa_warp_supported(*options);
    const bool sched = n >= kScheduleMin && !warp && !exact_warp_supported(*options);
    const size_t up_n = (sizeof(int32_t) * (size_t)n + 255) & ~size_t(255);
    const size_t order_bytes = sched ? up_n : 0;
    // fallback lists of the FP32 and FP64 warp searches, the FP32 search's refinement list
    const size_t fb_bytes = mixed ? 3 * up_n : 0;
    const size_t temp_bytes = sched ? (d3d::pair_order_temp_bytes(n) + 255) & ~size_t(255) : 0;
    void* block = nullptr;
    rc = d3d::scratch_alloc(&block, 256 + order_bytes + fb_bytes + temp_bytes, st);
    if (rc) return rc;
    char* p = static_cast<char*>(block);
    // counters: cursor, FP64 EPA cursor, fallback count, FP64 warp cursor, second fallback count,
    // refinement count
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(p);
    int32_t* order = sched ? reinterpret_cast<int32_t*>(p + 256) : nullptr;
    int32_t* fallback = mixed ? reinterpret_cast<int32_t*>(p + 256 + order_bytes) : nullptr;
    int32_t* fallback2 = mixed ? reinterpret_cast<int32_t*>(p + 256 + order_bytes + up_n) : nullptr;
    int32_t* refine = mixed ? reinterpret_cast<int32_t*>(p + 256 + order_bytes + 2 * up_n) : nullptr;
    const bool warp64 = warp && d3d::epa_warp_supported(*options, true);
    cudaMemsetAsync(ctr, 0, 6 * sizeof(unsigned long long), st);
    if (sched) rc = d3d::pair_order(*store, i1, i2, n, order, p + 256 + order_bytes + fb_bytes, temp_bytes, st);
    if (!rc && warp) {
        rc = d3d::epa_warp_launch(*store, i1, i2, nullptr, n, nullptr, ctr, simplex, *options, mtv, status, n_faces,
                                  faces, fallback, ctr + 2, st, false, refine, ctr + 5);
        if (!rc && warp64)
            rc = d3d::epa_warp_launch(*store, i1, i2, fallback, n, ctr + 2, ctr + 3, simplex, *options, mtv, status,
                                      n_faces, faces, fallback2, ctr + 4, st, true);
    } else if (!rc && mixed)
        rc = d3d::epa_mixed_launch(*store, i1, i2, order, n, ctr, simplex, *options, mtv, status, n_faces, faces,
                                   scratch, slots_for(n), fallback, ctr + 2, st);
    const int32_t* f64_list = warp64 ? fallback2 : (mixed ? fallback : order);
    const unsigned long long* f64_count = warp64 ? ctr + 4 : (mixed ? ctr + 2 : nullptr);
    if (!rc && exact_warp_supported(*options)) {
        // the FP64 EPA, one warp per pair: every pair, or the mixed form's fallback pairs
        rc = exact_warp_launch(*store, i1, i2, f64_list, n, f64_count, mixed ? ctr + 1 : ctr, simplex, *options, mtv,
                               status, n_faces, faces, st);
    } else if (!rc) {
        // the FP64 EPA: every pair, or the mixed form's fallback pairs
        int blocks = d3d::persistent_blocks((const void*)k_epa, kBlock, n);
        const int64_t max_blocks = slots_for(n) / kBlock;  // the scratch holds this many slots
        if (blocks > max_blocks) blocks = (int)max_blocks;
        k_epa<<<blocks, kBlock, 0, st>>>(*store, i1, i2, f64_list, n, f64_count, mixed ? ctr + 1 : ctr, simplex,
                                         *options,
                                         mtv, status, n_faces, faces, static_cast<double*>(scratch),
                                         slot_doubles(*options));
        rc = d3d::check_launch("d3d_epa");
    }
    d3d::scratch_free(block, st);
    return rc;
}

// ----------------------------------------------------------------------------
// EPA without any allocation.
//
// For callers that must not allocate device memory once they are running: a
// control loop with a fixed memory budget, a plugin whose host application
// owns every allocation on the GPU, or a process that pre-reserves all of its
// memory at start-up.  d3d_epa needs a caller buffer plus a small temporary
// from the library's pool; this variant instead keeps the polytope slots and
// its work counter in one array that is part of the loaded library image, so
// a call allocates nothing (no cudaMalloc, no pool, no sort temporaries:
// pairs run in input order).
//
// The array is kNoAllocBytes = 16 MiB on every GPU that loads the library,
// held until the process exits.  Options the one-warp-per-pair kernel takes
// (the defaults and the bench's 256 faces among them) keep each polytope in
// shared memory and use the array only for the work counter.  Otherwise the
// array holds the polytope slots: it bounds the per-pair polytope, not the
// number of pairs (each slot is reused across pairs), and a call fails with
// D3D_ERR_CAPACITY when a single slot of (12 * max_faces + 6 *
// max_loose_edges) doubles leaves room for fewer than 128 slots.
//
// Every call shares the array, and the array keeps the previous call's
// contents (the work counter is cleared on the stream at the start of each
// call).  Calls whose work overlaps on the GPU -- concurrent streams, or
// threads sharing a device -- race on it and must be serialised by the
// caller.
namespace {

constexpr size_t kNoAllocBytes = size_t(16) << 20;
constexpr int kMaxNoAllocDevices = 64;

static __device__ __align__(256) unsigned char g_epa_noalloc[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxNoAllocDevices] = {};

// The array's device address for the current device.  The first call on a
// device (with that device current) looks it up with cudaGetSymbolAddress;
// host code must never pass the symbol itself to a kernel.
int noalloc_base(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxNoAllocDevices) {
        d3d::set_error("d3d_epa_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_epa_noalloc);
        if (e != cudaSuccess || p == nullptr) {
            d3d::set_error("d3d_epa_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return D3D_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return D3D_SUCCESS;
}

}  // namespace

extern "C" int d3d_epa_noalloc(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                               const double* simplex, const d3d_epa_options* options, double* mtv, int8_t* status,
                               int32_t* n_faces, double* faces, void* stream) {
    int rc = d3d::check_store(store, "d3d_epa_noalloc");
    if (rc) return rc;
    D3D_REQUIRE(valid(options) && options->precision == D3D_PRECISION_FP64,
                "d3d_epa_noalloc: invalid options (need the FP64 form, max_faces >= 4, limits >= 0, epsilon >= 0)");
    D3D_REQUIRE(n >= 0, "d3d_epa_noalloc: n < 0");
    const bool warp = exact_warp_supported(*options);  // the polytopes in shared memory
    const int64_t slot_bytes = slot_doubles(*options) * (int64_t)sizeof(double);
    const int64_t slots = (int64_t)(kNoAllocBytes - 256) / slot_bytes;
    if (!warp && slots < kBlock) {
        d3d::set_error("d3d_epa_noalloc: max_faces=%d, max_loose_edges=%d need %lld bytes per pair; the static "
                       "scratch of %zu bytes holds fewer than %d pairs at a time (use d3d_epa)",
                       options->max_faces, options->max_loose_edges, (long long)slot_bytes, kNoAllocBytes, kBlock);
        return D3D_ERR_CAPACITY;
    }
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && simplex && mtv && status && n_faces, "d3d_epa_noalloc: null pointer");
    void* base = nullptr;
    rc = noalloc_base(&base);
    if (rc) return rc;
    {
        // the array's address is the current device's: the store must live there
        int cur = 0;
        cudaPointerAttributes pa = {};
        if (cudaGetDevice(&cur) == cudaSuccess) {
            if (cudaPointerGetAttributes(&pa, store->rec64) != cudaSuccess) {
                cudaGetLastError();  // not a pointer the runtime knows: nothing to compare, no error left behind
            } else if (pa.type == cudaMemoryTypeDevice && pa.device != cur) {
                d3d::set_error("d3d_epa_noalloc: the store is on device %d but device %d is current", pa.device,
                               cur);
                return D3D_ERR_INVALID;
            }
        }
    }
    cudaStream_t st = d3d::as_stream(stream);
    unsigned long long* cursor = static_cast<unsigned long long*>(base);
    double* slot_mem = reinterpret_cast<double*>(static_cast<char*>(base) + 256);
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_epa_noalloc: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    if (warp)  // the static array holds the counter only
        return exact_warp_launch(*store, i1, i2, nullptr, n, nullptr, cursor, simplex, *options, mtv, status,
                                 n_faces, faces, st);
    int blocks = d3d::persistent_blocks((const void*)k_epa, kBlock, n);
    if (blocks > slots / kBlock) blocks = (int)(slots / kBlock);
    k_epa<<<blocks, kBlock, 0, st>>>(*store, i1, i2, nullptr, n, nullptr, cursor, simplex, *options, mtv, status,
                                     n_faces, faces, slot_mem, slot_doubles(*options));
    return d3d::check_launch("d3d_epa_noalloc");
}
