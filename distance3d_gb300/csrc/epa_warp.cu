// epa_warp.cu -- mixed-precision EPA, one warp per pair.
//
// The search is the mixed EPA of epa_mixed.cu (FP32 polytope search on the
// FP32 mirror, validation with an FP64 fallback); this file lays it out for
// the GPU.  Each pair's polytope lives in its warp's slice of shared memory
// and the 32 lanes share the work of every expansion (epa.py:59-74):
//
//   closest face      lanes scan strided face slots, warp min-reduction
//   support           the two colliders on the two half warps; box / hull
//                     argmax split across a half warp's lanes (first
//                     maximum, as np.argmax)
//   visible faces     breadth-first search from the closest face over the
//                     face adjacency with the reference's visibility test
//                     (epa.py:157-165)
//   horizon           edges of visible faces whose neighbour is not visible,
//                     gathered by a warp prefix sum (epa.py:167-187)
//   validation        every horizon vertex starts and ends exactly one edge,
//                     and the edges form one loop (pointer jumping): the
//                     visible faces are a disk, so the new faces close the
//                     surface again
//   new faces         one per horizon edge, in the slots the visible faces
//                     freed (then fresh slots), with their adjacency set from
//                     the loop order (epa.py:126-146)
//
// Faces keep their three vertex ids, unit normal and offset, and the ids of
// the faces across their three edges; winding is outward by construction, as
// in epa_mixed.cu.  A pair whose polytope fails validation (degenerate face,
// horizon not one loop, more horizon edges than max_loose_edges) goes to the
// fallback list.  The converged face is refined along its FP32 normal with
// FP64 supports: in a second pass, one pair per thread (k_epa_refine), or in
// the search kernel itself (refine_face) when the caller gives no list for
// that pass.
//
// The same search is instantiated with an FP64 polytope and exact FP64
// supports.  It takes the FP32 search's fallback pairs: the plane tests
// behind a pinched horizon are FP32 noise on nearly coplanar faces, which
// FP64 resolves.  Its own fallback pairs go to the serial FP64 EPA (the
// reference's arithmetic).  Compiled with -fmad=true.
#include "capi_util.h"
#include "epa_mixed.cuh"
#include "epa_mixed.h"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned kDead = 0xffffffffu;  // vertex word of a free face slot

// xyz + w of the polytope's precision (16-byte aligned)
template <typename T>
struct alignas(16) Q4 {
    T x, y, z, w;
};

template <typename T>
__device__ __forceinline__ Q4<T> q4(T x, T y, T z, T w) {
    return Q4<T>{x, y, z, w};
}

template <typename T>
__device__ __forceinline__ T eps_of();
template <>
__device__ __forceinline__ float eps_of<float>() { return FLT_EPSILON; }
template <>
__device__ __forceinline__ double eps_of<double>() { return DBL_EPSILON; }

// Storage bounds of one polytope.  The search adds one vertex per iteration
// (nv <= max_iterations + 4) and keeps a closed triangulated surface (the
// visible faces are validated to be a disk), so its live faces number
// 2 V - 4 <= 2 nv - 4 for its V <= nv vertices in use (Euler), and a horizon
// loop visits distinct vertices (ne <= nv).  The face slots and horizon
// edges are bounded by those numbers as well as by max_faces and
// max_loose_edges; the search checks both bounds before it writes.
__host__ __device__ inline int vertex_cap(const d3d_epa_options& o) { return o.max_iterations + 4; }
__host__ __device__ inline int face_cap(const d3d_epa_options& o) {
    const int euler = 2 * vertex_cap(o) - 4;
    return o.max_faces < euler ? o.max_faces : euler;
}
__host__ __device__ inline int edge_cap(const d3d_epa_options& o) {
    const int e = o.max_loose_edges < vertex_cap(o) ? o.max_loose_edges : vertex_cap(o);
    return e > 0 ? e : 1;
}

// Byte offsets of one warp's polytope in shared memory.
struct Layout {
    int vy, fn, fv, adj, hz, freel, vis, se, ee, bytes;
};

template <typename T>
__host__ __device__ inline Layout layout_for(const d3d_epa_options& o) {
    const int nv = vertex_cap(o), F = face_cap(o), E = edge_cap(o);
    const int q = (int)sizeof(Q4<T>);
    Layout L;
    int p = 0;
    L.vy = p;
    p += q * nv;
    L.fn = p;
    p += q * F;
    L.adj = p;
    p += 8 * F;
    L.hz = p;
    p += 8 * E;
    L.fv = p;
    p += 4 * F;
    L.vis = p;
    p += 4 * F;
    L.freel = p;
    p += 2 * F;
    L.se = p;
    p += nv;
    L.ee = p;
    p += nv;
    L.bytes = (p + 15) & ~15;
    return L;
}

template <typename T>
struct Poly {
    Q4<T>* vy;             // vertex y.xyz
    Q4<T>* fn;             // unit normal .xyz, w = offset n . y_a
    ushort4* adj;          // faces across edges (a,b), (b,c), (c,a)
    int2* hz;              // horizon edge e: x = a | b << 8 | k << 16 (edge k of g faces it), y = g
    unsigned* fv;          // a | b << 8 | c << 16, kDead for a free slot
    unsigned short* freel; // free face slots (stack)
    int* vis;              // iteration stamp of the faces found visible
    unsigned char* se;     // horizon edge that starts at vertex v
    unsigned char* ee;     // horizon edge that ends at vertex v
};

template <typename T>
__device__ __forceinline__ Poly<T> poly_at(unsigned char* base, const Layout& L) {
    Poly<T> P;
    P.vy = reinterpret_cast<Q4<T>*>(base + L.vy);
    P.fn = reinterpret_cast<Q4<T>*>(base + L.fn);
    P.adj = reinterpret_cast<ushort4*>(base + L.adj);
    P.hz = reinterpret_cast<int2*>(base + L.hz);
    P.fv = reinterpret_cast<unsigned*>(base + L.fv);
    P.freel = reinterpret_cast<unsigned short*>(base + L.freel);
    P.vis = reinterpret_cast<int*>(base + L.vis);
    P.se = base + L.se;
    P.ee = base + L.ee;
    return P;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

template <typename T>
__device__ __forceinline__ V3<T> yv(const Poly<T>& P, int v) {
    const Q4<T> a = P.vy[v];
    return mk(a.x, a.y, a.z);
}

// Index of the first maximum of V . d over a polytope's vertices, the 16
// lanes of a half warp (mask hm) taking every 16th vertex (same products as
// hull_argmax, same winner).
template <typename T>
__device__ __forceinline__ int half_argmax(const T* verts, int off, int nv, V3<T> d, unsigned hm) {
    T best = T(0);
    int bi = -1;
    for (int k = lane_id() & 15; k < nv; k += 16) {
        const V3<T> v = load_vertex(verts, off + k);
        const T s = dot102(v.x, v.y, v.z, d.x, d.y, d.z);
        if (bi < 0 || s > best) {
            best = s;
            bi = k;
        }
    }
#pragma unroll
    for (int m = 8; m; m >>= 1) {
        const T ob = __shfl_xor_sync(hm, best, m);
        const int oi = __shfl_xor_sync(hm, bi, m);
        if (oi >= 0 && (bi < 0 || ob > best || (ob == best && oi < bi))) {
            best = ob;
            bi = oi;
        }
    }
    return bi;
}

// The FP32 instance with two warp reductions on order-preserving keys: the
// largest product, then the lowest index holding it (-0 counts as +0; a NaN
// product loses to every number).
template <>
__device__ __forceinline__ int half_argmax<float>(const float* verts, int off, int nv, f3 d, unsigned hm) {
    unsigned best = 0u;
    int bi = 0x7fffffff;
    bool any = false;
    for (int k = lane_id() & 15; k < nv; k += 16) {
        const f3 v = load_vertex(verts, off + k);
        const float x = dot102(v.x, v.y, v.z, d.x, d.y, d.z);
        const unsigned u = x == 0.f ? 0u : __float_as_uint(x);
        const unsigned key = x != x ? 0u : ((u & 0x80000000u) ? ~u : (u | 0x80000000u));
        if (!any || key > best) {
            best = key;
            bi = k;
            any = true;
        }
    }
    const unsigned m = __reduce_max_sync(hm, any ? best : 0u);
    return (int)__reduce_min_sync(hm, (any && best == m) ? (unsigned)bi : 0xffffffffu);
}

__device__ __forceinline__ unsigned half_mask() { return (lane_id() & 16) ? 0xffff0000u : 0x0000ffffu; }

// w = s_a(d) - s_b(-d) in FP32: the lower half warp evaluates collider a, the
// upper half collider b, together; every lane returns w.
template <bool MESH>
__device__ __forceinline__ f3 minkowski32(const d3d_store& st, int a, int b, f3 d) {
    const bool up = lane_id() & 16;
    Col<float> c;
    load_col(st, up ? b : a, c);
    const f3 dd = up ? -d : d;
    f3 s;
    if (c.type == D3D_BOX || c.type == D3D_HULL) {
        if (c.nv < 1)
            s = mk(NAN, NAN, NAN);
        else
            s = margin_fast(st, c, load_vertex(st.verts32, c.off + (c.nv == 1 ? 0 : half_argmax(st.verts32, c.off, c.nv, dd, half_mask()))), dd);
    } else {
        s = FastSupportT<MESH>::eval(c, st, dd);
    }
    const f3 o = mk(__shfl_xor_sync(kFull, s.x, 16), __shfl_xor_sync(kFull, s.y, 16), __shfl_xor_sync(kFull, s.z, 16));
    return up ? o - s : s - o;
}

// w in FP64 with the reference's supports (the polytope argmax in FP64), for
// the FP64 polytope.
__device__ __forceinline__ d3 minkowski64_exact(const d3d_store& st, int a, int b, d3 d) {
    const bool up = lane_id() & 16;
    Col<double> c;
    load_col(st, up ? b : a, c);
    const d3 dd = up ? -d : d;
    d3 s;
    if (c.type == D3D_BOX || c.type == D3D_HULL) {
        if (c.nv < 1)
            s = mk(double(NAN), double(NAN), double(NAN));
        else
            s = add_margin(c, load_vertex(st.verts64, c.off + (c.nv == 1 ? 0 : half_argmax(st.verts64, c.off, c.nv, dd, half_mask()))), dd);
    } else {
        s = support(c, st, dd);
    }
    const d3 o = mk(__shfl_xor_sync(kFull, s.x, 16), __shfl_xor_sync(kFull, s.y, 16), __shfl_xor_sync(kFull, s.z, 16));
    return up ? o - s : s - o;
}

// The polytope's precision: FP32 search on the FP32 mirror, or FP64 with the
// reference's supports.
template <bool MESH>
__device__ __forceinline__ f3 minkowski_of(const d3d_store& st, int a, int b, f3 d);
template <bool MESH>
__device__ __forceinline__ d3 minkowski_of(const d3d_store& st, int a, int b, d3 d) {
    return minkowski64_exact(st, a, b, d);
}

// The same in FP64 with RefineSupport (polytope vertex chosen by the FP32
// argmax of the rounded direction).
template <bool MESH>
__device__ __forceinline__ d3 minkowski64(const d3d_store& st, int a, int b, d3 d) {
    const bool up = lane_id() & 16;
    Col<double> c;
    load_col(st, up ? b : a, c);
    const d3 dd = up ? -d : d;
    d3 s;
    if (c.type == D3D_BOX || c.type == D3D_HULL) {
        if (c.nv < 1) {
            s = mk(double(NAN), double(NAN), double(NAN));
        } else {
            const f3 df = mk(__double2float_rn(dd.x), __double2float_rn(dd.y), __double2float_rn(dd.z));
            s = margin_fast(
                st, c, load_vertex(st.verts64, c.off + (c.nv == 1 ? 0 : half_argmax(st.verts32, c.off, c.nv, df, half_mask()))),
                dd);
        }
    } else {
        s = RefineSupportT<MESH>::eval(c, st, dd);
    }
    const d3 o = mk(__shfl_xor_sync(kFull, s.x, 16), __shfl_xor_sync(kFull, s.y, 16), __shfl_xor_sync(kFull, s.z, 16));
    return up ? o - s : s - o;
}

// exclusive prefix sum over lanes
__device__ __forceinline__ int warp_excl(int x) {
    int s = x;
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        const int t = __shfl_up_sync(kFull, s, m);
        if (lane_id() >= m) s += t;
    }
    return s - x;
}

template <bool MESH>
__device__ __forceinline__ f3 minkowski_of(const d3d_store& st, int a, int b, f3 d) {
    return minkowski32<MESH>(st, a, b, d);
}

// unit normal and offset of face (a, b, c); false if degenerate
template <typename T>
__device__ __forceinline__ bool plane_of(const Poly<T>& P, int a, int b, int c, Q4<T>& out) {
    const V3<T> ya = yv(P, a), yb = yv(P, b), yc = yv(P, c);
    V3<T> n = cross(yb - ya, yc - ya);
    const T l = sqrt_t(dot(n, n));
    if (!(l > T(0))) return false;
    n = n * (T(1) / l);
    out = q4(n.x, n.y, n.z, dot(ya, n));
    return true;
}

__device__ __forceinline__ unsigned pack3(int a, int b, int c) { return (unsigned)a | ((unsigned)b << 8) | ((unsigned)c << 16); }
__device__ __forceinline__ int vid(unsigned w, int j) { return (int)((w >> (8 * j)) & 0xffu); }
__device__ __forceinline__ int adj_at(ushort4 g, int j) { return j == 0 ? g.x : (j == 1 ? g.y : g.z); }

// Closest live face: (offset, slot), ties to the lower slot.
template <typename T>
__device__ __forceinline__ int closest_face(const Poly<T>& P, int nslots) {
    T bd = T(0);
    int bs = -1;
    for (int f = lane_id(); f < nslots; f += 32) {
        if (P.fv[f] == kDead) continue;
        const T d = P.fn[f].w;
        if (bs < 0 || d < bd) {
            bd = d;
            bs = f;
        }
    }
#pragma unroll
    for (int m = 16; m; m >>= 1) {
        const T od = __shfl_xor_sync(kFull, bd, m);
        const int os = __shfl_xor_sync(kFull, bs, m);
        if (os >= 0 && (bs < 0 || od < bd || (od == bd && os < bs))) {
            bd = od;
            bs = os;
        }
    }
    return bs;
}

// The same for the FP32 polytope with two warp reductions (REDUX) on
// order-preserving 32-bit keys of the offsets instead of five shuffle rounds:
// the smallest key, then the lowest slot holding it.  (-0 counts as +0; a NaN
// offset loses to every number.)
template <>
__device__ __forceinline__ int closest_face<float>(const Poly<float>& P, int nslots) {
    unsigned best = 0xffffffffu;
    int bs = 0x7fffffff;
    for (int f = lane_id(); f < nslots; f += 32) {
        if (P.fv[f] == kDead) continue;
        const float d = P.fn[f].w;
        const unsigned u = d == 0.f ? 0u : __float_as_uint(d);
        const unsigned key = d != d ? 0xfffffffeu : ((u & 0x80000000u) ? ~u : (u | 0x80000000u));
        if (key < best) {
            best = key;
            bs = f;
        }
    }
    const unsigned m = __reduce_min_sync(kFull, best);
    if (m == 0xffffffffu) return -1;
    return (int)__reduce_min_sync(kFull, best == m ? (unsigned)bs : 0xffffffffu);
}

// Outcome of the FP32 search for one pair.
struct Search {
    int status;   // a D3D status, or kEpaFallback
    int closest;  // face slot refined for OK / NOT_CONVERGED
    int nslots;
    int live;
};

// The expanding-polytope search for one pair in the polytope's precision T
// (uniform across the warp).
template <typename T, bool MESH>
__device__ Search search_pair(const Poly<T>& P, const d3d_store& st, int a, int b, const double* simplex,
                              const d3d_epa_options& o) {
    const int ln = lane_id();
    Search R{kEpaFallback, 0, 0, 0};
    // starting tetrahedron: the FP64 simplex (rounded to T)
    T scale = T(0);
    if (ln < 4) {
        const V3<T> y = mk((T)simplex[3 * ln], (T)simplex[3 * ln + 1], (T)simplex[3 * ln + 2]);
        P.vy[ln] = q4(y.x, y.y, y.z, T(0));
        scale = sqrt_t(dot(y, y));
    }
#pragma unroll
    for (int m = 16; m; m >>= 1) scale = maxf2(scale, (T)__shfl_xor_sync(kFull, scale, m));
    __syncwarp();
    // faces ABC, ACD, ADB, BDC, each wound away from the vertex it leaves out
    bool bad = false;
    if (ln < 4) {
        const int t = ln == 0 ? 0x3210 : (ln == 1 ? 0x1320 : (ln == 2 ? 0x2130 : 0x0231));
        int fa = t & 15, fb = (t >> 4) & 15;
        const int fc = (t >> 8) & 15, fd = (t >> 12) & 15;
        Q4<T> pl;
        if (!plane_of(P, fa, fb, fc, pl)) {
            bad = true;
        } else {
            const V3<T> yd = yv(P, fd) - yv(P, fa);
            if (pl.x * yd.x + pl.y * yd.y + pl.z * yd.z > T(0)) {
                const int s = fa;
                fa = fb;
                fb = s;
                pl = q4(-pl.x, -pl.y, -pl.z, -pl.w);
            }
            P.fv[ln] = pack3(fa, fb, fc);
            P.fn[ln] = pl;
            P.vis[ln] = 0;
        }
    }
    if (__any_sync(kFull, bad)) return R;
    __syncwarp();
    // adjacency of the tetrahedron: the face across (u, v) holds (v, u)
    if (ln < 12) {
        const int f = ln / 3, j = ln % 3;
        const unsigned w = P.fv[f];
        const int u = vid(w, j), v = vid(w, (j + 1) % 3);
        int g = -1;
        for (int h = 0; h < 4; ++h) {
            if (h == f) continue;
            const unsigned x = P.fv[h];
            for (int i = 0; i < 3; ++i)
                if (vid(x, i) == v && vid(x, (i + 1) % 3) == u) g = h;
        }
        if (g < 0) {
            bad = true;
        } else {
            unsigned short* ap = reinterpret_cast<unsigned short*>(&P.adj[f]);
            ap[j] = (unsigned short)g;
        }
    }
    if (__any_sync(kFull, bad)) return R;
    __syncwarp();

    const T vis_eps = (T)o.epsilon;  // the reference's visibility test
    int nslots = 4, nfree = 0, live = 4, nv = 4, it = 0;
    while (true) {
        const int cf = closest_face(P, nslots);
        R.closest = cf;
        R.nslots = nslots;
        R.live = live;
        if (cf < 0) {
            R.status = D3D_STATUS_EPA_DEGENERATE;
            return R;
        }
        if (it >= o.max_iterations) {
            R.status = D3D_STATUS_EPA_NOT_CONVERGED;
            return R;
        }
        ++it;
        const Q4<T> cn = P.fn[cf];
        const V3<T> sd = mk(cn.x, cn.y, cn.z);
        const V3<T> w = minkowski_of<MESH>(st, a, b, sd);
        scale = maxf2(scale, sqrt_t(dot(w, w)));
        const T eps = maxf2((T)o.epsilon, T(kSearchUlps) * eps_of<T>() * scale);
        if (dot(w, sd) - cn.w < eps) {
            R.status = D3D_STATUS_OK;
            return R;
        }
        if (nv >= o.max_iterations + 4) {
            R.status = D3D_STATUS_EPA_NOT_CONVERGED;
            return R;
        }
        const int vn = nv++;
        const int stamp = it;
        // Faces that see w: breadth first from the closest face over the
        // adjacency.  The visible faces are listed where they are about to
        // go, on the free list above its current top.
        unsigned short* const vl = P.freel + nfree;
        if (ln == 0) {
            P.vy[vn] = q4(w.x, w.y, w.z, T(0));
            P.vis[cf] = stamp;
            vl[0] = (unsigned short)cf;
        }
        __syncwarp();
        int head = 0, nvis = 1;
        while (head < nvis) {
            const int nc = 3 * (nvis - head);
            int added = 0;
            for (int i0 = 0; i0 < nc; i0 += 32) {
                const int i = i0 + ln;
                bool take = false;
                int g = 0;
                if (i < nc) {
                    g = adj_at(P.adj[vl[head + i / 3]], i % 3);
                    if (P.vis[g] != stamp) {
                        // w above the face's plane: n . w - n . y_a (the offset kept with the normal)
                        const Q4<T> pl = P.fn[g];
                        if (dot(mk(pl.x, pl.y, pl.z), w) - pl.w > vis_eps)
                            take = atomicExch(&P.vis[g], stamp) != stamp;
                    }
                }
                const unsigned m = __ballot_sync(kFull, take);
                if (take) vl[nvis + added + __popc(m & ((1u << ln) - 1u))] = (unsigned short)g;
                added += __popc(m);
            }
            __syncwarp();
            head = nvis;
            nvis += added;
        }
        // horizon: edges of visible faces whose neighbour is not visible (a
        // single visible face: its own three edges, in order)
        int ne = 3;
        if (nvis == 1) {
            if (3 > o.max_loose_edges) return R;
            if (ln < 3) {
                const unsigned fw = P.fv[cf];
                const int h = adj_at(P.adj[cf], ln);
                const ushort4 gh = P.adj[h];
                const int k = gh.x == cf ? 0 : (gh.y == cf ? 1 : 2);
                P.hz[ln] = make_int2(vid(fw, ln) | (vid(fw, (ln + 1) % 3) << 8) | (k << 16), h);
            }
        } else {
            int ne_l = 0;
            for (int i = ln; i < 3 * nvis; i += 32) ne_l += P.vis[adj_at(P.adj[vl[i / 3]], i % 3)] != stamp;
            int eb = warp_excl(ne_l);
            ne = __shfl_sync(kFull, eb + ne_l, 31);
            // more than edge_cap(o) < max_loose_edges edges: not one loop
            if (ne > o.max_loose_edges || ne > edge_cap(o) || ne < 3) return R;
            for (int i = ln; i < 3 * nvis; i += 32) {
                const int f = vl[i / 3], j = i % 3;
                const int h = adj_at(P.adj[f], j);
                if (P.vis[h] == stamp) continue;
                const unsigned fw = P.fv[f];
                const ushort4 gh = P.adj[h];
                const int k = gh.x == f ? 0 : (gh.y == f ? 1 : 2);
                P.hz[eb++] = make_int2(vid(fw, j) | (vid(fw, (j + 1) % 3) << 8) | (k << 16), h);
            }
        }
        __syncwarp();
        for (int i = ln; i < nvis; i += 32) P.fv[vl[i]] = kDead;
        __syncwarp();
        // The horizon must be one loop.  A single visible face gives its own
        // three edges, in order.  Otherwise: unique start and end per vertex ...
        if (nvis > 1) {
            for (int e = ln; e < ne; e += 32) {
                const int x = P.hz[e].x;
                P.se[x & 0xff] = (unsigned char)e;
                P.ee[(x >> 8) & 0xff] = (unsigned char)e;
            }
            __syncwarp();
            bool ok = true;
            for (int e = ln; e < ne; e += 32) {
                const int x = P.hz[e].x;
                const int nx = P.se[(x >> 8) & 0xff];
                ok &= P.se[x & 0xff] == e && P.ee[(x >> 8) & 0xff] == e && nx < ne &&
                      (P.hz[nx].x & 0xff) == ((x >> 8) & 0xff);
            }
            if (!__all_sync(kFull, ok)) return R;
            // ... and following next(e) from edge 0 visits every edge once
            if (ne <= 32) {
                int nxt = ln < ne ? P.se[(P.hz[ln].x >> 8) & 0xff] : ln;
                int lab = ln < ne ? ln : 0;
#pragma unroll
                for (int r = 0; r < 5; ++r) {
                    lab = min(lab, __shfl_sync(kFull, lab, nxt));
                    nxt = __shfl_sync(kFull, nxt, nxt);
                }
                ok = lab == 0;
            } else {
                int steps = 0, cur = 0;
                if (ln == 0) {
                    do {
                        cur = P.se[(P.hz[cur].x >> 8) & 0xff];
                        ++steps;
                    } while (cur != 0 && steps <= ne);
                }
                ok = __shfl_sync(kFull, steps == ne && cur == 0, 0);
            }
            if (!__all_sync(kFull, ok)) return R;
        }
        const int nlive = live - nvis + ne;
        if (nlive > o.max_faces) {
            R.status = D3D_STATUS_EPA_FACE_OVERFLOW;
            R.live = live - nvis;
            return R;
        }
        // new faces (a, b, w): slots from the top of the free list, then fresh
        const int nft = nfree + nvis;
        if (ne > nft && nslots + (ne - nft) > face_cap(o)) return R;  // beyond the Euler bound: never for a closed surface
        for (int e = ln; e < ne; e += 32) {
            const int2 h = P.hz[e];
            const int ea = h.x & 0xff, eb2 = (h.x >> 8) & 0xff, k = (h.x >> 16) & 3;
            const int nx = nvis == 1 ? (e == 2 ? 0 : e + 1) : P.se[eb2];
            const int pv = nvis == 1 ? (e == 0 ? 2 : e - 1) : P.ee[ea];
            const int s = e < nft ? P.freel[nft - 1 - e] : nslots + (e - nft);
            const int sn = nx < nft ? P.freel[nft - 1 - nx] : nslots + (nx - nft);
            const int sp = pv < nft ? P.freel[nft - 1 - pv] : nslots + (pv - nft);
            Q4<T> pl;
            if (!plane_of(P, ea, eb2, vn, pl)) bad = true;
            P.fn[s] = pl;
            P.fv[s] = pack3(ea, eb2, vn);
            P.adj[s] = make_ushort4((unsigned short)h.y, (unsigned short)sn, (unsigned short)sp, 0);
            P.vis[s] = 0;
            reinterpret_cast<unsigned short*>(&P.adj[h.y])[k] = (unsigned short)s;
        }
        if (__any_sync(kFull, bad)) return R;
        nslots = ne > nft ? nslots + (ne - nft) : nslots;
        nfree = ne < nft ? nft - ne : 0;
        live = nlive;
        __syncwarp();
    }
}

// FP64 refinement of face f: its FP32 unit normal, renormalised in FP64,
// n, and the depth along it from FP64 supports, mtv = n (n . w(n)) (the
// reference's expression at convergence, epa.py:69).  n . w(n) is the support
// depth h(n), an upper bound on the penetration depth for every n, and the
// FP32 normal of the converged face is within the search's tolerance of the
// optimal direction.
template <bool MESH>
__device__ __forceinline__ d3 refine_face(const Poly<float>& P, const d3d_store& st, int a, int b, int f) {
    const Q4<float> fn = P.fn[f];
    d3 n = mk((double)fn.x, (double)fn.y, (double)fn.z);
    n = n * (1.0 / sqrt(dot(n, n)));
    const d3 w = minkowski64<MESH>(st, a, b, n);
    return n * dot(w, n);
}

// The FP64 polytope's face: its own unit normal and the reference's supports.
template <bool MESH>
__device__ __forceinline__ d3 refine_face(const Poly<double>& P, const d3d_store& st, int a, int b, int f) {
    const Q4<double> fn = P.fn[f];
    const d3 n = mk(fn.x, fn.y, fn.z);
    const d3 w = minkowski64_exact(st, a, b, n);
    return n * dot(w, n);
}

// Resident warps per SM the register budget is set for: the FP32 search runs
// 32 (64 registers, a few spilled: latency hiding outweighs the spills), the
// FP64 search, which takes few pairs, 16.
template <typename T>
constexpr int kWarpsPerSm = sizeof(T) == 4 ? 32 : 16;

template <typename T, int WARPS, bool MESH>
__global__ void __launch_bounds__(32 * WARPS, kWarpsPerSm<T> / WARPS) k_epa_warp(d3d_store st, const int32_t* __restrict__ i1,
                                                          const int32_t* __restrict__ i2,
                                                          const int32_t* __restrict__ list, int64_t n,
                                                          const unsigned long long* __restrict__ n_dev,
                                                          unsigned long long* __restrict__ cursor,
                                                          const double* __restrict__ simplex, d3d_epa_options o,
                                                          double* __restrict__ mtv, int8_t* __restrict__ status,
                                                          int32_t* __restrict__ n_faces, double* __restrict__ faces,
                                                          int32_t* __restrict__ fallback,
                                                          unsigned long long* __restrict__ n_fallback,
                                                          int32_t* __restrict__ refine,
                                                          unsigned long long* __restrict__ n_refine) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Layout L = layout_for<T>(o);
    const Poly<T> P = poly_at<T>(smem + (threadIdx.x >> 5) * L.bytes, L);
    const int ln = lane_id();
    if (n_dev) n = (int64_t)*n_dev;
    while (true) {
        long long slot = 0;
        if (ln == 0) slot = (long long)atomicAdd(cursor, 1ull);
        slot = __shfl_sync(kFull, slot, 0);
        if (slot >= n) break;
        const int64_t k = list ? list[slot] : slot;
        const int a = i1[k], b = i2[k];
        if (!pair_ok(st, a, b)) {  // the same for every lane
            if (ln == 0) epa_store_bad_index(mtv, status, n_faces, k);
            __syncwarp();
            continue;
        }
        const double* sx = simplex + 12 * k;
        const Search R = search_pair<T, MESH>(P, st, a, b, sx, o);
        if (R.status == kEpaFallback) {
            if (ln == 0) fallback[atomicAdd(n_fallback, 1ull)] = (int32_t)k;
            __syncwarp();
            continue;
        }
        d3 m = mk(double(NAN), double(NAN), double(NAN));
        const bool ended = R.status == D3D_STATUS_OK || R.status == D3D_STATUS_EPA_NOT_CONVERGED;
        if (ended) {
            if (refine) {
                // the face's normal now; the FP64 depth along it in k_epa_refine
                const Q4<T> q = P.fn[R.closest];
                m = mk((double)q.x, (double)q.y, (double)q.z);
            } else {
                m = refine_face<MESH>(P, st, a, b, R.closest);
            }
        }
        const int nf = R.status == D3D_STATUS_EPA_DEGENERATE ? 0 : R.live;
        if (ln == 0) {
            mtv[3 * k] = m.x;
            mtv[3 * k + 1] = m.y;
            mtv[3 * k + 2] = m.z;
            status[k] = (int8_t)R.status;
            n_faces[k] = nf;
            if (refine && ended) refine[atomicAdd(n_refine, 1ull)] = (int32_t)k;
        }
        if (faces && nf > 0) {
            // live faces in slot order: three vertices and the normal
            double* out = faces + k * 12 * (int64_t)o.max_faces;
            int base = 0;
            for (int f0 = 0; f0 < R.nslots; f0 += 32) {
                const int f = f0 + ln;
                const bool live = f < R.nslots && P.fv[f] != kDead;
                const unsigned mask = __ballot_sync(kFull, live);
                if (live) {
                    double* q = out + 12 * (base + __popc(mask & ((1u << ln) - 1u)));
                    const unsigned fw = P.fv[f];
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const Q4<T> yy = P.vy[vid(fw, j)];
                        q[3 * j] = yy.x;
                        q[3 * j + 1] = yy.y;
                        q[3 * j + 2] = yy.z;
                    }
                    const Q4<T> pl = P.fn[f];
                    q[9] = pl.x;
                    q[10] = pl.y;
                    q[11] = pl.z;
                }
                base += __popc(mask);
            }
        }
        __syncwarp();
    }
}

// The FP64 refinement of the FP32 search's converged faces (refine_face),
// one pair per thread: the normal the search left in mtv, renormalised in
// FP64, and mtv = n (n . w(n)) with RefineSupport.  In the search kernel the
// whole warp waited on each pair's FP64 support chain.
template <bool MESH>
__global__ void __launch_bounds__(128) k_epa_refine(d3d_store st, const int32_t* __restrict__ i1,
                                                    const int32_t* __restrict__ i2, const int32_t* __restrict__ list,
                                                    const unsigned long long* __restrict__ n_dev,
                                                    double* __restrict__ mtv) {
    const int64_t n = (int64_t)*n_dev;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = list[j];
        d3 nrm = mk(mtv[3 * k], mtv[3 * k + 1], mtv[3 * k + 2]);
        nrm = nrm * (1.0 / sqrt(dot(nrm, nrm)));
        d3 p, q;
        pair_supports<double, RefineSupportT<MESH>>(st, i1[k], i2[k], nrm, p, q);
        const d3 m = nrm * dot(p - q, nrm);
        mtv[3 * k] = m.x;
        mtv[3 * k + 1] = m.y;
        mtv[3 * k + 2] = m.z;
    }
}

}  // namespace

namespace {

template <typename T, int WARPS, bool MESH>
int launch_warp(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                int32_t* fallback, unsigned long long* n_fallback, int32_t* refine, unsigned long long* n_refine,
                cudaStream_t stream) {
    const void* fn = (const void*)k_epa_warp<T, WARPS, MESH>;
    const int smem = layout_for<T>(o).bytes * WARPS;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) {
        set_error("d3d_epa (mixed): %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    const int blocks = persistent_blocks(fn, 32 * WARPS, n * 32, 0, smem);
    k_epa_warp<T, WARPS, MESH><<<blocks, 32 * WARPS, smem, stream>>>(store, i1, i2, list, n, n_dev, cursor, simplex,
                                                                     o, mtv, status, n_faces, faces, fallback,
                                                                     n_fallback, refine, n_refine);
    int rc = check_launch("d3d_epa (mixed)");
    if (rc || !refine) return rc;
    const void* kr = (const void*)k_epa_refine<MESH>;
    k_epa_refine<MESH><<<persistent_blocks(kr, 128, n), 128, 0, stream>>>(store, i1, i2, refine, n_refine, mtv);
    return check_launch("d3d_epa (mixed, refinement)");
}

// The kernels without the MeshGraph branch serve stores without meshes.
template <typename T, int WARPS>
int launch_warp(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                int32_t* fallback, unsigned long long* n_fallback, int32_t* refine, unsigned long long* n_refine,
                cudaStream_t stream) {
    if (store.n_links > 0)
        return launch_warp<T, WARPS, true>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces,
                                           faces, fallback, n_fallback, refine, n_refine, stream);
    return launch_warp<T, WARPS, false>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces,
                                        faces, fallback, n_fallback, refine, n_refine, stream);
}

}  // namespace

namespace d3d {

constexpr int64_t kSmemPerBlock = 227 * 1024;

bool epa_warp_supported(const d3d_epa_options& o, bool fp64) {
    if (o.max_iterations > 250 || o.max_loose_edges > 255 || o.max_faces > 65535) return false;
    const int bytes = fp64 ? layout_for<double>(o).bytes : layout_for<float>(o).bytes;
    return (int64_t)bytes * 2 <= kSmemPerBlock;
}

int epa_warp_launch(const d3d_store& store, const int32_t* i1, const int32_t* i2, const int32_t* list, int64_t n,
                    const unsigned long long* n_dev, unsigned long long* cursor, const double* simplex,
                    const d3d_epa_options& o, double* mtv, int8_t* status, int32_t* n_faces, double* faces,
                    int32_t* fallback, unsigned long long* n_fallback, cudaStream_t stream, bool fp64,
                    int32_t* refine, unsigned long long* n_refine) {
    // pairs per block as tuned, fewer if their polytopes do not fit in one block
    const int64_t bytes = fp64 ? layout_for<double>(o).bytes : layout_for<float>(o).bytes;
    int w = tuning().epa_warps;
    while (w > 2 && bytes * w > kSmemPerBlock) w /= 2;
#define D3D_WARP_LAUNCH(T, W)                                                                                      \
    return launch_warp<T, W>(store, i1, i2, list, n, n_dev, cursor, simplex, o, mtv, status, n_faces, faces, fallback, \
                             n_fallback, refine, n_refine, stream)
    if (fp64) {
        refine = nullptr;  // the FP64 search refines with exact supports itself
        if (w == 2) D3D_WARP_LAUNCH(double, 2);
        if (w == 8) D3D_WARP_LAUNCH(double, 8);
        D3D_WARP_LAUNCH(double, 4);
    }
    if (w == 2) D3D_WARP_LAUNCH(float, 2);
    if (w == 8) D3D_WARP_LAUNCH(float, 8);
    D3D_WARP_LAUNCH(float, 4);
#undef D3D_WARP_LAUNCH
}

}  // namespace d3d
