// mpr.cuh -- Minkowski portal refinement (distance3d mpr.py:21-110) as a
// per-lane state machine with one support evaluation per round, in the
// search precision T.  The FP64 drop-in (mpr.cu, -fmad=false) instantiates
// it with T = double and the reference's supports; the mixed form
// (mpr_mixed.cu) with T = float on the FP32 mirror, followed by an FP64
// evaluation of the final portal.
#pragma once

#include "jolt.cuh"

namespace d3d {
namespace mpr {

constexpr double kEps = DBL_EPSILON;

// utils.py:12-30
template <typename T>
__device__ __forceinline__ V3<T> norm_vector(V3<T> v) {
    const T n = sqrt_t(dot(v, v));
    return n == T(0) ? v : mk(v.x / n, v.y / n, v.z / n);
}

template <typename T>
__device__ __forceinline__ bool all_zero(V3<T> v) {
    return v.x == T(0) && v.y == T(0) && v.z == T(0);
}

// colliders.py center(): the pose translation, a hull's vertex mean
// (np.mean(axis=0): rows summed in order, then divided by the count), a
// mesh's vertex mean posed (:224-226), a cone's mid-axis point (:582-584);
// Margin passes through (:633-634).
template <typename T>
__device__ V3<T> collider_center(const d3d_store& st, int idx) {
    Col<T> c;
    load_col(st, idx, c);
    if (c.type == D3D_HULL || c.type == D3D_MESH) {
        if (c.nv < 1) return mk(T(NAN), T(NAN), T(NAN));
        const T* verts = store_verts(st, T(0));
        V3<T> s = load_vertex(verts, c.off);
        for (int k = 1; k < c.nv; ++k) s = s + load_vertex(verts, c.off + k);
        const T n = (T)c.nv;
        const V3<T> m = mk(s.x / n, s.y / n, s.z / n);
        return c.type == D3D_MESH ? xform(c.R, c.t, m) : m;
    }
    const V3<T> t = mk(c.t[0], c.t[1], c.t[2]);
    if (c.type == D3D_CONE) {
        const T f = T(0.5) * c.p[1];
        return t + mk(f * c.R[2], f * c.R[5], f * c.R[8]);
    }
    return t;
}

// The portal rows of one lane in shared memory (column stride BLOCK): vertex
// r of the Minkowski difference, and either the support points of the two
// colliders behind it (AB, the FP64 form) or the search direction that
// produced it (the FP32 search, whose final portal is evaluated again in
// FP64 along those directions).  Row 0 is the centers' difference.
template <typename T, int BLOCK, bool AB>
struct Portal {
    static constexpr int kVecs = AB ? 3 : 2;
    static constexpr int kWords = 4 * kVecs * 3;  // per lane
    T* base;
    __device__ T& at(int which, int r, int c) const { return base[((which * 4 + r) * 3 + c) * BLOCK]; }
    __device__ V3<T> get(int which, int r) const { return mk(at(which, r, 0), at(which, r, 1), at(which, r, 2)); }
    __device__ void put(int which, int r, V3<T> x) const {
        at(which, r, 0) = x.x;
        at(which, r, 1) = x.y;
        at(which, r, 2) = x.z;
    }
    __device__ V3<T> v(int r) const { return get(0, r); }
    __device__ V3<T> a(int r) const { return get(1, r); }
    __device__ V3<T> b(int r) const { return get(2, r); }
    __device__ V3<T> dir(int r) const { return get(1, r); }
    // row r from the supports pa, pb along d (minkowski.py:52-55)
    __device__ void set(int r, V3<T> pa, V3<T> pb, V3<T> d) const {
        put(0, r, pa - pb);
        if (AB) {
            put(1, r, pa);
            put(2, r, pb);
        } else {
            put(1, r, d);
        }
    }
    __device__ void set_center(V3<T> v0, V3<T> c1, V3<T> c2) const {
        put(0, 0, v0);
        if (AB) {
            put(1, 0, c1);
            put(2, 0, c2);
        }
    }
    __device__ void copy(int dst, int src) const {
        for (int w = 0; w < kVecs; ++w) put(w, dst, get(w, src));
    }
};

// :276-281
template <typename P>
__device__ __forceinline__ auto portal_direction(const P& Pt) {
    const auto v1 = Pt.v(1);
    return norm_vector(cross(Pt.v(2) - v1, Pt.v(3) - v1));
}

// :290-299: min over rows 1-3 of v4 . d - v_r . d (v[1:].dot(d) is a gemv)
template <typename T, typename P>
__device__ __forceinline__ bool reach_tolerance(const P& Pt, V3<T> v4, V3<T> d, double tol) {
    const T s4 = dot(v4, d);
    T m = T(0);
    for (int r = 1; r < 4; ++r) {
        const V3<T> v = Pt.v(r);
        const T e = s4 - dot102(v.x, v.y, v.z, d.x, d.y, d.z);
        if (r == 1 || e < m) m = e;
    }
    return m < T(tol + kEps);
}

// :302-317
template <typename T, typename P>
__device__ __forceinline__ void expand(const P& Pt, V3<T> pa, V3<T> pb, V3<T> d) {
    const V3<T> v4 = pa - pb;
    const V3<T> c = cross(v4, Pt.v(0));
    int r;
    if (dot(Pt.v(1), c) > T(0))
        r = dot(Pt.v(2), c) > T(0) ? 1 : 3;
    else
        r = dot(Pt.v(3), c) > T(0) ? 2 : 1;
    Pt.set(r, pa, pb, d);
}

// The test of :188-191 for the origin on the line of v0 and v1.  In FP64 the
// reference's absolute EPSILON; in FP32 also the FP32 noise of |v0 x v1|^2,
// so that the collinear case is recognised as it is in FP64.
__device__ __forceinline__ double collinear_eps(d3, d3) { return kEps; }
__device__ __forceinline__ float collinear_eps(f3 v0, f3 v1) {
    const float e = 8.f * FLT_EPSILON;
    return fmaxf((float)kEps, e * e * dot(v0, v0) * dot(v1, v1));
}

// The phases of one pair, each ending in one support evaluation.
enum Phase { kV1 = 0, kV2, kDiscover, kRefine, kPenetrate };

// One lane's pair between rounds.
template <typename T>
struct Lane {
    V3<T> d;  // direction of the next support evaluation
    int phase;
    int it;
};

// Outcome of a round.
enum Outcome { kRunning = -1, kMiss = 0, kHitV1 = 1, kHitSegment = 2, kHitPortal = 3 };

// Start a pair (:161-185): origin ray from the centers c1 - c2 (nudged off
// the origin), first direction towards the origin.
template <typename T, typename P>
__device__ __forceinline__ void begin(const P& Pt, Lane<T>& L, V3<T> c1, V3<T> c2) {
    V3<T> v0 = c1 - c2;
    if (all_zero(v0)) v0.x += T(kEps * 10.0);
    Pt.set_center(v0, c1, c2);
    L.d = norm_vector(-v0);
    L.phase = kV1;
    L.it = 0;
}

// Enter the refinement (:243-273) with the portal built: true if the portal
// already encloses the origin, else the first refinement support is next.
template <typename T, typename P>
__device__ __forceinline__ bool enter_refine(const P& Pt, Lane<T>& L) {
    L.d = portal_direction(Pt);
    if (dot(Pt.v(1), L.d) > T(-10.0 * kEps)) return true;
    L.phase = kRefine;
    L.it = 0;
    return false;
}

// Process the support points (pa, pb) along L.d for the lane's phase
// (:123-158 with :161-240, :243-273, :320-334).  Returns kRunning, kMiss
// (status may be D3D_STATUS_MAX_ITER), kHitV1 / kHitSegment (origin on v1 or
// on the segment v0-v1, :337-352), or kHitPortal (the portal encloses the
// origin; with penetration, the search has also ended).
template <typename T, typename P>
__device__ int round(const P& Pt, Lane<T>& L, V3<T> pa, V3<T> pb, const d3d_mpr_options& opt, int& status) {
    const V3<T> v0 = Pt.v(0);
    const T eps = T(kEps);
    switch (L.phase) {
    case kV1: {  // :177-201
        Pt.set(1, pa, pb, L.d);
        const V3<T> v1 = Pt.v(1);
        if (!all_zero(v1) && dot(v1, L.d) < eps) return kMiss;
        const V3<T> d = cross(v0, v1);
        if (dot(d, d) < collinear_eps(v0, v1)) return all_zero(v1) ? kHitV1 : kHitSegment;
        L.d = norm_vector(d);
        L.phase = kV2;
        return kRunning;
    }
    case kV2: {  // :198-210; the reference's row swap (:232-240) keeps row 1
                 // as a NumPy view, so both rows end up holding the old row 2
        Pt.set(2, pa, pb, L.d);
        if (dot(Pt.v(2), L.d) < eps) return kMiss;
        L.d = norm_vector(cross(Pt.v(1) - v0, Pt.v(2) - v0));
        if (dot(L.d, v0) > T(0)) {
            Pt.copy(1, 2);
            L.d = L.d * T(-1);
        }
        L.phase = kDiscover;
        L.it = 0;
        return kRunning;
    }
    case kDiscover: {  // :145-158, :213-229
        Pt.set(3, pa, pb, L.d);
        const V3<T> v3 = Pt.v(3);
        if (dot(v3, L.d) < eps) return kMiss;
        bool cont = false;
        if (dot(cross(Pt.v(1), v3), v0) < eps) {
            Pt.copy(2, 3);
            cont = true;
        }
        if (!cont && dot(cross(v3, Pt.v(2)), v0) < eps) {
            Pt.copy(1, 3);
            cont = true;
        }
        if (cont) L.d = norm_vector(cross(Pt.v(1) - v0, Pt.v(2) - v0));
        if (cont && ++L.it < opt.max_iterations) return kRunning;
        if (!enter_refine(Pt, L)) return kRunning;
        break;  // the built portal encloses the origin
    }
    case kRefine: {  // :243-273, bounded
        const V3<T> v4 = pa - pb;
        if (!(dot(v4, L.d) > T(-10.0 * kEps)) || reach_tolerance(Pt, v4, L.d, opt.tolerance)) return kMiss;
        if (L.it >= opt.refine_limit) {
            status = D3D_STATUS_MAX_ITER;
            return kMiss;
        }
        expand(Pt, pa, pb, L.d);
        ++L.it;
        L.d = portal_direction(Pt);
        if (!(dot(Pt.v(1), L.d) > T(-10.0 * kEps))) return kRunning;
        break;  // the origin is inside
    }
    default: {  // kPenetrate, :320-334
        if (reach_tolerance(Pt, pa - pb, L.d, opt.tolerance) || L.it > opt.max_iterations) return kHitPortal;
        expand(Pt, pa, pb, L.d);
        ++L.it;
        L.d = portal_direction(Pt);
        return kRunning;
    }
    }
    // the portal encloses the origin
    if (!opt.penetration) return kHitPortal;
    L.phase = kPenetrate;
    L.it = 0;
    L.d = portal_direction(Pt);
    return kRunning;
}

// distance/_triangle.py:12-89 point_to_triangle for the origin
__device__ inline double origin_to_triangle(d3 A, d3 B, d3 C, d3& cp) {
    const d3 o = mk(0.0, 0.0, 0.0);
    const d3 ab = B - A, ac = C - A;
    const d3 ap = o - A;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        cp = A;
    } else {
        const d3 bp = o - B;
        const double d3_ = dot(ab, bp), d4 = dot(ac, bp);
        if (d3_ >= 0.0 && d4 <= d3_) {
            cp = B;
        } else {
            const double vc = d1 * d4 - d3_ * d2;
            if (vc <= 0.0 && 0.0 <= d1 && d3_ <= 0.0) {
                cp = A + ab * (d1 / (d1 - d3_));
            } else {
                const d3 q = o - C;
                const double d5 = dot(ab, q), d6 = dot(ac, q);
                if (d6 >= 0.0 && d5 <= d6) {
                    cp = C;
                } else {
                    const double vb = d5 * d2 - d1 * d6;
                    if (vb <= 0.0 && 0.0 <= d2 && d6 <= 0.0) {
                        cp = A + ac * (d2 / (d2 - d6));
                    } else {
                        const double va = d3_ * d6 - d5 * d4;
                        if (va <= 0.0 && 0.0 <= d4 - d3_ && d5 - d6 >= 0.0) {
                            cp = B + (C - B) * ((d4 - d3_) / ((d4 - d3_) + (d5 - d6)));
                        } else {
                            const double denom = 1.0 / ((va + vb) + vc);
                            cp = (A + ab * (vb * denom)) + ac * (vc * denom);
                        }
                    }
                }
            }
        }
    }
    const d3 r = o - cp;
    return sqrt(dot(r, r));
}

// :372-393 _contact_position: barycentric weights of the origin (np.sum in
// order; b.dot(V) through gemv: fma(b0,V0,b1*V1) + fma(b2,V2,b3*V3)).  R
// gives the FP64 rows: v(k), a(k), b(k).
template <typename R>
__device__ inline d3 contact_position(const R& P, d3 d) {
    const d3 v0 = P.v(0), v1 = P.v(1), v2 = P.v(2), v3 = P.v(3);
    double w0 = dot(cross(v1, v2), v3), w1 = dot(cross(v3, v2), v0), w2 = dot(cross(v0, v1), v3),
           w3 = dot(cross(v2, v1), v0);
    double sum = ((w0 + w1) + w2) + w3;
    if (sum < kEps) {
        w0 = 0.0;
        w1 = dot(cross(v2, v3), d);
        w2 = dot(cross(v3, v1), d);
        w3 = dot(cross(v1, v2), d);
        sum = ((w0 + w1) + w2) + w3;
    }
    w0 = w0 / sum;
    w1 = w1 / sum;
    w2 = w2 / sum;
    w3 = w3 / sum;
    const d3 a0 = P.a(0), a1 = P.a(1), a2 = P.a(2), a3 = P.a(3);
    const d3 p1 = mk(fma(w0, a0.x, w1 * a1.x) + fma(w2, a2.x, w3 * a3.x),
                     fma(w0, a0.y, w1 * a1.y) + fma(w2, a2.y, w3 * a3.y),
                     fma(w0, a0.z, w1 * a1.z) + fma(w2, a2.z, w3 * a3.z));
    const d3 b0 = P.b(0), b1 = P.b(1), b2 = P.b(2), b3 = P.b(3);
    const d3 p2 = mk(fma(w0, b0.x, w1 * b1.x) + fma(w2, b2.x, w3 * b3.x),
                     fma(w0, b0.y, w1 * b1.y) + fma(w2, b2.y, w3 * b3.y),
                     fma(w0, b0.z, w1 * b1.z) + fma(w2, b2.z, w3 * b3.z));
    return mk(0.5 * (p1.x + p2.x), 0.5 * (p1.y + p2.y), 0.5 * (p1.z + p2.z));
}

// The result of a hit with penetration (:337-362) from the FP64 portal rows
// (row 0: the centers): depth, unit direction (zero if touching), contact
// position.
template <typename R>
__device__ inline void penetration(int outcome, const R& P, double& depth, d3& dir, d3& pos) {
    const d3 v1 = P.v(1);
    if (outcome == kHitV1 || outcome == kHitSegment) {
        pos = (P.a(1) + P.b(1)) * 0.5;
        if (outcome == kHitV1) {
            depth = 0.0;
            dir = mk(0.0, 0.0, 0.0);
        } else {
            depth = sqrt(dot(v1, v1));
            dir = norm_vector(v1);
        }
        return;
    }
    d3 cp;
    depth = origin_to_triangle(v1, P.v(2), P.v(3), cp);
    if (fabs(depth) < kEps) cp = mk(0.0, 0.0, 0.0);
    pos = contact_position(P, norm_vector(cross(P.v(2) - v1, P.v(3) - v1)));
    dir = norm_vector(cp);
}

struct Out {
    int8_t* hit;
    double* depth;
    double* dir;
    double* pos;
    int8_t* status;
};

__device__ __forceinline__ void put3(double* p, int64_t k, d3 x) {
    if (!p) return;
    p[3 * k] = x.x;
    p[3 * k + 1] = x.y;
    p[3 * k + 2] = x.z;
}

// Write pair k's result; depth / dir / pos only with penetration (NaN for a
// miss).
__device__ __forceinline__ void store(const Out& o, int64_t k, bool hit, int status, bool pen, double depth, d3 dir,
                                      d3 pos) {
    o.hit[k] = hit ? 1 : 0;
    o.status[k] = (int8_t)status;
    if (!pen) return;
    if (!hit) {
        depth = NAN;
        dir = pos = mk(double(NAN), double(NAN), double(NAN));
    }
    if (o.depth) o.depth[k] = depth;
    put3(o.dir, k, dir);
    put3(o.pos, k, pos);
}

}  // namespace mpr
}  // namespace d3d
