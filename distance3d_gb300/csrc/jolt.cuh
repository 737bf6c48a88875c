// jolt.cuh -- Jolt / van den Bergen GJK on the device, one thread per pair.
//
// The simplex lives in registers: Y (Minkowski-difference points), P and Q
// (support points on each collider), four rows each, indexed only by
// compile-time constants after unrolling.  Sub-algorithms follow
// distance3d gjk/_gjk_jolt.py (cited per function); all thresholds come in
// through JoltEps so the FP32 phase of the mixed form can scale them.
#pragma once

#include "d3d_device.cuh"

namespace d3d {

template <typename T>
__device__ __forceinline__ T maxf2(T a, T b) { return a > b ? a : b; }

template <typename T>
__device__ __forceinline__ T maxf();
template <>
__device__ __forceinline__ double maxf<double>() { return DBL_MAX; }
template <>
__device__ __forceinline__ float maxf<float>() { return FLT_MAX; }

// Thresholds.  The reference uses one constant, EPSILON = DBL_EPSILON
// (utils.py:8), in four roles; the FP64 form sets all of them from it, the
// FP32 phase of the mixed form scales each role to single precision.
template <typename T>
struct JoltEps {
    T plane;  // |plane determinant| (_gjk_jolt.py:339,358) and tetrahedron side tests (:565-567)
    T sq;     // EPSILON^2: degenerate segment / triangle (:18, :299, :450)
    T conv;   // relative progress that counts as converged (:127, :283)
    T isect;  // |v|^2 <= isect * max|Y|^2 counts as touching (:115, :270)
    T point;  // dist below this: closest points merged (:219)
};

template <typename T>
__device__ __forceinline__ JoltEps<T> reference_eps() {
    T e = T(DBL_EPSILON);
    return JoltEps<T>{e, e * e, e, e, e};
}

// _gjk_jolt.py:292-312
template <typename T>
__device__ __forceinline__ void bary_line(V3<T> a, V3<T> b, const JoltEps<T>& E, T& u, T& v) {
    V3<T> ab = b - a;
    T den = dot(ab, ab);
    if (den < E.sq) {
        if (dot(a, a) < dot(b, b)) {
            u = T(1);
            v = T(0);
        } else {
            u = T(0);
            v = T(1);
        }
    } else {
        v = -dot(a, ab) / den;
        u = T(1) - v;
    }
}

// _gjk_jolt.py:316-372.  The reference tests the determinant against an
// absolute EPSILON, so a well-shaped triangle with edges below ~1e-8 counts as
// degenerate and is reduced to an edge; SCALED makes the test relative to the
// product of the squared edge lengths (the mixed form's final simplices are
// that small, being built around an accurate FP32 direction).
template <typename T, bool SCALED = false>
__device__ __forceinline__ void bary_plane(V3<T> a, V3<T> b, V3<T> c, const JoltEps<T>& E, T& u, T& v, T& w) {
    V3<T> v0 = b - a, v1 = c - a, v2 = c - b;
    T d00 = dot(v0, v0), d11 = dot(v1, v1), d22 = dot(v2, v2);
    if (d00 <= d22) {
        T d01 = dot(v0, v1);
        T den = d00 * d11 - d01 * d01;
        if (abs_t(den) < (SCALED ? E.plane * (d00 * d11) : E.plane)) {
            if (d00 > d11) {
                bary_line(a, b, E, u, v);
                w = T(0);
            } else {
                bary_line(a, c, E, u, w);
                v = T(0);
            }
        } else {
            T a0 = dot(a, v0), a1 = dot(a, v1);
            v = (d01 * a1 - d11 * a0) / den;
            w = (d01 * a0 - d00 * a1) / den;
            u = T(1) - v - w;
        }
    } else {
        T d12 = dot(v1, v2);
        T den = d11 * d22 - d12 * d12;
        if (abs_t(den) < (SCALED ? E.plane * (d11 * d22) : E.plane)) {
            if (d11 > d22) {
                bary_line(a, c, E, u, w);
                v = T(0);
            } else {
                bary_line(b, c, E, v, w);
                u = T(0);
            }
        } else {
            T c1 = dot(c, v1), c2 = dot(c, v2);
            u = (d22 * c1 - d12 * c2) / den;
            v = (d11 * c2 - d12 * c1) / den;
            w = T(1) - u - v;
        }
    }
}

// scalar triple product a . (b x c), utils.py:33-73
template <typename T>
__device__ __forceinline__ T stp(V3<T> a, V3<T> b, V3<T> c) { return dot(a, cross(b, c)); }

// _gjk_jolt.py:376-390
template <typename T>
__device__ __forceinline__ void bary_tetra(V3<T> a, V3<T> b, V3<T> c, V3<T> d, T* o) {
    V3<T> vab = b - a, vac = c - a, vad = d - a;
    T va6 = -stp(b, d - b, c - b);
    T vb6 = -stp(a, vac, vad);
    T vc6 = -stp(a, vad, vab);
    T vd6 = -stp(a, vab, vac);
    T v6 = T(1) / stp(vab, vac, vad);
    o[0] = va6 * v6;
    o[1] = vb6 * v6;
    o[2] = vc6 * v6;
    o[3] = vd6 * v6;
}

// _gjk_jolt.py:394-412
template <typename T>
__device__ __forceinline__ V3<T> cp_line(V3<T> a, V3<T> b, const JoltEps<T>& E, int& set) {
    T u, v;
    bary_line(a, b, E, u, v);
    if (v <= T(0)) {
        set = 1;
        return a;
    }
    if (u <= T(0)) {
        set = 2;
        return b;
    }
    set = 3;
    return a * u + b * v;
}

// _gjk_jolt.py:416-523.  FAST (the mixed form only) divides once in the face
// projection instead of per component.
template <typename T, bool FAST = false>
__device__ __forceinline__ V3<T> cp_triangle(V3<T> a, V3<T> b, V3<T> c, const JoltEps<T>& E, int& set) {
    V3<T> ab = b - a, ac = c - a, bc = c - b;
    V3<T> n = (dot(bc, bc) < dot(ac, ac)) ? cross(ab, bc) : cross(ab, ac);
    T nl = dot(n, n);
    if (nl < E.sq) {
        int s, ns;
        V3<T> cp = cp_line(a, b, E, s);
        T best = dot(cp, cp);
        V3<T> q = cp_line(a, c, E, ns);
        T d2 = dot(q, q);
        if (d2 < best) {
            cp = q;
            best = d2;
            s = (ns & 1) + ((ns & 2) << 1);
        }
        q = cp_line(b, c, E, ns);
        d2 = dot(q, q);
        if (d2 < best) {
            cp = q;
            s = ns << 1;
        }
        set = s;
        return cp;
    }
    V3<T> ap = -a;
    T d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= T(0) && d2 <= T(0)) {
        set = 1;
        return a;
    }
    V3<T> bp = -b;
    T d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= T(0) && d4 <= d3) {
        set = 2;
        return b;
    }
    T vc = d1 * d4 - d3 * d2;
    if (vc <= T(0) && T(0) <= d1 && d3 <= T(0)) {
        T v = d1 / (d1 - d3);
        set = 3;
        return a + ab * v;
    }
    V3<T> cpp = -c;
    T d5 = dot(ab, cpp), d6 = dot(ac, cpp);
    if (d6 >= T(0) && d5 <= d6) {
        set = 4;
        return c;
    }
    T vb = d5 * d2 - d1 * d6;
    if (vb <= T(0) && T(0) <= d2 && d6 <= T(0)) {
        T w = d2 / (d2 - d6);
        set = 5;
        return a + ac * w;
    }
    T va = d3 * d6 - d5 * d4;
    T d43 = d4 - d3, d56 = d5 - d6;
    if (va <= T(0) && T(0) <= d43 && d56 >= T(0)) {
        T w = d43 / (d43 + d56);
        set = 6;
        return b + bc * w;
    }
    set = 7;
    // n * (a + b + c).dot(n) / (3.0 * n_len_sq), left to right
    T s = dot((a + b) + c, n);
    T den = T(3) * nl;
    if (FAST) {
        const T f = s / den;
        return mk(n.x * f, n.y * f, n.z * f);
    }
    return mk(n.x * s / den, n.y * s / den, n.z * s / den);
}

// _gjk_jolt.py:527-570; returns a 4-bit mask of "origin outside plane i"
template <typename T>
__device__ __forceinline__ int outside_planes(V3<T> a, V3<T> b, V3<T> c, V3<T> d, const JoltEps<T>& E) {
    V3<T> ab = b - a, ac = c - a, ad = d - a, bd = d - b, bc = c - b;
    V3<T> abac = cross(ab, ac), acad = cross(ac, ad), adab = cross(ad, ab), bdbc = cross(bd, bc);
    T sp0 = dot(a, abac), sp1 = dot(a, acad), sp2 = dot(a, adab), sp3 = dot(b, bdbc);
    T sd0 = dot(ad, abac), sd1 = dot(ab, acad), sd2 = dot(ac, adab), sd3 = -dot(ab, bdbc);
    if (sd0 > T(0) && sd1 > T(0) && sd2 > T(0) && sd3 > T(0))
        return (sp0 >= -E.plane) | ((sp1 >= -E.plane) << 1) | ((sp2 >= -E.plane) << 2) | ((sp3 >= -E.plane) << 3);
    if (sd0 < T(0) && sd1 < T(0) && sd2 < T(0) && sd3 < T(0))
        return (sp0 <= E.plane) | ((sp1 <= E.plane) << 1) | ((sp2 <= E.plane) << 2) | ((sp3 <= E.plane) << 3);
    return 15;
}

// Where a simplex keeps its P and Q rows (the support points on each collider;
// the solve reads only Y).  RegRows: registers, indexed by compile-time
// constants after unrolling.  SmemRows: this lane's column of a shared-memory
// block, six values per row strided by the block size, so that the FP64
// kernels hold only Y in registers.
template <typename T>
struct RegRows {
    V3<T> P[4], Q[4];
    __device__ __forceinline__ void put(int k, V3<T> p, V3<T> q) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j == k) {
                P[j] = p;
                Q[j] = q;
            }
    }
    __device__ __forceinline__ void move(int dst, int src) {
        P[dst] = P[src];
        Q[dst] = Q[src];
    }
    __device__ __forceinline__ V3<T> p(int k) const { return P[k]; }
    __device__ __forceinline__ V3<T> q(int k) const { return Q[k]; }
};

template <typename T, int kStride>
struct SmemRows {
    T* base;  // element e (0..5: p.xyz, q.xyz) of row r at base[(6 r + e) kStride]
    __device__ __forceinline__ T& at(int r, int e) const { return base[(6 * r + e) * kStride]; }
    __device__ __forceinline__ void put(int k, V3<T> p, V3<T> q) {
        at(k, 0) = p.x;
        at(k, 1) = p.y;
        at(k, 2) = p.z;
        at(k, 3) = q.x;
        at(k, 4) = q.y;
        at(k, 5) = q.z;
    }
    __device__ __forceinline__ void move(int dst, int src) {
#pragma unroll
        for (int e = 0; e < 6; ++e) at(dst, e) = at(src, e);
    }
    __device__ __forceinline__ V3<T> p(int k) const { return mk(at(k, 0), at(k, 1), at(k, 2)); }
    __device__ __forceinline__ V3<T> q(int k) const { return mk(at(k, 3), at(k, 4), at(k, 5)); }
};

// Simplex: rows 0..n-1 of Y (Minkowski-difference points, registers) and of
// P, Q (in Rows).
template <typename T, typename Rows = RegRows<T>>
struct Simplex {
    V3<T> Y[4];
    Rows R;
    int n;
};

// Y rows cleared (rows GJK never writes are reported as zero); P and Q rows
// are only read below n.
template <typename T, typename Rows>
__device__ __forceinline__ void simplex_clear(Simplex<T, Rows>& S) {
#pragma unroll
    for (int k = 0; k < 4; ++k) S.Y[k] = mk(T(0), T(0), T(0));
    S.n = 0;
}

template <typename T, typename Rows>
__device__ __forceinline__ void simplex_push(Simplex<T, Rows>& S, V3<T> w, V3<T> p, V3<T> q) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k == S.n) S.Y[k] = w;
    S.R.put(S.n, p, q);
    ++S.n;
}

// keep the rows whose bit is set, in order (_gjk_jolt.py:655-664); rows at
// and above the new count keep their old contents, as in the reference
template <typename T, bool WITH_PQ, typename Rows>
__device__ __forceinline__ void simplex_compact(Simplex<T, Rows>& S, int set) {
    int m = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i < S.n && ((set >> i) & 1)) {
#pragma unroll
            for (int j = 0; j <= i; ++j)
                if (j == m && j != i) {
                    S.Y[j] = S.Y[i];
                    if (WITH_PQ) S.R.move(j, i);
                }
            ++m;
        }
    }
    S.n = m;
}

// Row k of a register-resident array (k < 4) without dynamic indexing.
template <typename T>
__device__ __forceinline__ V3<T> row_of(const V3<T>* Y, int k) {
    V3<T> r = Y[0];
    if (k == 1) r = Y[1];
    if (k == 2) r = Y[2];
    if (k == 3) r = Y[3];
    return r;
}

// _gjk_jolt.py:691-711: closest point of the simplex to the origin; true iff
// its squared length is below prev (NaN compares false).
//
// Triangles and tetrahedra share one face loop: a triangle is its own single
// face, a tetrahedron contributes the faces whose plane has the origin on the
// outside (_gjk_jolt.py:574-631: faces abc, acd, adb, bdc in that order, the
// first tested face taken unconditionally, later ones only if strictly
// closer).  Lanes of a warp holding simplices of 3 and 4 rows therefore run
// cp_triangle together instead of in separate branches.
//
// (Reconverging the lanes inside this function as well -- after the plane
// tests and in every round of the face loop -- measured slower than leaving
// it to the compiler: 4.83 against 4.69 ms for the mixed GJK at 1M pairs.)
template <typename T, typename Rows, bool FAST = false>
__device__ __forceinline__ bool closest_to_origin(const Simplex<T, Rows>& S, T prev, const JoltEps<T>& E, V3<T>& v,
                                                  T& vl, int& set) {
    V3<T> r = S.Y[0];
    int s = 1;
    if (S.n == 2) {
        r = cp_line(S.Y[0], S.Y[1], E, s);
    } else if (S.n >= 3) {
        int faces = S.n == 3 ? 1 : outside_planes(S.Y[0], S.Y[1], S.Y[2], S.Y[3], E);
        r = mk(T(0), T(0), T(0));
        s = 15;
        T best = maxf<T>();
        while (faces) {
            const int f = __ffs(faces) - 1;
            faces &= faces - 1;
            // corners of face f: (0,1,2) (0,2,3) (0,3,1) (1,3,2)
            const int i0 = f == 3 ? 1 : 0;
            const int i1 = f == 0 ? 1 : (f == 1 ? 2 : 3);
            const int i2 = f == 0 ? 2 : (f == 1 ? 3 : (f == 2 ? 1 : 2));
            int ns;
            const V3<T> q = cp_triangle<T, FAST>(row_of(S.Y, i0), row_of(S.Y, i1), row_of(S.Y, i2), E, ns);
            const T d2 = dot(q, q);
            if (f == 0 || d2 < best) {
                best = d2;
                r = q;
                s = ((ns & 1) << i0) | (((ns >> 1) & 1) << i1) | (((ns >> 2) & 1) << i2);
            }
        }
    }
    T l = dot(r, r);
    if (l < prev) {
        v = r;
        vl = l;
        set = s;
        return true;
    }
    return false;
}

// _gjk_jolt.py:635-640
template <typename T, typename Rows>
__device__ __forceinline__ T max_y_len_sq(const Simplex<T, Rows>& S) {
    T m = dot(S.Y[0], S.Y[0]);
#pragma unroll
    for (int i = 1; i < 4; ++i)
        if (i < S.n) {
            T l = dot(S.Y[i], S.Y[i]);
            if (l > m) m = l;
        }
    return m;
}

// _gjk_jolt.py:668-687 (SCALED: see bary_plane)
template <typename T, bool SCALED = false, typename Rows>
__device__ __forceinline__ void closest_points(const Simplex<T, Rows>& S, const JoltEps<T>& E, V3<T>& a, V3<T>& b) {
    switch (S.n) {
    case 1:
        a = S.R.p(0);
        b = S.R.q(0);
        break;
    case 2: {
        T u, v;
        bary_line(S.Y[0], S.Y[1], E, u, v);
        a = S.R.p(0) * u + S.R.p(1) * v;
        b = S.R.q(0) * u + S.R.q(1) * v;
        break;
    }
    case 3: {
        T u, v, w;
        bary_plane<T, SCALED>(S.Y[0], S.Y[1], S.Y[2], E, u, v, w);
        a = (S.R.p(0) * u + S.R.p(1) * v) + S.R.p(2) * w;
        b = (S.R.q(0) * u + S.R.q(1) * v) + S.R.q(2) * w;
        break;
    }
    default: {
        T o[4];
        bary_tetra(S.Y[0], S.Y[1], S.Y[2], S.Y[3], o);
        a = ((S.R.p(0) * o[0] + S.R.p(1) * o[1]) + S.R.p(2) * o[2]) + S.R.p(3) * o[3];
        b = ((S.R.q(0) * o[0] + S.R.q(1) * o[1]) + S.R.q(2) * o[2]) + S.R.q(3) * o[3];
        break;
    }
    }
}

enum GjkEnd { GJK_NO_INTERSECTION = 0, GJK_INTERSECTION = 1, GJK_CLIPPED = 3 };


// Support evaluated in the loop's own precision (the reference's function).
struct ExactSupport {
    template <typename T>
    static __device__ __forceinline__ V3<T> eval(const Col<T>& c, const d3d_store& s, V3<T> d) {
        return support(c, s, d);
    }
};

// Support points p of collider a along d and q of collider b along -d.  The
// records are read from the store (L1-resident) inside a two-trip loop, so
// the support code exists once per kernel and holds no registers across the
// simplex solve.
template <typename T, typename Sup>
__device__ __forceinline__ void pair_supports(const d3d_store& st, int a, int b, V3<T> d, V3<T>& p, V3<T>& q) {
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        Col<T> c;
        load_col(st, k ? b : a, c);
        const V3<T> x = Sup::eval(c, st, k ? -d : d);
        if (k)
            q = x;
        else
            p = x;
    }
}

// The same with the reference's supports and a MeshGraph vertex cache per
// collider (cache[0] for a, cache[1] for b; see base_support).
template <typename T>
__device__ __forceinline__ void pair_supports_cached(const d3d_store& st, int a, int b, V3<T> d, V3<T>& p, V3<T>& q,
                                                     int* cache) {
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        Col<T> c;
        load_col(st, k ? b : a, c);
        const V3<T> x = support(c, st, k ? -d : d, cache + k);
        if (k)
            q = x;
        else
            p = x;
    }
}

template <typename T>
struct GjkResult {
    T dist;
    V3<T> a, b;
    int status;
    int iters;
};

// State of one pair's Jolt GJK distance loop between iterations.
enum { GJK_RUNNING = -1 };
template <typename T, typename Rows = RegRows<T>>
struct GjkLoop {
    Simplex<T, Rows> S;
    V3<T> dir;  // next search direction
    T vl;       // v_len_sq as the reference keeps it
    T prev;     // prev_v_len_sq
    int it;
    int state;   // GJK_RUNNING or a GjkEnd value once finished
    int status;  // D3D_STATUS_OK or D3D_STATUS_MAX_ITER
};

// Start the loop.  S must already hold the starting simplex (n = 0 for the
// reference's cold start, dir = (1,0,0), vl = 1, prev = MAX_FLOAT).
template <typename T, typename Rows>
__device__ __forceinline__ void gjk_begin(GjkLoop<T, Rows>& g, V3<T> dir, T vl, T prev) {
    g.dir = dir;
    g.vl = vl;
    g.prev = prev;
    g.it = 0;
    g.state = GJK_RUNNING;
    g.status = D3D_STATUS_OK;
}

// One iteration of gjk_distance_jolt's loop (_gjk_jolt.py:200-210) with
// _distance_loop (:224-288) inlined; returns true once the loop has ended.
//
// GAP adds the duality-gap termination of van den Bergen's GJK, which the
// reference does not have: with v the current closest point and w the new
// support point along -v, |v| - (|v|^2 - v.w) / |v| <= distance <= |v|.  The
// loop stops once that bracket is within rel_gap |v| (relative) or within
// sqrt(abs_gap2) max(1, |w|) (absolute, on the scene's scale).  The FP64
// drop-in is compiled without it.  A non-null `mesh_cache` (two ints) takes
// the reference's supports with MeshGraph vertex caching
// (pair_supports_cached) instead of Sup.
template <typename T, typename Sup = ExactSupport, bool GAP = false, typename Rows>
__device__ __forceinline__ bool gjk_step_begin(GjkLoop<T, Rows>& g, const d3d_store& st, int a, int b, T max_d2,
                                               int max_iter, T rel_gap = T(0), T abs_gap2 = T(0),
                                               int* mesh_cache = nullptr) {
    if (g.it >= max_iter) {
        g.status = D3D_STATUS_MAX_ITER;
        g.state = GJK_NO_INTERSECTION;
        return true;
    }
    ++g.it;
    const unsigned together = __activemask();
    V3<T> p, q;
    if (mesh_cache)
        pair_supports_cached<T>(st, a, b, g.dir, p, q, mesh_cache);
    else
        pair_supports<T, Sup>(st, a, b, g.dir, p, q);
    // The supports branch by collider type and polytope size; without this
    // the lanes would reach the simplex solve in the groups those branches
    // left and run it once per group.
    __syncwarp(together);
    V3<T> w = p - q;
    T dd = dot(g.dir, w);
    if (dd < T(0) && dd * dd > g.vl * max_d2) {
        g.state = GJK_CLIPPED;
        return true;
    }
    if (GAP && g.S.n > 0) {
        // gap = |v|^2 - v.w >= 0 (up to rounding): |v| - gap / |v| <= distance <= |v|
        const T gap = g.vl + dd;
        if (gap <= rel_gap * g.vl || gap * gap <= abs_gap2 * maxf2(T(1), dot(w, w)) * g.vl) {
            g.dir = -g.dir;  // the state the reference leaves on convergence
            g.state = GJK_NO_INTERSECTION;
            return true;
        }
    }
    simplex_push(g.S, w, p, q);
    return false;
}

// The rest of the iteration, given the result of
// closest_to_origin(g.S, g.prev, E, nv, nl, set) (`closer`: its return value).
template <typename T, typename Rows>
__device__ __forceinline__ bool gjk_step_end(GjkLoop<T, Rows>& g, T tol_sq, const JoltEps<T>& E, bool closer,
                                             V3<T> nv, T nl, int set) {
    if (closer) {
        g.dir = nv;
        g.vl = nl;
    } else {
        --g.S.n;
        set = (1 << g.S.n) - 1;
    }
    if (set == 15) {
        g.vl = T(0);
        g.state = GJK_INTERSECTION;
        return true;
    }
    simplex_compact<T, true>(g.S, set);
    if (g.vl <= tol_sq || g.vl <= E.isect * max_y_len_sq(g.S)) {
        g.vl = T(0);
        g.state = GJK_INTERSECTION;
        return true;
    }
    g.dir = -g.dir;
    if (g.prev - g.vl <= E.conv * g.prev) {
        g.state = GJK_NO_INTERSECTION;
        return true;
    }
    g.prev = g.vl;
    return false;
}

// One iteration: gjk_step_begin, the simplex solve, gjk_step_end (kernels
// that solve the simplices of a block together call the halves themselves).
template <typename T, typename Sup = ExactSupport, bool GAP = false, typename Rows>
__device__ __forceinline__ bool gjk_step(GjkLoop<T, Rows>& g, const d3d_store& st, int a, int b, T tol_sq, T max_d2,
                                         int max_iter, const JoltEps<T>& E, T rel_gap = T(0), T abs_gap2 = T(0),
                                         int* mesh_cache = nullptr) {
    if (gjk_step_begin<T, Sup, GAP>(g, st, a, b, max_d2, max_iter, rel_gap, abs_gap2, mesh_cache)) return true;
    V3<T> nv = mk(T(0), T(0), T(0));
    T nl = T(0);
    int set = 0;
    const bool closer = closest_to_origin(g.S, g.prev, E, nv, nl, set);
    return gjk_step_end(g, tol_sq, E, closer, nv, nl, set);
}

// After the loop: closest points, sanity check, distance
// (_gjk_jolt.py:209-221).
template <typename T, bool SCALED = false, typename Rows>
__device__ __forceinline__ void gjk_end(const GjkLoop<T, Rows>& g, T sanity, const JoltEps<T>& E, GjkResult<T>& out) {
    out.iters = g.it;
    out.status = g.status;
    if (g.state == GJK_CLIPPED) {
        out.status = D3D_STATUS_CLIPPED;
        return;
    }
    V3<T> a, b;
    closest_points<T, SCALED>(g.S, E, a, b);
    T check = abs_t(dot(g.dir, g.dir) - g.vl);
    if (!(check < sanity) && out.status == D3D_STATUS_OK) out.status = D3D_STATUS_SANITY;
    T dist = sqrt_t(g.vl);
    if (dist < E.point) {
        V3<T> m = (a + b) * T(0.5);
        a = m;
        b = m;
    }
    out.dist = dist;
    out.a = a;
    out.b = b;
}

// The rest of the loop for one pair, from the state gjk_begin (and any
// starting simplex) left in g: gjk_distance_jolt (_gjk_jolt.py:138-221).
template <typename T, typename Sup = ExactSupport, bool GAP = false, bool SCALED = false, typename Rows>
__device__ __forceinline__ void gjk_run(GjkLoop<T, Rows>& g, const d3d_store& st, int a, int b, T tol_sq, T max_d2,
                                        T sanity, int max_iter, const JoltEps<T>& E, GjkResult<T>& out,
                                        T rel_gap = T(0), T abs_gap2 = T(0)) {
    while (!gjk_step<T, Sup, GAP>(g, st, a, b, tol_sq, max_d2, max_iter, E, rel_gap, abs_gap2)) {
    }
    gjk_end<T, SCALED>(g, sanity, E, out);
}

// gjk_intersection_jolt, _gjk_jolt.py:29-135.  Returns 1 on intersection.
template <typename T, typename Sup = ExactSupport>
__device__ __forceinline__ int gjk_intersection_loop(const d3d_store& st, int a, int b, T tol_sq, int max_iter,
                                                     const JoltEps<T>& E, int& status) {
    Simplex<T> S;
    simplex_clear(S);
    T prev = maxf<T>();
    V3<T> dir = mk(T(1), T(0), T(0));
    status = D3D_STATUS_OK;
    for (int it = 1;; ++it) {
        if (it > max_iter) {
            status = D3D_STATUS_MAX_ITER;
            return 0;
        }
        V3<T> p, q;
        pair_supports<T, Sup>(st, a, b, dir, p, q);
        V3<T> w = p - q;
        if (dot(dir, w) < -E.conv) return 0;
        simplex_push(S, w, p, q);
        V3<T> nv;
        T vl;
        int set;
        if (!closest_to_origin(S, prev, E, nv, vl, set)) return 0;
        dir = nv;
        if (set == 15) return 1;
        if (vl <= tol_sq) return 1;
        if (vl <= E.isect * max_y_len_sq(S)) return 1;
        dir = -dir;
        if (prev - vl <= E.conv * prev) return 0;
        prev = vl;
        simplex_compact<T, false>(S, set);
    }
}

}  // namespace d3d
