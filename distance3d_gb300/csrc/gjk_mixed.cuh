// gjk_mixed.cuh -- the two phases of the mixed-precision GJK distance (see
// gjk_mixed.cu for the method), written as per-lane state machines so that
// the persistent kernels can refill a lane as soon as its pair is done.
#pragma once

#include "jolt.cuh"

namespace d3d {

// ---------------------------------------------------------------- supports
// The mixed form evaluates the curved supports in the collider's own frame:
// l = R^T d, one local point per type, then t + R v.  Wherever a support is
// discontinuous -- the vertex of a polytope, the end of a capsule or a
// cylinder (local z near 0), the tip or the rim of a cone -- the choice is
// made in FP32 on the FP32 record (the FP64 record rounded), and the FP64
// refinement repeats that FP32 choice and evaluates only the point in FP64.
// A row re-evaluated along the direction that produced it in FP32 therefore
// lands on the same feature; near a discontinuity both features are supports
// to within the FP32 rounding of the direction.  Norms are one reciprocal
// square root (the reference divides by the norm; equal up to the last bits).

__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }

// The discrete choice of the two-feature supports, in FP32: capsule and
// cylinder upper end, cone rim (otherwise its tip).
__device__ __forceinline__ bool upper_feature(int type, const float* R, float r, float h, f3 d) {
    if (type == D3D_CONE) {
        Col<float> cf;
        cf.p[0] = r;
        cf.p[1] = h;
        f3 q;
        return cone_rim(cf, rt_mul(R, d), q);
    }
    const float lz = dot102(R[2], R[5], R[8], d.x, d.y, d.z);
    return type == D3D_CAPSULE ? lz > 0.f : !(lz < 0.f);
}

// Local support point v of a curved collider (not sphere, box or hull) for
// the local direction l, with the discrete choice `up` made beforehand.
template <typename T>
__device__ __forceinline__ V3<T> local_point(const Col<T>& c, V3<T> l, bool up) {
    const T r = c.p[0];
    switch (c.type) {
    case D3D_CAPSULE: {
        const T n2 = dot(l, l);
        V3<T> v = n2 == T(0) ? mk(r, T(0), T(0)) : l * (r * rsqrt_t(n2));
        v.z += up ? T(0.5) * c.p[1] : T(-0.5) * c.p[1];
        return v;
    }
    case D3D_ELLIPSOID: {
        const V3<T> a = mk(l.x * c.p[0], l.y * c.p[1], l.z * c.p[2]);
        const T n2 = dot(a, a);
        const T f = n2 != T(0) ? rsqrt_t(n2) : T(1);
        return mk(a.x * f * c.p[0], a.y * f * c.p[1], a.z * f * c.p[2]);
    }
    case D3D_ELLIPSE: {
        const T a0 = l.x * c.p[0], a1 = l.y * c.p[1];
        const T n2 = a0 * a0 + a1 * a1;
        const T f = n2 != T(0) ? rsqrt_t(n2) : T(1);
        return mk(a0 * f * c.p[0], a1 * f * c.p[1], T(0));
    }
    default: {  // cylinder, disk, cone: the rim point r (l.x, l.y) / |(l.x, l.y)|
        const T n2 = l.x * l.x + l.y * l.y;
        const T f = n2 != T(0) ? r * rsqrt_t(n2) : T(0);
        if (c.type == D3D_CYLINDER) {
            const T z = up ? T(0.5) * c.p[1] : T(-0.5) * c.p[1];
            return n2 == T(0) ? mk(r, T(0), z) : mk(l.x * f, l.y * f, z);
        }
        if (c.type == D3D_CONE && !up) return mk(T(0), T(0), c.p[1]);
        return mk(l.x * f, l.y * f, T(0));
    }
    }
}

// Margin: s + m d / |d| (the zero direction adds nothing).  The margin is
// read from the record only here, so that no register holds it through the
// support evaluation.
__device__ __forceinline__ float record_margin(const d3d_store& st, const Col<float>& c) {
    return __ldg(st.rec32 + (size_t)c.idx * 16 + 15);
}
__device__ __forceinline__ double record_margin(const d3d_store& st, const Col<double>& c) {
    return __ldg(st.rec64 + (size_t)c.idx * 16 + 15);
}
template <typename T>
__device__ __forceinline__ V3<T> margin_fast(const d3d_store& st, const Col<T>& c, V3<T> s, V3<T> d) {
    if (!c.wrapped) return s;
    const T n2 = dot(d, d);
    return n2 == T(0) ? s : s + d * (record_margin(st, c) * rsqrt_t(n2));
}

// Corner of a box (the store's 8 vertices in itertools.product order) that
// maximises V . d: bit 2, 1, 0 of the index set where R^T d is positive along
// box axis 0, 1, 2.  Where a component is zero the two faces tie and the
// lower index is the first maximum, as in hull_argmax; near such ties the
// rounded FP32 products may pick the other corner, a support all the same.
__device__ __forceinline__ int box_corner(const float* R, f3 d) {
    const f3 l = rt_mul(R, d);
    return (l.x > 0.f ? 4 : 0) | (l.y > 0.f ? 2 : 0) | (l.z > 0.f ? 1 : 0);
}

// FP32 support of the mixed form's search phases.  MESH = false leaves out
// the MeshGraph branch, for kernels launched on stores without meshes.  A
// non-null `vi` receives the vertex a box, hull or MeshGraph support took
// (unchanged for the other types), so that the FP64 phases can take the same
// vertex without searching again (RefineSupportT::eval_at).
template <bool MESH>
struct FastSupportT {
    static __device__ __forceinline__ f3 base(const Col<float>& c, const d3d_store& s, f3 d, int* vi = nullptr) {
        if (c.type == D3D_BOX && c.nv == 8) {
            const int k = box_corner(c.R, d);
            if (vi) *vi = k;
            return load_vertex(s.verts32, c.off + k);
        }
        if (c.type == D3D_BOX || c.type == D3D_HULL) {
            if (c.nv < 1) return mk(NAN, NAN, NAN);
            const int k = hull_argmax(s.verts32, c.off, c.nv, d);
            if (vi) *vi = k;
            return load_vertex(s.verts32, c.off + k);
        }
        if (c.type == D3D_SPHERE) {
            const float n2 = dot(d, d);
            const f3 ctr = mk(c.t[0], c.t[1], c.t[2]);
            return n2 == 0.f ? ctr + mk(0.f, 0.f, c.p[0]) : ctr + d * (c.p[0] * rsqrtf(n2));
        }
        if (MESH && c.type == D3D_MESH) {
            if (c.nv < 1) return mk(NAN, NAN, NAN);
            const int k = mesh_climb(c, s, rt_mul(c.R, d));
            if (vi) *vi = k;
            return xform(c.R, c.t, load_vertex(s.verts32, c.off + k));
        }
        const bool up = upper_feature(c.type, c.R, c.p[0], c.p[1], d);
        return xform(c.R, c.t, local_point(c, rt_mul(c.R, d), up));
    }
    static __device__ __forceinline__ f3 eval(const Col<float>& c, const d3d_store& s, f3 d, int* vi = nullptr) {
        return margin_fast(s, c, base(c, s, d, vi), d);
    }
};
using FastSupport = FastSupportT<true>;

// FP64 support of the refinement phases, with FastSupport's FP32 choices.
template <bool MESH>
struct RefineSupportT {
    static __device__ __forceinline__ d3 eval(const Col<double>& c, const d3d_store& s, d3 d) {
        return margin_fast(s, c, base(c, s, d), d);
    }

    // eval, given the vertex FastSupport took along the FP32 rounding of d
    // (vi >= 0; -1: unknown): a box, hull or MeshGraph reads that vertex
    // instead of searching again (the same search on the same FP32 inputs
    // would return it), the other types evaluate as eval does.
    static __device__ __forceinline__ d3 eval_at(const Col<double>& c, const d3d_store& s, d3 d, int vi) {
        if (vi >= 0 && vi < c.nv) {
            if (c.type == D3D_BOX || c.type == D3D_HULL) return margin_fast(s, c, load_vertex(s.verts64, c.off + vi), d);
            if (MESH && c.type == D3D_MESH)
                return margin_fast(s, c, xform(c.R, c.t, load_vertex(s.verts64, c.off + vi)), d);
        }
        return eval(c, s, d);
    }

    static __device__ __forceinline__ d3 base(const Col<double>& c, const d3d_store& s, d3 d) {
        const f3 df = mk(__double2float_rn(d.x), __double2float_rn(d.y), __double2float_rn(d.z));
        if (c.type == D3D_BOX && c.nv == 8) {
            // the FP32 record's rotation, as FastSupport sees it
            float Rf[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) Rf[k] = __double2float_rn(c.R[k]);
            return load_vertex(s.verts64, c.off + box_corner(Rf, df));
        }
        if (c.type == D3D_BOX || c.type == D3D_HULL) {
            if (c.nv < 1) return mk(double(NAN), double(NAN), double(NAN));
            return load_vertex(s.verts64, c.off + hull_argmax(s.verts32, c.off, c.nv, df));
        }
        if (c.type == D3D_SPHERE) {
            const double n2 = dot(d, d);
            const d3 ctr = mk(c.t[0], c.t[1], c.t[2]);
            return n2 == 0.0 ? ctr + mk(0.0, 0.0, c.p[0]) : ctr + d * (c.p[0] * rsqrt(n2));
        }
        if (MESH && c.type == D3D_MESH) {
            // the vertex the FP32 climb reaches on the FP32 mirror
            if (c.nv < 1) return mk(double(NAN), double(NAN), double(NAN));
            Col<float> cf;
            cf.nv = c.nv;
            cf.off = c.off;
            cf.idx = c.idx;
            for (int k = 0; k < 9; ++k) cf.R[k] = __double2float_rn(c.R[k]);
            return xform(c.R, c.t, load_vertex(s.verts64, c.off + mesh_climb<true>(cf, s, rt_mul(cf.R, df))));
        }
        bool up = false;
        if (c.type == D3D_CAPSULE || c.type == D3D_CYLINDER || c.type == D3D_CONE) {
            // the FP32 record's rotation: column 2 (capsule, cylinder) or all (cone)
            float Rf[9] = {};
            Rf[2] = __double2float_rn(c.R[2]);
            Rf[5] = __double2float_rn(c.R[5]);
            Rf[8] = __double2float_rn(c.R[8]);
            if (c.type == D3D_CONE) {
                Rf[0] = __double2float_rn(c.R[0]);
                Rf[1] = __double2float_rn(c.R[1]);
                Rf[3] = __double2float_rn(c.R[3]);
                Rf[4] = __double2float_rn(c.R[4]);
                Rf[6] = __double2float_rn(c.R[6]);
                Rf[7] = __double2float_rn(c.R[7]);
            }
            up = upper_feature(c.type, Rf, __double2float_rn(c.p[0]), __double2float_rn(c.p[1]), df);
        }
        return xform(c.R, c.t, local_point(c, rt_mul(c.R, d), up));
    }
};

using RefineSupport = RefineSupportT<true>;

// Duality gap at which the FP64 refinement stops: the distance bracket
// within 1e-6 of the distance, or within 1e-9 of the scene's scale
// (max(1, |w|)) for nearly touching pairs, where the relative test would
// chase FP32-resolution directions for dozens of FP64 iterations.  Both are
// at least 10x below the form's 1e-5 tolerance on max(1, distance).  (A
// bracket of 1e-7 took 50% more FP64 iterations -- 1.8 per separated pair
// instead of 1.2 on the six-type workload -- for errors below 5e-8 instead of
// 3e-7.)
constexpr double kMixedRelGap = 1e-6;
constexpr double kMixedAbsGap2 = 1e-18;

__device__ __forceinline__ JoltEps<float> fp32_eps() {
    const float e = FLT_EPSILON;
    // plane/side tests at a few ulps, relative convergence at one ulp of
    // |v|^2 (the FP64 refinement starts from this direction); the touching
    // test at the FP32 noise floor of |v|^2 relative to max|Y|^2
    return JoltEps<float>{4.f * e, e * e, e, 16.f * e * e, 0.f};
}

enum PhaseAOutcome { PA_SEPARATED = 0, PA_TOUCHING = 1, PA_CLIPPED = 2, PA_FAILED = 3, PA_BAD_INDEX = 4 };

// What phase A hands to the refinement pass for one pair (80 bytes): the
// final closest point (xyz) with the outcome, simplex size and iteration
// count packed in w, and per simplex row the search direction (xyz) and, in
// w, the vertices the supports of a box, hull or MeshGraph took along it
// (16 bits per collider, 0xffff for none; see handoff_vertex).
struct __align__(16) Handoff {
    float4 v;
    float4 d[4];
};

__device__ __forceinline__ int handoff_outcome(const Handoff& h) { return __float_as_int(h.v.w) & 0xff; }
__device__ __forceinline__ int handoff_rows(const Handoff& h) { return (__float_as_int(h.v.w) >> 8) & 0xff; }
__device__ __forceinline__ int handoff_iters(float4 v) { return (__float_as_int(v.w) >> 16) & 0xffff; }
// the vertex collider k (0: i1, 1: i2) of a row took, -1 if none
__device__ __forceinline__ int handoff_vertex(float4 d, int k) {
    const int x = (int)((__float_as_uint(d.w) >> (16 * k)) & 0xffffu);
    return x == 0xffff ? -1 : x;
}

// ---------------------------------------------------------------- phase A
// The Jolt loop (gjk_step) in FP32 on the FP32 mirror; row j of S.P holds
// the search direction that produced row j of S.Y, and row j of S.Q the
// vertices its polytope supports took (bits of a float, moved with the row).
// Phase A's P/Q rows in shared memory, one float4 per row: the FP32
// direction that produced the row (P) and, in w, the vertex ids its supports
// took (Q.x; Q.y and Q.z are zero).  Element (row r) of the lane at base[r kStride].
template <int kStride>
struct ARows {
    float4* base;
    __device__ __forceinline__ void put(int k, f3 p, f3 q) { base[k * kStride] = make_float4(p.x, p.y, p.z, q.x); }
    __device__ __forceinline__ void move(int dst, int src) { base[dst * kStride] = base[src * kStride]; }
    __device__ __forceinline__ f3 p(int k) const {
        const float4 r = base[k * kStride];
        return mk(r.x, r.y, r.z);
    }
    __device__ __forceinline__ f3 q(int k) const { return mk(base[k * kStride].w, 0.f, 0.f); }
};

template <typename Rows>
struct PhaseALoop {
    Simplex<float, Rows> S;
    f3 dir;
    f3 v;
    float vl, prev;
    int it;
};

template <typename Rows>
__device__ __forceinline__ void pa_begin(PhaseALoop<Rows>& L) {
    simplex_clear(L.S);
    L.dir = mk(1.f, 0.f, 0.f);
    L.v = L.dir;
    L.vl = 1.f;
    L.prev = FLT_MAX;
    L.it = 0;
}

// one iteration; -1 while running, else a PhaseAOutcome
template <bool MESH, typename Rows>
__device__ __forceinline__ int pa_step(PhaseALoop<Rows>& L, const d3d_store& s, int a, int b, float tol_sq, float max_d2,
                                       int max_iter) {
    const JoltEps<float> E = fp32_eps();
    if (L.it >= max_iter) return PA_FAILED;
    ++L.it;
    const unsigned together = __activemask();
    f3 p, q;
    // the vertices the polytope supports took, 16 bits per collider (0xffff: none), ride in the
    // Q row of the simplex (phase A reads only Y and the directions in P) to the handoff
    unsigned vis = 0;
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        Col<float> c;
        load_col(s, k ? b : a, c);
        int vi = -1;
        const f3 x = FastSupportT<MESH>::eval(c, s, k ? -L.dir : L.dir, &vi);
        vis |= (unsigned)(vi >= 0 && vi < 0xffff ? vi : 0xffff) << (16 * k);
        if (k)
            q = x;
        else
            p = x;
    }
    // reconverge after the type- and size-dependent supports, so that the
    // lanes solve their simplices together (see gjk_step)
    __syncwarp(together);
    f3 w = p - q;
    float dd = dot(L.dir, w);
    if (dd < 0.f && dd * dd > L.vl * max_d2) return PA_CLIPPED;
    simplex_push(L.S, w, L.dir, mk(__uint_as_float(vis), 0.f, 0.f));
    f3 nv;
    float nl;
    int set;
    if (closest_to_origin<float, Rows, true>(L.S, L.prev, E, nv, nl, set)) {
        L.dir = nv;
        L.vl = nl;
    } else {
        --L.S.n;
        set = (1 << L.S.n) - 1;
        L.dir = -L.dir;  // the closest point so far
    }
    L.v = L.dir;
    if (set == 15) return PA_TOUCHING;
    simplex_compact<float, true>(L.S, set);
    if (L.vl <= tol_sq || L.vl <= E.isect * max_y_len_sq(L.S)) return PA_TOUCHING;
    L.dir = -L.dir;
    if (L.prev - L.vl <= E.conv * L.prev) return (L.vl == L.vl && L.vl <= FLT_MAX) ? PA_SEPARATED : PA_FAILED;
    L.prev = L.vl;
    return -1;
}

template <typename Rows>
__device__ __forceinline__ Handoff pa_handoff(const PhaseALoop<Rows>& L, int outcome) {
    Handoff h;
    int it = L.it < 0xffff ? L.it : 0xffff;
    h.v = make_float4(L.v.x, L.v.y, L.v.z, __int_as_float(outcome | (L.S.n << 8) | (it << 16)));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const f3 p = L.S.R.p(j);
        h.d[j] = make_float4(p.x, p.y, p.z, L.S.R.q(j).x);
    }
    return h;
}

// ---------------------------------------------------------------- phase B
enum PhaseBMode { PB_RUN = 0, PB_DONE = 1, PB_FALLBACK = 2, PB_REPLAY = 3 };

// The FP64 rows of one pair that the refinement pass hands to B: the support
// points p and q of each row of A's final simplex, evaluated in FP64 along
// the FP32 direction that produced the row, and their count.  B writes the
// state of a pair whose loop it ends into the same record for the end pass.
struct alignas(16) EndRecord {
    double pq[4][6];  // P and Q rows below n
    double dir[3];
    double vl;
    int it;  // A's and B's iterations
    int state;
    int status;
    int n;
};

// FP64 continuation of the reference's loop for one pair, a per-lane state
// machine.  REPLAY: the simplex holds the FP64 rows handed over by the
// refinement pass, and the first round solves it as the loop's first
// iteration would (nothing to beat yet).  If it encloses or touches the
// origin the pair is done; otherwise RUN continues the reference's loop from
// there, stopped by the duality gap.
template <typename Rows>
struct PhaseB {
    GjkLoop<double, Rows> g;
    int mode;
};

template <typename Rows>
__device__ __forceinline__ void pb_begin(PhaseB<Rows>& B, const EndRecord& rec) {
    simplex_clear(B.g.S);
    B.g.it = 0;
    B.g.state = GJK_RUNNING;
    B.g.status = D3D_STATUS_OK;
    const int n = rec.n;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j < n) {
            const d3 p = mk(rec.pq[j][0], rec.pq[j][1], rec.pq[j][2]);
            const d3 q = mk(rec.pq[j][3], rec.pq[j][4], rec.pq[j][5]);
            simplex_push(B.g.S, p - q, p, q);
        }
    }
    B.mode = n > 0 && n <= 4 ? PB_REPLAY : PB_FALLBACK;
}

// One round for one lane: nothing to evaluate in the REPLAY round (the rows
// are in the simplex), one FP64 support pair along the loop's direction in a
// RUN round, then the simplex update (_gjk_jolt.py:224-288).  Every round ends
// in the simplex solve, so a warp's lanes reach it together whatever mode
// each is in.  Returns true once the loop has ended: g.state is
// GJK_INTERSECTION or GJK_NO_INTERSECTION (pb_end finishes the pair), or
// B.mode is PB_FALLBACK (clipped, iteration bound, failed replay).
template <bool MESH = true, typename Rows>
__device__ __forceinline__ bool pb_round(PhaseB<Rows>& B, const d3d_store& s, int a, int b, double tol_sq,
                                         const d3d_gjk_options& opt, const JoltEps<double>& E) {
    GjkLoop<double, Rows>& g = B.g;
    const bool replay = B.mode == PB_REPLAY;
    // The lanes that call together solve together: the support and its
    // checks only set `ended`, and all lanes reconverge before the solve (see
    // gjk_step).
    const unsigned together = __activemask();
    int ended = 0;  // 1: to the fallback (iteration bound, clipped); 2: the duality gap closed
    if (!replay) {
        if (g.it >= opt.max_iterations) {
            ended = 1;
        } else {
            ++g.it;
            d3 p, q;
            pair_supports<double, RefineSupportT<MESH>>(s, a, b, g.dir, p, q);
            const d3 w = p - q;
            const double dd = dot(g.dir, w);
            // duality gap: |v| - (|v|^2 - v.w) / |v| <= distance <= |v|
            const double gap = g.vl + dd;
            if (dd < 0.0 && dd * dd > g.vl * opt.max_distance_squared) {
                ended = 1;  // clipped: the FP64 kernel reports it
            } else if (g.S.n > 0 && (gap <= kMixedRelGap * g.vl ||
                                     gap * gap <= kMixedAbsGap2 * maxf2(1.0, dot(w, w)) * g.vl)) {
                g.dir = -g.dir;
                g.state = GJK_NO_INTERSECTION;
                ended = 2;
            } else {
                simplex_push(g.S, w, p, q);
            }
        }
    }
    __syncwarp(together);
    if (ended) {
        if (ended == 1) B.mode = PB_FALLBACK;
        return true;
    }
    d3 nv;
    double nl;
    int set;
    const double prev = replay ? DBL_MAX : g.prev;
    if (closest_to_origin<double, Rows, true>(g.S, prev, E, nv, nl, set)) {
        g.dir = nv;
        g.vl = nl;
    } else if (replay) {
        B.mode = PB_FALLBACK;
        return true;
    } else {
        --g.S.n;
        set = (1 << g.S.n) - 1;
    }
    if (replay) {
        B.mode = PB_RUN;
        g.prev = DBL_MAX;
    }
    if (set == 15) {
        g.vl = 0.0;
        g.state = GJK_INTERSECTION;
        return true;
    }
    simplex_compact<double, true>(g.S, set);
    if (g.vl <= tol_sq || g.vl <= E.isect * max_y_len_sq(g.S)) {
        g.vl = 0.0;
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

// ---------------------------------------------------------------- refinement pass
// Closest point to the origin of the affine hull of the rows w[0..n), n <= 3,
// and its barycentric coordinates (a Gram-system solve for a triangle, one
// division).  True only if the point lies strictly inside the feature and the
// feature is not degenerate (|det| above 1e-10 of d00 d11, i.e. the edges are
// more than ~1e-5 rad from parallel); otherwise the reference's solve in B
// decides.  Whether the point is the closest point of the Minkowski
// difference is certified separately by the duality gap.
__device__ __forceinline__ bool feature_point(const d3* w, int n, d3& v, double* lam) {
    lam[1] = lam[2] = 0.0;
    if (n == 1) {
        v = w[0];
        lam[0] = 1.0;
        return true;
    }
    const d3 e0 = w[1] - w[0];
    if (n == 2) {
        const double den = dot(e0, e0);
        const double t = -dot(w[0], e0) / den;
        v = w[0] + e0 * t;
        lam[0] = 1.0 - t;
        lam[1] = t;
        return den > 0.0 && t > 0.0 && t < 1.0;
    }
    const d3 e1 = w[2] - w[0];
    const double d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1);
    const double b0 = -dot(w[0], e0), b1 = -dot(w[0], e1);
    const double det = d00 * d11 - d01 * d01;
    const double inv = 1.0 / det;
    const double s = (d11 * b0 - d01 * b1) * inv;
    const double t = (d00 * b1 - d01 * b0) * inv;
    v = (w[0] + e0 * s) + e1 * t;
    lam[0] = 1.0 - s - t;
    lam[1] = s;
    lam[2] = t;
    return det > 1e-10 * (d00 * d11) && s > 0.0 && t > 0.0 && lam[0] > 0.0;
}

// Finish a pair after its loop.  The closest points use the scale-invariant
// degeneracy test of bary_plane (the simplex built around an accurate FP32
// direction is tiny).  Should they still disagree with |v| (a sliver
// triangle), the pair, like any non-OK status, goes to the cold FP64
// fallback.
template <typename Rows>
__device__ __forceinline__ int pb_end(const GjkLoop<double, Rows>& g, const d3d_gjk_options& opt,
                                      const JoltEps<double>& E, GjkResult<double>& r) {
    gjk_end<double, true>(g, opt.sanity_check, E, r);
    if (r.status != D3D_STATUS_OK) return PB_FALLBACK;
    const d3 ab = r.a - r.b;
    if (abs_t(sqrt_t(dot(ab, ab)) - r.dist) > 1e-10 * (r.dist > 1.0 ? r.dist : 1.0)) return PB_FALLBACK;
    return PB_DONE;
}

}  // namespace d3d
