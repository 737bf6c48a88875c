// gjk_mixed.cuh -- the two phases of the mixed-precision GJK distance (see
// gjk_mixed.cu for the method), written as per-lane state machines so that
// the persistent kernels can refill a lane as soon as its pair is done.
#pragma once

#include "jolt.cuh"

namespace d3d {

// FP64 support for the refinement phases.  Wherever the support function is
// discontinuous -- the vertex of a polytope, the end of a capsule or a
// cylinder (local z of the direction near 0) -- the choice is made in FP32,
// exactly as the FP32 phase makes it (the FP32 record is the FP64 one
// rounded, so its values are recomputed from the FP64 record here), and only
// the point itself is evaluated in FP64.  A row re-evaluated along the
// direction that produced it in FP32 therefore lands on the same feature; near
// a discontinuity both features are supports to within the FP32 rounding of
// the direction.
struct RefineSupport {
    static __device__ __forceinline__ d3 eval(const Col<double>& c, const d3d_store& s, d3 d) {
        const f3 df = mk(__double2float_rn(d.x), __double2float_rn(d.y), __double2float_rn(d.z));
        if (c.type == D3D_BOX || c.type == D3D_HULL) {
            if (c.nv < 1) return mk(double(NAN), double(NAN), double(NAN));
            return load_vertex(s.verts64, c.off + hull_argmax(s.verts32, c.off, c.nv, df));
        }
        if (c.type == D3D_CAPSULE || c.type == D3D_CYLINDER) {
            // local z of the direction as the FP32 support computes it
            const float lz = dot102(__double2float_rn(c.R[2]), __double2float_rn(c.R[5]),
                                    __double2float_rn(c.R[8]), df.x, df.y, df.z);
            const bool up = c.type == D3D_CAPSULE ? lz > 0.f : !(lz < 0.f);
            const d3 l = rt_mul(c.R, d);
            d3 v;
            if (c.type == D3D_CAPSULE) {
                const double sn = sqrt(l.x * l.x + l.y * l.y + l.z * l.z);
                v = sn == 0.0 ? mk(c.p[0], 0.0, 0.0) : l * (c.p[0] / sn);
                v.z += up ? 0.5 * c.p[1] : -0.5 * c.p[1];
            } else {
                const double sn = sqrt(l.x * l.x + l.y * l.y);
                const double z = up ? 0.5 * c.p[1] : -0.5 * c.p[1];
                v = sn == 0.0 ? mk(c.p[0], 0.0, z) : mk(l.x * (c.p[0] / sn), l.y * (c.p[0] / sn), z);
            }
            return xform(c.R, c.t, v);
        }
        return support(c, s.verts64, d);
    }
};

// Relative duality gap at which phase B stops; it bounds the relative
// distance error of the mixed form (apart from the FP32 vertex choice).
constexpr double kMixedRelGap = 1e-9;

__device__ __forceinline__ JoltEps<float> fp32_eps() {
    const float e = FLT_EPSILON;
    // plane/side tests and relative convergence at a few ulps; the touching
    // test at the FP32 noise floor of |v|^2 relative to max|Y|^2
    return JoltEps<float>{4.f * e, e * e, 4.f * e, 16.f * e * e, 0.f};
}

enum PhaseAOutcome { PA_SEPARATED = 0, PA_TOUCHING = 1, PA_CLIPPED = 2, PA_FAILED = 3 };

// What phase A hands to phase B for one pair (80 bytes): the final closest
// point (xyz) with the outcome, simplex size and iteration count packed in w,
// and the search direction of each simplex row.
struct __align__(16) Handoff {
    float4 v;
    float4 d[4];
};

__device__ __forceinline__ int handoff_outcome(const Handoff& h) { return __float_as_int(h.v.w) & 0xff; }
__device__ __forceinline__ int handoff_rows(const Handoff& h) { return (__float_as_int(h.v.w) >> 8) & 0xff; }
__device__ __forceinline__ int handoff_iters(const Handoff& h) { return (__float_as_int(h.v.w) >> 16) & 0xffff; }

// ---------------------------------------------------------------- phase A
// The Jolt loop (gjk_step) in FP32 on the FP32 mirror; row j of S.P holds
// the search direction that produced row j of S.Y.
struct PhaseALoop {
    Simplex<float> S;
    f3 dir;
    f3 v;
    float vl, prev;
    int it;
};

__device__ __forceinline__ void pa_begin(PhaseALoop& L) {
    simplex_clear(L.S);
    L.dir = mk(1.f, 0.f, 0.f);
    L.v = L.dir;
    L.vl = 1.f;
    L.prev = FLT_MAX;
    L.it = 0;
}

// one iteration; -1 while running, else a PhaseAOutcome
__device__ __forceinline__ int pa_step(PhaseALoop& L, const Col<float>& c1, const Col<float>& c2, const d3d_store& s,
                                       float tol_sq, float max_d2, int max_iter) {
    const JoltEps<float> E = fp32_eps();
    if (L.it >= max_iter) return PA_FAILED;
    ++L.it;
    f3 p = support(c1, s.verts32, L.dir);
    f3 q = support(c2, s.verts32, -L.dir);
    f3 w = p - q;
    float dd = dot(L.dir, w);
    if (dd < 0.f && dd * dd > L.vl * max_d2) return PA_CLIPPED;
    simplex_push(L.S, w, L.dir, q);
    f3 nv;
    float nl;
    int set;
    if (closest_to_origin(L.S, L.prev, E, nv, nl, set)) {
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

__device__ __forceinline__ Handoff pa_handoff(const PhaseALoop& L, int outcome) {
    Handoff h;
    int it = L.it < 0xffff ? L.it : 0xffff;
    h.v = make_float4(L.v.x, L.v.y, L.v.z, __int_as_float(outcome | (L.S.n << 8) | (it << 16)));
#pragma unroll
    for (int j = 0; j < 4; ++j) h.d[j] = make_float4(L.S.P[j].x, L.S.P[j].y, L.S.P[j].z, 0.f);
    return h;
}

// ---------------------------------------------------------------- phase B
enum PhaseBMode { PB_RUN = 0, PB_DONE = 1, PB_FALLBACK = 2 };

// Start phase B for one pair.  Separated pairs: the reference's loop from the
// FP32 closest point's direction instead of (1,0,0), stopped by the duality
// gap.  Touching pairs: the FP32 simplex rows re-evaluated in FP64 along the
// directions that produced them; if that simplex already encloses (or
// touches) the origin the pair is done, otherwise the loop resumes there.
__device__ __forceinline__ int pb_begin(const Handoff& h, const Col<double>& c1, const Col<double>& c2,
                                        const d3d_store& s, double tol_sq, const JoltEps<double>& E,
                                        GjkLoop<double>& g, GjkResult<double>& r) {
    const int outcome = handoff_outcome(h);
    simplex_clear(g.S);
    if (outcome == PA_SEPARATED) {
        d3 dir = mk(-(double)h.v.x, -(double)h.v.y, -(double)h.v.z);
        gjk_begin(g, dir, dot(dir, dir), DBL_MAX);
        return PB_RUN;
    }
    if (outcome != PA_TOUCHING) return PB_FALLBACK;
    const int rows = handoff_rows(h);
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (j < rows) {
            d3 d = mk((double)h.d[j].x, (double)h.d[j].y, (double)h.d[j].z);
            d3 p = RefineSupport::eval(c1, s, d);
            d3 q = RefineSupport::eval(c2, s, -d);
            simplex_push(g.S, p - q, p, q);
        }
    d3 v;
    double vl;
    int set;
    if (g.S.n == 0 || !closest_to_origin(g.S, DBL_MAX, E, v, vl, set)) return PB_FALLBACK;
    if (set != 15) simplex_compact<double, true>(g.S, set);
    if (set == 15 || vl <= tol_sq || vl <= E.isect * max_y_len_sq(g.S)) {
        d3 a, b;
        closest_points(g.S, E, a, b);
        d3 m = (a + b) * 0.5;
        r.dist = 0.0;
        r.a = m;
        r.b = m;
        r.status = D3D_STATUS_OK;
        r.iters = 0;
        return PB_DONE;
    }
    gjk_begin(g, -v, vl, vl);
    return PB_RUN;
}

__device__ __forceinline__ bool pb_step(GjkLoop<double>& g, const Col<double>& c1, const Col<double>& c2,
                                        const d3d_store& s, double tol_sq, const d3d_gjk_options& opt,
                                        const JoltEps<double>& E) {
    return gjk_step<double, RefineSupport, true>(g, c1, c2, s, tol_sq, opt.max_distance_squared,
                                                 opt.max_iterations, E, kMixedRelGap);
}

// Finish phase B.  Jolt's face-region projection can leave the simplex on a
// sliver triangle; the barycentric closest points then disagree with |v|,
// and such pairs (and any non-OK status) go to the cold FP64 fallback.
__device__ __forceinline__ int pb_end(const GjkLoop<double>& g, const d3d_gjk_options& opt, const JoltEps<double>& E,
                                      GjkResult<double>& r) {
    gjk_end(g, opt.sanity_check, E, r);
    if (r.status != D3D_STATUS_OK) return PB_FALLBACK;
    d3 ab = r.a - r.b;
    if (abs_t(sqrt_t(dot(ab, ab)) - r.dist) > 1e-10 * (r.dist > 1.0 ? r.dist : 1.0)) return PB_FALLBACK;
    return PB_DONE;
}

// One pair end to end (phase A, phase B, cold fallback): the single-thread
// form of the three kernels, used where a pair is computed in isolation.
__device__ __forceinline__ void gjk_mixed_pair(const d3d_store& s, int a, int b, const d3d_gjk_options& opt,
                                               GjkResult<double>& r, Simplex<double>& S) {
    const JoltEps<double> E = reference_eps<double>();
    const double tol_sq = opt.tolerance * opt.tolerance;
    Handoff h;
    {
        Col<float> f1, f2;
        load_col(s, a, f1);
        load_col(s, b, f2);
        PhaseALoop L;
        pa_begin(L);
        int o;
        while ((o = pa_step(L, f1, f2, s, (float)tol_sq, (float)opt.max_distance_squared, opt.max_iterations)) < 0) {
        }
        h = pa_handoff(L, o);
    }
    Col<double> c1, c2;
    load_col(s, a, c1);
    load_col(s, b, c2);
    GjkLoop<double> g;
    int mode = pb_begin(h, c1, c2, s, tol_sq, E, g, r);
    if (mode == PB_RUN) {
        while (!pb_step(g, c1, c2, s, tol_sq, opt, E)) {
        }
        mode = pb_end(g, opt, E, r);
    }
    if (mode == PB_DONE) {
        r.iters += handoff_iters(h);
        S = g.S;
        return;
    }
    simplex_clear(S);
    const d3 dir = mk(1.0, 0.0, 0.0);
    gjk_distance_loop(c1, c2, s, tol_sq, opt.max_distance_squared, opt.sanity_check, opt.max_iterations, E, S, dir,
                      dot(dir, dir), DBL_MAX, r);
}

}  // namespace d3d
