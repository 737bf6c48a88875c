// mpr.cu -- Minkowski portal refinement (MPR), the plain FP64 drop-in for
// distance3d's mpr_intersection and mpr_penetration (mpr.py:21-110).
// Compiled with -fmad=false: every step is the reference's
// rounding sequence (NumPy orders as in d3d_device.cuh), so flags, depths,
// directions and contact positions are the reference's bit for bit.
//
// Each lane of the persistent kernel runs one pair as a state machine with
// one support evaluation per round (portal discovery, refinement,
// penetration search), and takes the next pair of the type-sorted order when
// its pair ends.  The portal (four Minkowski-difference vertices and the two
// colliders' support points behind each) lives in shared memory, one column
// per lane (stride kBlock), because the reference replaces its rows by
// data-dependent index.  The refinement loop of the reference has no bound;
// here it stops after `refine_limit` expansions with status
// D3D_STATUS_MAX_ITER.
#include "capi_util.h"
#include "jolt.cuh"
#include "persist.cuh"
#include "scratch.h"

namespace {

using namespace d3d;

constexpr int kBlock = 128;
constexpr double kEps = DBL_EPSILON;

// colliders.py center(): the pose translation, a hull's vertex mean
// (np.mean(axis=0): rows summed in order, then divided by the count), a
// mesh's vertex mean posed, a cone's mid-axis point (:582-584); Margin passes
// through (:633-634).
__device__ d3 collider_center(const d3d_store& st, int idx) {
    Col<double> c;
    load_col(st, idx, c);
    if (c.type == D3D_HULL || c.type == D3D_MESH) {
        if (c.nv < 1) return mk(double(NAN), double(NAN), double(NAN));
        d3 s = load_vertex(st.verts64, c.off);
        for (int k = 1; k < c.nv; ++k) s = s + load_vertex(st.verts64, c.off + k);
        const double n = (double)c.nv;
        const d3 m = mk(s.x / n, s.y / n, s.z / n);
        // a mesh's vertices are in its frame: t + R mean (colliders.py:224-226)
        return c.type == D3D_MESH ? xform(c.R, c.t, m) : m;
    }
    const d3 t = mk(c.t[0], c.t[1], c.t[2]);
    if (c.type == D3D_CONE) {
        const double f = 0.5 * c.p[1];
        return t + mk(f * c.R[2], f * c.R[5], f * c.R[8]);
    }
    return t;
}

// utils.py:12-30
__device__ __forceinline__ d3 norm_vector(d3 v) {
    const double n = sqrt(dot(v, v));
    return n == 0.0 ? v : mk(v.x / n, v.y / n, v.z / n);
}

__device__ __forceinline__ bool all_zero(d3 v) { return v.x == 0.0 && v.y == 0.0 && v.z == 0.0; }

// The portal rows of one lane: vertex r of the Minkowski difference (v) and
// the support points of collider 1 (a) and collider 2 (b) behind it.
struct Portal {
    double* base;  // shared memory, lane column
    __device__ double& at(int which, int r, int c) const { return base[((which * 4 + r) * 3 + c) * kBlock]; }
    __device__ d3 get(int which, int r) const { return mk(at(which, r, 0), at(which, r, 1), at(which, r, 2)); }
    __device__ void put(int which, int r, d3 x) const {
        at(which, r, 0) = x.x;
        at(which, r, 1) = x.y;
        at(which, r, 2) = x.z;
    }
    __device__ d3 v(int r) const { return get(0, r); }
    __device__ d3 a(int r) const { return get(1, r); }
    __device__ d3 b(int r) const { return get(2, r); }
    __device__ void set(int r, d3 va, d3 vb) const {
        put(1, r, va);
        put(2, r, vb);
        put(0, r, va - vb);  // minkowski.py:52-55
    }
    __device__ void set3(int r, d3 vv, d3 va, d3 vb) const {
        put(0, r, vv);
        put(1, r, va);
        put(2, r, vb);
    }
    __device__ void copy(int dst, int src) const { set3(dst, v(src), a(src), b(src)); }
};

// minkowski.py:23-49: support points of both colliders along d
__device__ __forceinline__ void supports(const d3d_store& st, int i, int j, d3 d, d3& pa, d3& pb) {
    pair_supports<double, ExactSupport>(st, i, j, d, pa, pb);
}

// :276-281
__device__ __forceinline__ d3 portal_direction(const Portal& P) {
    const d3 v1 = P.v(1);
    return norm_vector(cross(P.v(2) - v1, P.v(3) - v1));
}

// :290-299: min over rows 1-3 of v4 . d - v_r . d (v[1:].dot(d) is a gemv)
__device__ __forceinline__ bool reach_tolerance(const Portal& P, d3 v4, d3 d, double tol) {
    const double s4 = dot(v4, d);
    double m = 0.0;
    for (int r = 1; r < 4; ++r) {
        const d3 v = P.v(r);
        const double e = s4 - dot102(v.x, v.y, v.z, d.x, d.y, d.z);
        if (r == 1 || e < m) m = e;
    }
    return m < tol + kEps;
}

// :302-317
__device__ __forceinline__ void expand(const Portal& P, d3 pa, d3 pb) {
    const d3 v4 = pa - pb;
    const d3 c = cross(v4, P.v(0));
    int r;
    if (dot(P.v(1), c) > 0.0)
        r = dot(P.v(2), c) > 0.0 ? 1 : 3;
    else
        r = dot(P.v(3), c) > 0.0 ? 2 : 1;
    P.set3(r, v4, pa, pb);
}

// distance/_triangle.py:12-89 point_to_triangle for the origin
__device__ double origin_to_triangle(d3 A, d3 B, d3 C, d3& cp) {
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
// order; b.dot(V) through gemv: fma(b0,V0,b1*V1) + fma(b2,V2,b3*V3))
__device__ d3 contact_position(const Portal& P, d3 d) {
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
    double out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double p1 = fma(w0, P.at(1, 0, c), w1 * P.at(1, 1, c)) + fma(w2, P.at(1, 2, c), w3 * P.at(1, 3, c));
        const double p2 = fma(w0, P.at(2, 0, c), w1 * P.at(2, 1, c)) + fma(w2, P.at(2, 2, c), w3 * P.at(2, 3, c));
        out[c] = 0.5 * (p1 + p2);
    }
    return mk(out[0], out[1], out[2]);
}

struct MprOut {
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

// The phases of one pair, each ending in one support evaluation.
enum Phase { kV1 = 0, kV2, kDiscover, kRefine, kPenetrate };

// One lane's pair between rounds.
struct Lane {
    d3 d;         // direction of the next support evaluation
    int phase;
    int it;
};

// Enter the refinement (:243-273) with the portal built: returns 1 if the
// portal already encloses the origin, else prepares the first refinement
// support.
__device__ __forceinline__ int enter_refine(const Portal& P, Lane& L) {
    L.d = portal_direction(P);
    if (dot(P.v(1), L.d) > -10.0 * kEps) return 1;
    L.phase = kRefine;
    L.it = 0;
    return 0;
}

// Outcome of a round: still running, or finished with (hit, status) and the
// penetration fields set.
enum { kRunning = -1, kMiss = 0, kHit = 1 };

// Process the support points (pa, pb) along L.d for the lane's phase
// (mpr.py:123-158 with :161-240, :243-273, :320-334); returns kRunning or the
// outcome.  On a penetrating hit with `pen`, depth / dir / pos are set.
__device__ int mpr_round(const Portal& P, Lane& L, d3 pa, d3 pb, const d3d_mpr_options& opt, int& status,
                         double& depth, d3& dir, d3& pos) {
    const d3 v0 = P.v(0);
    switch (L.phase) {
    case kV1: {  // :177-201
        P.set(1, pa, pb);
        const d3 v1 = P.v(1);
        if (!all_zero(v1) && dot(v1, L.d) < kEps) return kMiss;
        d3 d = cross(v0, v1);
        if (dot(d, d) < kEps) {  // :337-352
            if (opt.penetration) {
                pos = (P.a(1) + P.b(1)) * 0.5;
                if (all_zero(v1)) {
                    depth = 0.0;
                    dir = mk(0.0, 0.0, 0.0);
                } else {
                    depth = sqrt(dot(v1, v1));
                    dir = norm_vector(v1);
                }
            }
            return kHit;
        }
        L.d = norm_vector(d);
        L.phase = kV2;
        return kRunning;
    }
    case kV2: {  // :198-210; the reference's row swap (:232-240) keeps row 1
                 // as a NumPy view, so both rows end up holding the old row 2
        P.set(2, pa, pb);
        if (dot(P.v(2), L.d) < kEps) return kMiss;
        L.d = norm_vector(cross(P.v(1) - v0, P.v(2) - v0));
        if (dot(L.d, v0) > 0.0) {
            P.copy(1, 2);
            L.d = L.d * -1.0;
        }
        L.phase = kDiscover;
        L.it = 0;
        return kRunning;
    }
    case kDiscover: {  // :145-158, :213-229
        P.set(3, pa, pb);
        const d3 v3 = P.v(3);
        if (dot(v3, L.d) < kEps) return kMiss;
        bool cont = false;
        if (dot(cross(P.v(1), v3), v0) < kEps) {
            P.copy(2, 3);
            cont = true;
        }
        if (!cont && dot(cross(v3, P.v(2)), v0) < kEps) {
            P.copy(1, 3);
            cont = true;
        }
        if (cont) L.d = norm_vector(cross(P.v(1) - v0, P.v(2) - v0));
        if (cont && ++L.it < opt.max_iterations) return kRunning;
        if (!enter_refine(P, L)) return kRunning;
        break;  // the built portal encloses the origin
    }
    case kRefine: {  // :243-273, bounded
        const d3 v4 = pa - pb;
        if (!(dot(v4, L.d) > -10.0 * kEps) || reach_tolerance(P, v4, L.d, opt.tolerance)) return kMiss;
        if (L.it >= opt.refine_limit) {
            status = D3D_STATUS_MAX_ITER;
            return kMiss;
        }
        expand(P, pa, pb);
        ++L.it;
        L.d = portal_direction(P);
        if (!(dot(P.v(1), L.d) > -10.0 * kEps)) return kRunning;
        break;  // the origin is inside
    }
    default: {  // kPenetrate, :320-334 and :355-362
        if (reach_tolerance(P, pa - pb, L.d, opt.tolerance) || L.it > opt.max_iterations) {
            d3 cp;
            depth = origin_to_triangle(P.v(1), P.v(2), P.v(3), cp);
            if (fabs(depth) < kEps) cp = mk(0.0, 0.0, 0.0);
            pos = contact_position(P, L.d);
            dir = norm_vector(cp);
            return kHit;
        }
        expand(P, pa, pb);
        ++L.it;
        L.d = portal_direction(P);
        return kRunning;
    }
    }
    // the portal encloses the origin
    if (!opt.penetration) return kHit;
    L.phase = kPenetrate;
    L.it = 0;
    L.d = portal_direction(P);
    return kRunning;
}

// Persistent MPR: each lane runs one pair's MPR one support evaluation per
// round and fetches the next pair (in the type-sorted `order`) when its pair
// ends, so the support code runs once per round for the whole warp.
__global__ void __launch_bounds__(kBlock) k_mpr(d3d_store st, const int32_t* __restrict__ i1,
                                                const int32_t* __restrict__ i2, const int32_t* __restrict__ order,
                                                int64_t n, unsigned long long* __restrict__ cursor,
                                                d3d_mpr_options opt, MprOut o) {
    __shared__ double rows[36 * kBlock];
    const Portal P{rows + threadIdx.x};
    const d3 nan3 = mk(double(NAN), double(NAN), double(NAN));
    Lane L;
    int64_t pid = 0;
    int i = 0, j = 0;
    bool need = true;
    while (true) {
        const long long slot = fetch_slot(cursor, need);
        if (need) {
            if (slot >= n) break;
            pid = order ? order[slot] : slot;
            i = i1[pid];
            j = i2[pid];
            // :161-185: origin ray from the centers, first direction
            const d3 c1 = collider_center(st, i), c2 = collider_center(st, j);
            d3 v0 = c1 - c2;
            if (all_zero(v0)) v0.x += kEps * 10.0;
            P.set3(0, v0, c1, c2);
            L.d = norm_vector(-v0);
            L.phase = kV1;
            L.it = 0;
            need = false;
        }
        d3 pa, pb;
        supports(st, i, j, L.d, pa, pb);
        int status = D3D_STATUS_OK;
        double depth = NAN;
        d3 dir = nan3, pos = nan3;
        const int r = mpr_round(P, L, pa, pb, opt, status, depth, dir, pos);
        if (r != kRunning) {
            o.hit[pid] = (int8_t)r;
            o.status[pid] = (int8_t)status;
            if (opt.penetration) {
                if (o.depth) o.depth[pid] = depth;
                put3(o.dir, pid, dir);
                put3(o.pos, pid, pos);
            }
            need = true;
        }
    }
}

}  // namespace

extern "C" int d3d_mpr(const d3d_store* store, const int32_t* i1, const int32_t* i2, int64_t n,
                       const d3d_mpr_options* opt, int8_t* hit, double* depth, double* dir, double* pos,
                       int8_t* status, void* stream) {
    int rc = d3d::check_store(store, "d3d_mpr");
    if (rc) return rc;
    D3D_REQUIRE(opt, "d3d_mpr: null options");
    D3D_REQUIRE(n >= 0, "d3d_mpr: n < 0");
    D3D_REQUIRE(opt->max_iterations >= 0 && opt->refine_limit >= 0, "d3d_mpr: negative iteration bound");
    D3D_REQUIRE(opt->tolerance >= 0.0, "d3d_mpr: negative tolerance");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(i1 && i2 && hit && status, "d3d_mpr: null pointer");
    D3D_REQUIRE(n <= INT32_MAX, "d3d_mpr: more than 2^31 pairs");
    cudaStream_t st = d3d::as_stream(stream);
    const bool sched = n >= d3d::tuning().sort_min;
    const size_t order_bytes = (sizeof(int32_t) * (size_t)n + 255) & ~size_t(255);
    const size_t bytes = 256 + (sched ? order_bytes + d3d::pair_order_temp_bytes(n) : 0);
    void* scratch = nullptr;
    rc = d3d::scratch_alloc(&scratch, bytes, st);
    if (rc) return rc;
    unsigned long long* cursor = static_cast<unsigned long long*>(scratch);
    int32_t* order = sched ? reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + 256) : nullptr;
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) {
        d3d::scratch_free(scratch, st);
        d3d::set_error("d3d_mpr: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    if (sched)
        rc = d3d::pair_order(*store, i1, i2, n, order, static_cast<char*>(scratch) + 256 + order_bytes,
                             d3d::pair_order_temp_bytes(n), st);
    if (!rc) {
        MprOut o{hit, depth, dir, pos, status};
        const int blocks = d3d::persistent_blocks((const void*)k_mpr, kBlock, n);
        k_mpr<<<blocks, kBlock, 0, st>>>(*store, i1, i2, order, n, cursor, *opt, o);
        rc = d3d::check_launch("d3d_mpr");
    }
    d3d::scratch_free(scratch, st);
    return rc;
}
