// d3d_device.cuh -- device-side building blocks shared by the kernels of
// libd3d_gb300: vector arithmetic with the reference's rounding sequence,
// collider loads from the store, and the support functions of the ten
// collider types and of the Margin wrapper.
//
// Rounding.  The reference computes its small dot products through NumPy,
// whose BLAS rounds them as fused multiply-add chains in two fixed orders
// (dot012 and dot102 below); element-wise arithmetic, np.cross and Python
// scalar arithmetic are unfused.  Translation units that must reproduce the
// reference bit for bit are compiled with -fmad=false, so that only the fma()
// calls written here fuse.  The same code compiled with -fmad=true (the
// mixed-precision unit) is free to contract.
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "d3d_gb300.h"

namespace d3d {

template <typename T>
struct V3 {
    T x, y, z;
};
using d3 = V3<double>;
using f3 = V3<float>;

template <typename T>
__device__ __forceinline__ V3<T> mk(T x, T y, T z) {
    V3<T> r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
template <typename T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a) { return mk(-a.x, -a.y, -a.z); }
template <typename T>
__device__ __forceinline__ V3<T> operator*(V3<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double sqrt_t(double a) { return sqrt(a); }
__device__ __forceinline__ float sqrt_t(float a) { return sqrtf(a); }
__device__ __forceinline__ double abs_t(double a) { return fabs(a); }
__device__ __forceinline__ float abs_t(float a) { return fabsf(a); }

// np.dot of two 3-vectors (ddot), np.linalg.norm, and the small GEMMs of
// geometry.py:157 / containment.py:147: fma(a2,b2, fma(a1,b1, a0*b0))
template <typename T>
__device__ __forceinline__ T dot012(T a0, T a1, T a2, T b0, T b1, T b2) {
    return fma_t(a2, b2, fma_t(a1, b1, a0 * b0));
}
// matrix-times-vector through BLAS gemv (pose products utils.py:143,
// geometry.py:198,245,281; hull support colliders.py:132):
// fma(a2,b2, fma(a0,b0, a1*b1))
template <typename T>
__device__ __forceinline__ T dot102(T a0, T a1, T a2, T b0, T b1, T b2) {
    return fma_t(a2, b2, fma_t(a0, b0, a1 * b1));
}
template <typename T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return dot012(a.x, a.y, a.z, b.x, b.y, b.z); }
template <typename T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ----------------------------------------------------------------------------
// Colliders
// ----------------------------------------------------------------------------

// One collider as the kernels see it.  R row-major, t, params; hull vertex
// range [off, off + nv) for boxes and hulls; margin m when wrapped (a Margin
// of margin 0 still adds 0 * d/|d|, as the reference does).
template <typename T>
struct Col {
    int type, nv, off, wrapped, idx;
    T R[9], t[3], p[3], m;
};

// True iff both collider indices of a pair lie in [0, n_colliders).  Every
// kernel that takes caller indices tests them before reading a record; a pair
// that fails gets D3D_STATUS_BAD_INDEX and touches no store memory.
__device__ __forceinline__ bool index_ok(const d3d_store& s, int i) {
    return (unsigned long long)(unsigned)i < (unsigned long long)s.n_colliders;
}
__device__ __forceinline__ bool pair_ok(const d3d_store& s, int a, int b) { return index_ok(s, a) && index_ok(s, b); }

// The EPA slots of such a pair.
__device__ __forceinline__ void epa_store_bad_index(double* mtv, int8_t* status, int32_t* n_faces, int64_t k) {
    mtv[3 * k] = NAN;
    mtv[3 * k + 1] = NAN;
    mtv[3 * k + 2] = NAN;
    status[k] = (int8_t)D3D_STATUS_BAD_INDEX;
    n_faces[k] = 0;
}

__device__ __forceinline__ void load_meta(const d3d_store& s, int idx, int& type, int& nv, int& off) {
    int4 m = __ldg(reinterpret_cast<const int4*>(s.meta) + idx);
    type = m.x;
    nv = m.y;
    off = m.z;
}
template <typename T>
__device__ __forceinline__ void load_meta(const d3d_store& s, int idx, Col<T>& c) {
    int4 m = __ldg(reinterpret_cast<const int4*>(s.meta) + idx);
    c.type = m.x;
    c.nv = m.y;
    c.off = m.z;
    c.wrapped = m.w;
    c.idx = idx;
}

__device__ __forceinline__ void load_col(const d3d_store& s, int idx, Col<double>& c) {
    load_meta(s, idx, c);
    const double2* r = reinterpret_cast<const double2*>(s.rec64) + (size_t)idx * 8;
    double v[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        double2 q = __ldg(r + k);
        v[2 * k] = q.x;
        v[2 * k + 1] = q.y;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) c.R[k] = v[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c.t[k] = v[9 + k];
        c.p[k] = v[12 + k];
    }
    c.m = v[15];
}

__device__ __forceinline__ void load_col(const d3d_store& s, int idx, Col<float>& c) {
    load_meta(s, idx, c);
    const float4* r = reinterpret_cast<const float4*>(s.rec32) + (size_t)idx * 4;
    float v[16];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float4 q = __ldg(r + k);
        v[4 * k] = q.x;
        v[4 * k + 1] = q.y;
        v[4 * k + 2] = q.z;
        v[4 * k + 3] = q.w;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) c.R[k] = v[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        c.t[k] = v[9 + k];
        c.p[k] = v[12 + k];
    }
    c.m = v[15];
}

__device__ __forceinline__ d3 load_vertex(const double* verts, int row) {
    const double2* v = reinterpret_cast<const double2*>(verts) + (size_t)row * 2;
    double2 a = __ldg(v), b = __ldg(v + 1);
    return mk(a.x, a.y, b.x);
}
__device__ __forceinline__ f3 load_vertex(const float* verts, int row) {
    float4 a = __ldg(reinterpret_cast<const float4*>(verts) + row);
    return mk(a.x, a.y, a.z);
}

// R^T d (np.dot(pose[:3, :3].T, d))
template <typename T>
__device__ __forceinline__ V3<T> rt_mul(const T* R, V3<T> d) {
    return mk(dot102(R[0], R[3], R[6], d.x, d.y, d.z), dot102(R[1], R[4], R[7], d.x, d.y, d.z),
              dot102(R[2], R[5], R[8], d.x, d.y, d.z));
}
// t + R v (utils.py:125-143 transform_point)
template <typename T>
__device__ __forceinline__ V3<T> xform(const T* R, const T* t, V3<T> v) {
    return mk(t[0] + dot102(R[0], R[1], R[2], v.x, v.y, v.z), t[1] + dot102(R[3], R[4], R[5], v.x, v.y, v.z),
              t[2] + dot102(R[6], R[7], R[8], v.x, v.y, v.z));
}

// Index of the first maximum of V . d over a hull's vertices
// (np.argmax(vertices.dot(d)), colliders.py:131-132).  A one-row vertex
// array goes through ddot instead of gemv, hence the dot012 special case.
template <typename T>
__device__ __forceinline__ int hull_argmax(const T* verts, int off, int nv, V3<T> d) {
    if (nv == 1) return 0;
    int best = 0;
    V3<T> v = load_vertex(verts, off);
    T bd = dot102(v.x, v.y, v.z, d.x, d.y, d.z);
    for (int k = 1; k < nv; ++k) {
        v = load_vertex(verts, off + k);
        T s = dot102(v.x, v.y, v.z, d.x, d.y, d.z);
        if (s > bd) {
            bd = s;
            best = k;
        }
    }
    return best;
}

// The same first maximum over the FP64 vertices (v64), found with the FP32
// mirror (v32, each coordinate the FP64 one rounded to nearest) so that the
// FP64 pipe evaluates only the vertices that can win.  For vertex k the FP32
// product s_k = v32_k . d32 (dot102 order) and the FP64 product the
// reference computes differ by at most
//     E_k = 2^-20 S_k + 2^-126 (|v32_k|_1 + |d32|_1 + 1),   S_k = sum_i |v32_ki d32_i|
// (16 unit roundoffs of the FP32 operands and products, 2^-24 each, plus an
// absolute term that covers denormal operands).  A first FP32 pass finds
// L = max_k (s_k - E_k), a lower bound on the FP64 maximum; the second pass
// computes the FP64 product only where s_k + E_k >= L, in index order with
// the strict comparison of hull_argmax.  Every vertex it skips has an FP64
// product below L, so the index is hull_argmax's, bit for bit.  With a
// non-finite FP32 value (NaN or infinite coordinates, or magnitudes beyond
// FP32) the plain FP64 scan runs instead.
struct Filter32 {
    float dx, dy, dz, dabs;
};
__device__ __forceinline__ Filter32 filter32(V3<double> d) {
    Filter32 f;
    f.dx = __double2float_rn(d.x);
    f.dy = __double2float_rn(d.y);
    f.dz = __double2float_rn(d.z);
    f.dabs = fabsf(f.dx) + fabsf(f.dy) + fabsf(f.dz);
    return f;
}
// (s_k, E_k) of vertex row `row` of the FP32 mirror
__device__ __forceinline__ float2 filter_product(const float* v32, int row, const Filter32& f) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(v32) + row);
    const float s = fmaf(v.z, f.dz, fmaf(v.x, f.dx, v.y * f.dy));
    const float sa = fmaf(fabsf(v.z), fabsf(f.dz), fmaf(fabsf(v.x), fabsf(f.dx), fabsf(v.y) * fabsf(f.dy)));
    const float e = fmaf(sa, 0x1p-20f, 0x1p-126f * (fabsf(v.x) + fabsf(v.y) + fabsf(v.z) + f.dabs + 1.f));
    return make_float2(s, e);
}

__device__ __forceinline__ int hull_argmax_filtered(const double* v64, const float* v32, int off, int nv, V3<double> d) {
    if (nv <= 1) return 0;
    const Filter32 f = filter32(d);
    float lo = -INFINITY;
    bool finite = isfinite(f.dabs);
#pragma unroll 1
    for (int k = 0; k < nv; ++k) {
        const float2 se = filter_product(v32, off + k, f);
        finite &= isfinite(se.x) && isfinite(se.y);
        lo = fmaxf(lo, se.x - se.y);
    }
    // not finite: every vertex is a candidate, which is hull_argmax's scan
    const bool all = !finite;
    int best = -1;
    double bd = 0.0;
#pragma unroll 1
    for (int k = 0; k < nv; ++k) {
        const float2 se = filter_product(v32, off + k, f);
        if (all || se.x + se.y >= lo) {
            const V3<double> w = load_vertex(v64, off + k);
            const double x = dot102(w.x, w.y, w.z, d.x, d.y, d.z);
            if (best < 0 || x > bd) {
                bd = x;
                best = k;
            }
        }
    }
    return best;
}

// The first-maximum vertex of a box or hull in the store: FP64 through the
// FP32 filter, FP32 directly.
__device__ __forceinline__ int polytope_argmax(const d3d_store& st, int off, int nv, V3<double> d) {
    return hull_argmax_filtered(st.verts64, st.verts32, off, nv, d);
}
__device__ __forceinline__ int polytope_argmax(const d3d_store& st, int off, int nv, V3<float> d) {
    return hull_argmax(st.verts32, off, nv, d);
}

// utils.py:78-122 plane_basis_from_normal: x, y of the plane with normal n
// (unfused Python scalar arithmetic); the record of a disk stores them as R
// columns 0 and 1.
template <typename T>
__device__ __forceinline__ void plane_basis(T n0, T n1, T n2, V3<T>& x, V3<T>& y) {
    if (abs_t(n0) >= abs_t(n1)) {
        const T len = sqrt_t(n0 * n0 + n2 * n2);
        x = mk(-n2 / len, T(0), n0 / len);
        y = mk(n1 * x.z, n2 * x.x - n0 * x.z, -n1 * x.x);
    } else {
        const T len = sqrt_t(n1 * n1 + n2 * n2);
        x = mk(T(0), n2 / len, -n1 / len);
        y = mk(n1 * x.z - n2 * x.y, -n0 * x.z, n0 * x.y);
    }
}

// Cone (geometry.py:421-455): the disk point of the local direction l, and
// whether the rim wins over the tip (np.dot(local_dir, disk_point) >=
// local_dir[2] * height).  The FP32 refinement of the mixed form repeats this
// decision on the FP32 record.
template <typename T>
__device__ __forceinline__ bool cone_rim(const Col<T>& c, V3<T> l, V3<T>& q) {
    const T n = sqrt_t(fma_t(l.y, l.y, l.x * l.x));
    if (n == T(0)) {
        q = mk(T(0), T(0), T(0));
    } else {
        const T f = c.p[0] / n;
        q = mk(l.x * f, l.y * f, T(0) * f);
    }
    return dot(l, q) >= l.z * c.p[1];
}

__device__ __forceinline__ const double* store_verts(const d3d_store& s, double) { return s.verts64; }
__device__ __forceinline__ const float* store_verts(const d3d_store& s, float) { return s.verts32; }

// mesh.py:12-127 hill_climb_mesh_extreme for the mesh-frame direction l:
// from the start vertex, the six shortcut vertices, then passes over the
// neighbours of the vertex a pass starts at (the reference iterates that
// vertex's list even after it has moved), moving whenever the projection of
// the step exceeds 10 EPSILON (PROJECTION_LENGTH_EPSILON).  The climb
// strictly increases the projection, so it ends within nv passes; the bound
// is a guard.  Out-of-range links are skipped.
template <typename T>
__device__ __forceinline__ int mesh_climb_body(const T* __restrict__ verts, const int32_t* __restrict__ blk, int off,
                                               int nv, int best, T lx, T ly, T lz) {
    const V3<T> l = mk(lx, ly, lz);
    const T eps = T(10.0 * DBL_EPSILON);
    if (best < 0 || best >= nv) best = 0;
    V3<T> vb = load_vertex(verts, off + best);
    for (int k = 0; k < 6; ++k) {
        const int cand = __ldg(blk + k);
        if (cand < 0 || cand >= nv) continue;
        const V3<T> v = load_vertex(verts, off + cand);
        if (dot(l, v - vb) > eps) {
            best = cand;
            vb = v;
        }
    }
    for (int pass = 0; pass <= nv; ++pass) {
        bool converged = true;
        const int lo = __ldg(blk + 6 + best), hi = __ldg(blk + 7 + best);
        for (int e = lo; e < hi; ++e) {
            const int cand = __ldg(blk + e);
            if (cand < 0 || cand >= nv) continue;
            const V3<T> v = load_vertex(verts, off + cand);
            if (dot(l, v - vb) > eps) {
                best = cand;
                vb = v;
                converged = false;
            }
        }
        if (converged) break;
    }
    return best;
}

// The same as a call (scalar arguments, nothing through the stack), for
// kernels that keep the climb out of their hot loop.
template <typename T>
__device__ __noinline__ int mesh_climb_call(const T* __restrict__ verts, const int32_t* __restrict__ blk, int off,
                                            int nv, int best, T lx, T ly, T lz) {
    return mesh_climb_body(verts, blk, off, nv, best, lx, ly, lz);
}

// The climb for collider c, inlined (CALL = false) or called.  The links
// offset and the start vertex are read from the FP64 record (exact integers
// there; the FP32 record cannot hold large offsets).  `from` >= 0 starts the
// climb at that vertex instead (the reference's cached answer of its
// previous call, mesh.py:84-85); out-of-range values start at vertex 0, as
// mesh_climb_body clamps them.
template <bool CALL = false, typename T>
__device__ __forceinline__ int mesh_climb(const Col<T>& c, const d3d_store& st, V3<T> l, int from = -1) {
    const double* rec = st.rec64 + (size_t)c.idx * 16;
    const int32_t* blk = st.links + (int64_t)__ldg(rec + 12);
    const int start = from >= 0 ? from : (int)__ldg(rec + 13);
    if (CALL) return mesh_climb_call(store_verts(st, T(0)), blk, c.off, c.nv, start, l.x, l.y, l.z);
    return mesh_climb_body(store_verts(st, T(0)), blk, c.off, c.nv, start, l.x, l.y, l.z);
}

// Support point of the collider itself (without its margin) along d.  Sphere
// geometry.py:314-346, capsule :209-256, cylinder :160-206, ellipsoid
// :259-284 (norm_vector utils.py:12-30), disk :353-387, ellipse :390-418,
// cone :421-455; box and hull: first-maximum vertex (colliders.py:131-132);
// mesh: hill climb (mesh.py:77-85).  Without `cache` each mesh call starts
// from the mesh's start vertex; with it, the climb starts from *cache (a
// negative value: the start vertex) and leaves its answer there, the vertex
// caching of the reference's support object.
template <typename T>
__device__ __forceinline__ V3<T> base_support(const Col<T>& c, const d3d_store& st, V3<T> d, int* cache = nullptr) {
    const T* verts = store_verts(st, T(0));
    switch (c.type) {
    case D3D_SPHERE: {
        T n = sqrt_t(dot(d, d));
        V3<T> ctr = mk(c.t[0], c.t[1], c.t[2]);
        if (n == T(0)) return ctr + mk(T(0), T(0), c.p[0]);
        return ctr + mk(d.x / n * c.p[0], d.y / n * c.p[0], d.z / n * c.p[0]);
    }
    case D3D_CAPSULE: {
        V3<T> l = rt_mul(c.R, d);
        T s = sqrt_t(l.x * l.x + l.y * l.y + l.z * l.z);
        V3<T> v;
        if (s == T(0)) {
            v = mk(c.p[0], T(0), T(0));
        } else {
            T f = c.p[0] / s;
            v = mk(l.x * f, l.y * f, l.z * f);
        }
        if (l.z > T(0))
            v.z += T(0.5) * c.p[1];
        else
            v.z -= T(0.5) * c.p[1];
        return xform(c.R, c.t, v);
    }
    case D3D_CYLINDER: {
        V3<T> l = rt_mul(c.R, d);
        T s = sqrt_t(l.x * l.x + l.y * l.y);
        T z = (l.z < T(0)) ? T(-0.5) * c.p[1] : T(0.5) * c.p[1];
        V3<T> v;
        if (s == T(0)) {
            v = mk(c.p[0], T(0), z);
        } else {
            T f = c.p[0] / s;
            v = mk(l.x * f, l.y * f, z);
        }
        return xform(c.R, c.t, v);
    }
    case D3D_ELLIPSOID: {
        V3<T> l = rt_mul(c.R, d);
        V3<T> a = mk(l.x * c.p[0], l.y * c.p[1], l.z * c.p[2]);
        T n = sqrt_t(dot(a, a));
        if (n != T(0)) a = mk(a.x / n, a.y / n, a.z / n);
        a = mk(a.x * c.p[0], a.y * c.p[1], a.z * c.p[2]);
        return xform(c.R, c.t, a);
    }
    case D3D_DISK: {
        // point = np.dot(R.T, d) with R = column_stack(x, y, normal); the
        // third component is dropped; center + np.dot(R, point)
        const T p0 = dot012(c.R[0], c.R[3], c.R[6], d.x, d.y, d.z);
        const T p1 = dot012(c.R[1], c.R[4], c.R[7], d.x, d.y, d.z);
        const T n = sqrt_t(fma_t(p1, p1, p0 * p0));
        const V3<T> ctr = mk(c.t[0], c.t[1], c.t[2]);
        if (n == T(0)) return ctr;
        const T f = c.p[0] / n;
        const T q0 = p0 * f, q1 = p1 * f, q2 = T(0) * f;
        return ctr + mk(dot102(c.R[0], c.R[1], c.R[2], q0, q1, q2), dot102(c.R[3], c.R[4], c.R[5], q0, q1, q2),
                        dot102(c.R[6], c.R[7], c.R[8], q0, q1, q2));
    }
    case D3D_ELLIPSE: {
        // axes.dot(d) over the two axis rows; norm_vector(radii * l) * radii;
        // center + np.dot(l, axes)
        T v0 = c.p[0] * dot102(c.R[0], c.R[3], c.R[6], d.x, d.y, d.z);
        T v1 = c.p[1] * dot102(c.R[1], c.R[4], c.R[7], d.x, d.y, d.z);
        const T n = sqrt_t(fma_t(v1, v1, v0 * v0));
        if (n != T(0)) {
            v0 = v0 / n;
            v1 = v1 / n;
        }
        v0 = v0 * c.p[0];
        v1 = v1 * c.p[1];
        return mk(c.t[0] + fma_t(v1, c.R[1], v0 * c.R[0]), c.t[1] + fma_t(v1, c.R[4], v0 * c.R[3]),
                  c.t[2] + fma_t(v1, c.R[7], v0 * c.R[6]));
    }
    case D3D_CONE: {
        const V3<T> l = rt_mul(c.R, d);
        V3<T> q;
        if (!cone_rim(c, l, q)) q = mk(T(0), T(0), c.p[1]);
        return xform(c.R, c.t, q);
    }
    case D3D_MESH: {
        if (c.nv < 1) return mk(T(NAN), T(NAN), T(NAN));  // rejected by d3d_store_pack
        const int k = mesh_climb(c, st, rt_mul(c.R, d), cache ? *cache : -1);
        if (cache) *cache = k;
        return xform(c.R, c.t, load_vertex(verts, c.off + k));
    }
    default:
        if (c.nv < 1) return mk(T(NAN), T(NAN), T(NAN));  // rejected by d3d_store_pack
        return load_vertex(verts, c.off + polytope_argmax(st, c.off, c.nv, d));
    }
}

// Margin (colliders.py:629-631): s + margin * norm_vector(d), the zero
// direction staying zero (utils.py:26-30).
template <typename T>
__device__ __forceinline__ V3<T> add_margin(const Col<T>& c, V3<T> s, V3<T> d) {
    if (!c.wrapped) return s;
    const T n = sqrt_t(dot(d, d));
    const V3<T> u = n == T(0) ? d : mk(d.x / n, d.y / n, d.z / n);
    return mk(s.x + c.m * u.x, s.y + c.m * u.y, s.z + c.m * u.z);
}

template <typename T>
__device__ __forceinline__ V3<T> support(const Col<T>& c, const d3d_store& st, V3<T> d, int* cache = nullptr) {
    return add_margin(c, base_support(c, st, d, cache), d);
}

}  // namespace d3d
