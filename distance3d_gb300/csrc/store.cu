// store.cu -- the device collider store: packing, pose updates, support
// points and axis-aligned bounding boxes.  Compiled with -fmad=false: every
// value here must match the reference's FP64 rounding sequence.
#include "capi_util.h"
#include "d3d_device.cuh"

namespace {

using namespace d3d;

// geometry.py:135,138-157 convert_box_to_vertices:
// t + (BOX_COORDS * size) . R^T with BOX_COORDS in itertools.product order
__device__ void write_box_vertices(const d3d_store& s, int off, const double* R, const double* t,
                                   const double* size) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        double a0 = (((k >> 2) & 1) ? 0.5 : -0.5) * size[0];
        double a1 = (((k >> 1) & 1) ? 0.5 : -0.5) * size[1];
        double a2 = ((k & 1) ? 0.5 : -0.5) * size[2];
        double v[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) v[i] = t[i] + dot012(a0, a1, a2, R[i * 3], R[i * 3 + 1], R[i * 3 + 2]);
        double2* d = reinterpret_cast<double2*>(s.verts64) + (size_t)(off + k) * 2;
        d[0] = make_double2(v[0], v[1]);
        d[1] = make_double2(v[2], 0.0);
        reinterpret_cast<float4*>(s.verts32)[off + k] =
            make_float4(__double2float_rn(v[0]), __double2float_rn(v[1]), __double2float_rn(v[2]), 0.f);
    }
}

// A disk's rotation is column_stack(x, y, normal) with x, y derived from its
// normal, R column 2 (colliders.py:483-487 keeps only the normal of a pose;
// geometry.py:375-376 derives the basis in every support call).
__device__ void canonical_rotation(int type, double* R) {
    if (type != D3D_DISK) return;
    d3 x, y;
    plane_basis(R[2], R[5], R[8], x, y);
    R[0] = x.x;
    R[3] = x.y;
    R[6] = x.z;
    R[1] = y.x;
    R[4] = y.y;
    R[7] = y.z;
}

__device__ void write_record(const d3d_store& s, int i, const double* R, const double* t, const double* p,
                             double margin) {
    double* r = s.rec64 + (size_t)i * 16;
    float* f = s.rec32 + (size_t)i * 16;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        r[k] = R[k];
        f[k] = __double2float_rn(R[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r[9 + k] = t[k];
        f[9 + k] = __double2float_rn(t[k]);
        r[12 + k] = p[k];
        f[12 + k] = __double2float_rn(p[k]);
    }
    r[15] = margin;
    f[15] = __double2float_rn(margin);
}

__global__ void k_pack(d3d_store s, const int32_t* __restrict__ types, const double* __restrict__ poses,
                       const double* __restrict__ params, const int64_t* __restrict__ hull_offset,
                       const int32_t* __restrict__ hull_count, int64_t n, int* __restrict__ bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int wrapped = (types[i] & D3D_MARGIN) ? 1 : 0;
    const int type = types[i] & ~D3D_MARGIN;
    double R[9], t[3], p[3];
    for (int k = 0; k < 9; ++k) R[k] = poses[i * 12 + k];
    for (int k = 0; k < 3; ++k) {
        t[k] = poses[i * 12 + 9 + k];
        p[k] = params[i * 4 + k];
    }
    canonical_rotation(type, R);
    write_record(s, (int)i, R, t, p, wrapped ? params[i * 4 + 3] : 0.0);
    int count = 0, off = 0;
    if (type == D3D_BOX) {
        count = 8;
        int64_t o = hull_offset[i];
        if (o < 0 || o + 8 > s.n_vertices) {
            atomicExch(bad, 1);
            count = 0;
        } else {
            off = (int)o;
            write_box_vertices(s, off, R, t, p);
        }
    } else if (type == D3D_HULL || type == D3D_MESH) {
        int64_t o = hull_offset[i];
        count = hull_count[i];
        bool ok = o >= 0 && count >= 1 && o + count <= s.n_vertices;
        if (ok && type == D3D_MESH) {
            // links block: 6 shortcuts, count + 1 offsets, the lists (mesh.py:26-52)
            const double b = p[0], start = p[1];
            ok = b >= 0.0 && b == floor(b) && b + 7.0 + count <= (double)s.n_links && start >= 0.0 &&
                 start < (double)count && start == floor(start);
            if (ok) {
                const int32_t* blk = s.links + (int64_t)b;
                ok = blk[6] == 7 + count && blk[6 + count] >= blk[6] && (int64_t)b + blk[6 + count] <= s.n_links;
            }
        }
        if (!ok) {
            atomicExch(bad, 1);
            count = 0;
        } else {
            off = (int)o;
        }
    } else if (type < 0 || type > D3D_MESH) {
        atomicExch(bad, 1);
    }
    reinterpret_cast<int4*>(s.meta)[i] = make_int4(type, count, off, wrapped);
}

__global__ void k_hull_to_f32(d3d_store s, int64_t rows) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const double2* v = reinterpret_cast<const double2*>(s.verts64) + r * 2;
    double2 a = v[0], b = v[1];
    reinterpret_cast<float4*>(s.verts32)[r] =
        make_float4(__double2float_rn(a.x), __double2float_rn(a.y), __double2float_rn(b.x), 0.f);
}

__global__ void k_set_poses(d3d_store s, const int32_t* __restrict__ idx, const double* __restrict__ poses,
                            int64_t n) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int i = idx[k];
    if (i < 0 || i >= s.n_colliders) return;
    double R[9], t[3], p[3];
    for (int j = 0; j < 9; ++j) R[j] = poses[k * 12 + j];
    for (int j = 0; j < 3; ++j) {
        t[j] = poses[k * 12 + 9 + j];
        p[j] = s.rec64[(size_t)i * 16 + 12 + j];
    }
    int type, nv, off;
    load_meta(s, i, type, nv, off);
    if (type == D3D_HULL) return;
    canonical_rotation(type, R);
    write_record(s, i, R, t, p, s.rec64[(size_t)i * 16 + 15]);
    if (type == D3D_BOX && nv == 8) write_box_vertices(s, off, R, t, p);
}

__global__ void k_support(d3d_store s, const int32_t* __restrict__ idx, const double* __restrict__ dirs,
                          int64_t n, double* __restrict__ out) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = idx[k];
    if (!index_ok(s, i)) {  // out of range: NaN, no record read
        out[3 * k] = out[3 * k + 1] = out[3 * k + 2] = NAN;
        return;
    }
    Col<double> c;
    load_col(s, i, c);
    d3 r = support(c, s, mk(dirs[3 * k], dirs[3 * k + 1], dirs[3 * k + 2]));
    out[3 * k] = r.x;
    out[3 * k + 1] = r.y;
    out[3 * k + 2] = r.z;
}

// np.minimum / np.maximum: a NaN operand gives NaN
__device__ __forceinline__ double np_min(double a, double b) { return (a != a || a < b) ? a : b; }
__device__ __forceinline__ double np_max(double a, double b) { return (a != a || a > b) ? a : b; }

// containment.py:25-229: the box of a collider of an analytic type (the
// polytopes and meshes are scanned by aabb_scan)
__device__ void analytic_aabb(const Col<double>& c, double* lo, double* hi) {
    const double* R = c.R;
    const double* t = c.t;
    switch (c.type) {
    case D3D_SPHERE:  // :25-44
        for (int i = 0; i < 3; ++i) {
            lo[i] = t[i] - c.p[0];
            hi[i] = t[i] + c.p[0];
        }
        break;
    case D3D_CAPSULE:  // :99-122
        for (int i = 0; i < 3; ++i) {
            double e = 0.5 * c.p[1] * fabs(R[i * 3 + 2]) + c.p[0];
            lo[i] = t[i] - e;
            hi[i] = t[i] + e;
        }
        break;
    case D3D_CYLINDER:  // :70-96
        for (int i = 0; i < 3; ++i) {
            double a = R[i * 3 + 2];
            double e = 0.5 * c.p[1] * fabs(a) + c.p[0] * sqrt(1.0 - a * a);
            lo[i] = t[i] - e;
            hi[i] = t[i] + e;
        }
        break;
    case D3D_ELLIPSOID: {  // :125-148
        double E[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) E[i * 3 + j] = R[i * 3 + j] * c.p[j];
        for (int j = 0; j < 3; ++j) {
            double nn = sqrt((E[j] * E[j] + E[3 + j] * E[3 + j]) + E[6 + j] * E[6 + j]);
            for (int i = 0; i < 3; ++i) E[i * 3 + j] = E[i * 3 + j] / nn;
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) E[i * 3 + j] = E[i * 3 + j] * c.p[j];
        for (int kk = 0; kk < 3; ++kk) {
            double m = 0.0;
            for (int i = 0; i < 3; ++i) {
                double v = dot012(R[i * 3], R[i * 3 + 1], R[i * 3 + 2], E[kk * 3], E[kk * 3 + 1], E[kk * 3 + 2]);
                if (i == 0 || v > m) m = v;
            }
            lo[kk] = t[kk] - m;
            hi[kk] = t[kk] + m;
        }
        break;
    }
    case D3D_DISK:  // :151-174
        for (int i = 0; i < 3; ++i) {
            const double a = R[i * 3 + 2];
            const double e = c.p[0] * sqrt(1.0 - a * a);
            lo[i] = t[i] - e;
            hi[i] = t[i] + e;
        }
        break;
    case D3D_ELLIPSE:  // :206-229
        for (int i = 0; i < 3; ++i) {
            const double a = c.p[0] * R[i * 3], b = c.p[1] * R[i * 3 + 1];
            const double e = sqrt(a * a + b * b);
            lo[i] = t[i] - e;
            hi[i] = t[i] + e;
        }
        break;
    case D3D_CONE:  // :177-203
        for (int i = 0; i < 3; ++i) {
            const double pb = t[i] + c.p[1] * R[i * 3 + 2];
            const double a = pb - t[i];
            const double e = sqrt(1.0 - a * a / (c.p[1] * c.p[1]));
            lo[i] = np_min(t[i] - e * c.p[0], pb);
            hi[i] = np_max(t[i] + e * c.p[0], pb);
        }
        break;
    default:
        break;
    }
}

// Ordering key of a coordinate for the min / max scans: unsigned order equals
// the order of the doubles, -0 and +0 equal (the scan keeps the first).
__device__ __forceinline__ unsigned long long coord_key(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if ((u << 1) == 0ull) return 0x8000000000000000ull;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// The warp's smallest (key, index): REDUX on the key halves, then on the index.
__device__ __forceinline__ int warp_first_min(unsigned long long k, int i) {
    const unsigned hi = __reduce_min_sync(0xffffffffu, (unsigned)(k >> 32));
    const unsigned lo = __reduce_min_sync(0xffffffffu, (unsigned)(k >> 32) == hi ? (unsigned)k : 0xffffffffu);
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    return (int)__reduce_min_sync(0xffffffffu, k == m ? (unsigned)i : 0xffffffffu);
}

// Per axis the minimum and maximum of a polytope's or mesh's coordinates, by
// the 32 lanes of the warp (every lane calls it with the same collider): box
// :47-67 and hull :6-22 (np.min / np.max of the vertices), mesh
// colliders.py:234-237 (t + V R^T, dgemm in the order of dot012).  The values
// are those of the sequential scan that starts from vertex 0 and replaces on
// a strict comparison: the first of equal values (-0 and +0 included), a NaN
// coordinate of vertex 0 kept, later NaNs skipped.  The compares are integer
// ones, off the FP64 pipe.
__device__ void aabb_scan(const d3d_store& s, int off, int nv, bool mesh, const double* R, const double* t,
                          double* lo, double* hi) {
    const int ln = threadIdx.x & 31;
    unsigned long long kmin[3], kmax[3];
    int imin[3], imax[3];
    double vmin[3], vmax[3], v0[3];
    for (int i = 0; i < 3; ++i) {
        kmin[i] = ~0ull;
        kmax[i] = 0ull;
        imin[i] = imax[i] = 0x7fffffff;
        vmin[i] = vmax[i] = v0[i] = 0.0;
    }
    for (int r = ln; r < nv; r += 32) {
        const d3 v = load_vertex(s.verts64, off + r);
        double w[3] = {v.x, v.y, v.z};
        if (mesh)
            for (int i = 0; i < 3; ++i) w[i] = t[i] + dot012(v.x, v.y, v.z, R[i * 3], R[i * 3 + 1], R[i * 3 + 2]);
        for (int i = 0; i < 3; ++i) {
            if (r == 0) v0[i] = w[i];
            if (w[i] != w[i]) continue;
            const unsigned long long key = coord_key(w[i]);
            if (key < kmin[i]) {
                kmin[i] = key;
                imin[i] = r;
                vmin[i] = w[i];
            }
            if (key > kmax[i]) {
                kmax[i] = key;
                imax[i] = r;
                vmax[i] = w[i];
            }
        }
    }
    for (int i = 0; i < 3; ++i) {
        const int a = warp_first_min(kmin[i], imin[i]);
        const int b = warp_first_min(~kmax[i], imax[i]);
        const double x0 = __shfl_sync(0xffffffffu, v0[i], 0);
        // the winner's value from the lane that holds it (vertex r sits on lane r % 32); every
        // value a NaN: vertex 0's, as the scan keeps it
        const double xa = __shfl_sync(0xffffffffu, vmin[i], a == 0x7fffffff ? 0 : (a & 31));
        const double xb = __shfl_sync(0xffffffffu, vmax[i], b == 0x7fffffff ? 0 : (b & 31));
        lo[i] = (x0 != x0 || a == 0x7fffffff) ? x0 : xa;
        hi[i] = (x0 != x0 || b == 0x7fffffff) ? x0 : xb;
    }
}

// containment.py:6-229, one collider per thread; writes [axis][min,max].  The
// analytic types each on its own thread; the boxes, hulls and meshes of a
// warp's lanes one after the other by the whole warp (aabb_scan), so that no
// thread scans up to 256 vertices alone.
__global__ void k_aabbs(d3d_store s, const int32_t* __restrict__ idx, int64_t n, double* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ln = threadIdx.x & 31;
    const bool valid = k < n;
    const int ci = valid ? (idx ? idx[k] : (int)k) : 0;
    const bool ok = valid && index_ok(s, ci);
    if (valid && !ok)  // out of range: NaN, no record read
        for (int j = 0; j < 6; ++j) out[6 * k + j] = NAN;
    Col<double> c;
    bool poly = false;
    double lo[3], hi[3];
    if (ok) {
        load_col(s, ci, c);
        poly = c.type == D3D_BOX || c.type == D3D_HULL || c.type == D3D_MESH;
        if (!poly) analytic_aabb(c, lo, hi);
        else if (c.nv < 1)  // rejected by d3d_store_pack
            for (int i = 0; i < 3; ++i) lo[i] = hi[i] = NAN;
    }
    // the lanes' polytopes and meshes, one at a time across the warp
    unsigned todo = __ballot_sync(0xffffffffu, ok && poly && c.nv >= 1);
    while (todo) {
        const int owner = __ffs(todo) - 1;
        todo &= todo - 1;
        const int off = __shfl_sync(0xffffffffu, ok ? c.off : 0, owner);
        const int nv = __shfl_sync(0xffffffffu, ok ? c.nv : 0, owner);
        const bool mesh = __shfl_sync(0xffffffffu, ok && c.type == D3D_MESH ? 1 : 0, owner) != 0;
        double R[9] = {}, t[3] = {};  // read only for a mesh
        if (mesh) {
            for (int j = 0; j < 9; ++j) R[j] = __shfl_sync(0xffffffffu, ok ? c.R[j] : 0.0, owner);
            for (int j = 0; j < 3; ++j) t[j] = __shfl_sync(0xffffffffu, ok ? c.t[j] : 0.0, owner);
        }
        double l[3], h[3];
        aabb_scan(s, off, nv, mesh, R, t, l, h);
        if (ln == owner)
            for (int i = 0; i < 3; ++i) {
                lo[i] = l[i];
                hi[i] = h[i];
            }
    }
    if (!ok) return;
    if (c.wrapped) {  // colliders.py:639-643
        for (int i = 0; i < 3; ++i) {
            lo[i] = lo[i] - c.m;
            hi[i] = hi[i] + c.m;
        }
    }
    for (int i = 0; i < 3; ++i) {
        out[6 * k + 2 * i] = lo[i];
        out[6 * k + 2 * i + 1] = hi[i];
    }
}

}  // namespace

extern "C" int d3d_store_pack(const d3d_store* store, const int32_t* types, const double* poses,
                              const double* params, const int64_t* hull_offset, const int32_t* hull_count,
                              int64_t n_hull_vertices, void* stream) {
    int rc = d3d::check_store(store, "d3d_store_pack");
    if (rc) return rc;
    const int64_t n = store->n_colliders;
    D3D_REQUIRE(n == 0 || (types && poses && params && hull_offset && hull_count),
                "d3d_store_pack: null input array");
    D3D_REQUIRE(n_hull_vertices >= 0 && n_hull_vertices <= store->n_vertices,
                "d3d_store_pack: n_hull_vertices %lld outside [0, %lld]", (long long)n_hull_vertices,
                (long long)store->n_vertices);
    cudaStream_t st = d3d::as_stream(stream);
    int* bad = nullptr;
    if (cudaMallocAsync(&bad, sizeof(int), st) != cudaSuccess || cudaMemsetAsync(bad, 0, sizeof(int), st) != cudaSuccess)
        return d3d::check_launch("d3d_store_pack: flag");
    if (n_hull_vertices > 0) k_hull_to_f32<<<d3d::grid_for(n_hull_vertices, 256), 256, 0, st>>>(*store, n_hull_vertices);
    if (n > 0)
        k_pack<<<d3d::grid_for(n, 128), 128, 0, st>>>(*store, types, poses, params, hull_offset, hull_count, n, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(bad, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_store_pack: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    D3D_REQUIRE(!hbad, "d3d_store_pack: a collider has an unknown type or a vertex range outside the pool");
    return d3d::check_launch("d3d_store_pack");
}

extern "C" int d3d_store_set_poses(const d3d_store* store, const int32_t* idx, const double* poses, int64_t n,
                                   void* stream) {
    int rc = d3d::check_store(store, "d3d_store_set_poses");
    if (rc) return rc;
    D3D_REQUIRE(n >= 0, "d3d_store_set_poses: n < 0");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(idx && poses, "d3d_store_set_poses: null pointer");
    k_set_poses<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(*store, idx, poses, n);
    return d3d::check_launch("d3d_store_set_poses");
}

extern "C" int d3d_support(const d3d_store* store, const int32_t* idx, const double* dirs, int64_t n, double* out,
                           void* stream) {
    int rc = d3d::check_store(store, "d3d_support");
    if (rc) return rc;
    D3D_REQUIRE(n >= 0, "d3d_support: n < 0");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(idx && dirs && out, "d3d_support: null pointer");
    k_support<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(*store, idx, dirs, n, out);
    return d3d::check_launch("d3d_support");
}

extern "C" int d3d_aabbs(const d3d_store* store, const int32_t* idx, int64_t n, double* out, void* stream) {
    int rc = d3d::check_store(store, "d3d_aabbs");
    if (rc) return rc;
    D3D_REQUIRE(n >= 0, "d3d_aabbs: n < 0");
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(out, "d3d_aabbs: null output");
    D3D_REQUIRE(idx || n <= store->n_colliders, "d3d_aabbs: n > n_colliders");
    k_aabbs<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(*store, idx, n, out);
    return d3d::check_launch("d3d_aabbs");
}
