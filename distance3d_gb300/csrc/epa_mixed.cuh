// epa_mixed.cuh -- device functions of the mixed-precision EPA (see
// epa_mixed.cu for the method): the FP32 polytope search as a per-lane state
// machine and the FP64 refinement of the final face.
#pragma once

#include "gjk_mixed.cuh"

namespace d3d {

constexpr int kEpaFallback = 100;  // pair handed to the FP64 EPA

// The FP32 search stops when the support along the closest face's normal
// rises above the face by less than max(epsilon, kSearchUlps FP32 machine
// epsilons of the polytope's scale).  The FP64 refinement then returns h(n), the
// support depth along that normal, which lies between the face's distance
// and the true depth plus that tolerance, so the depth error is at most
// about 32 * 2^-23 = 3.8e-6 of the scale, under the form's 1e-5.  On the
// bench workload's EPA pairs: 8 units gave 6.03 ms, max error 1.9e-6 and
// p99 5.7e-7; 16 gave 5.61 ms, 2.4e-6, 1.1e-6; 32 gives 5.24 ms, 4.5e-6,
// 2.2e-6 (and converges on more pairs within the iteration bound).
constexpr int kSearchUlps = 32;

// slot layout (bytes): vertices (max_iter + 4) x 32, faces max_faces x 32,
// edges max_loose_edges x 8, flood-fill queue max_faces x 4
struct Slot {
    float4* vy;   // y.xyz, w unused
    float4* vd;   // direction.xyz, w: input simplex row (0..3) for starting vertices, -1 otherwise
    int4* fi;     // vertex ids (x, y, z); w: iteration that marked the face visible
    float4* fn;   // normal.xyz, w = n . y0
    int2* edges;
    int* queue;
};

__device__ __forceinline__ Slot slot_at(char* base, const d3d_epa_options& o) {
    Slot s;
    const int nv = o.max_iterations + 4;
    s.vy = reinterpret_cast<float4*>(base);
    s.vd = s.vy + nv;
    s.fi = reinterpret_cast<int4*>(s.vd + nv);
    s.fn = reinterpret_cast<float4*>(s.fi + o.max_faces);
    s.edges = reinterpret_cast<int2*>(s.fn + o.max_faces);
    s.queue = reinterpret_cast<int*>(s.edges + o.max_loose_edges);
    return s;
}

__device__ __forceinline__ f3 y_of(const Slot& s, int v) {
    float4 a = s.vy[v];
    return mk(a.x, a.y, a.z);
}

// unit normal of (a, b, c) and plane offset; false if degenerate
__device__ __forceinline__ bool face_plane(const Slot& s, int a, int b, int c, float4& out) {
    f3 ya = y_of(s, a), yb = y_of(s, b), yc = y_of(s, c);
    f3 n = cross(yb - ya, yc - ya);
    float l = sqrtf(dot(n, n));
    if (!(l > 0.f)) return false;
    n = n * (1.f / l);
    out = make_float4(n.x, n.y, n.z, dot(ya, n));
    return true;
}

struct MixedEpa {
    int nv, nf, it, closest;
    float scale;  // max |y| so far
};

__device__ __forceinline__ void mepa_begin(MixedEpa& L, const Slot& s, const double* simplex) {
    float scale = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        f3 y = mk((float)simplex[3 * j], (float)simplex[3 * j + 1], (float)simplex[3 * j + 2]);
        s.vy[j] = make_float4(y.x, y.y, y.z, 0.f);
        s.vd[j] = make_float4(0.f, 0.f, 0.f, (float)j);
        scale = fmaxf(scale, sqrtf(dot(y, y)));
    }
    // faces ABC, ACD, ADB, BDC with the vertex each one leaves out
    const int init[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
    int nf = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float4 pl;
        int a = init[i][0], b = init[i][1], c = init[i][2];
        if (!face_plane(s, a, b, c, pl)) continue;
        // wind every face so that its normal points away from the opposite
        // vertex; new faces inherit this winding from their horizon edge
        const f3 yd = y_of(s, init[i][3]) - y_of(s, a);
        if (pl.x * yd.x + pl.y * yd.y + pl.z * yd.z > 0.f) {
            int t = a;
            a = b;
            b = t;
            pl = make_float4(-pl.x, -pl.y, -pl.z, -pl.w);
        }
        s.fi[nf] = make_int4(a, b, c, 0);
        s.fn[nf] = pl;
        ++nf;
    }
    L.nv = 4;
    L.nf = nf;
    L.it = 0;
    L.closest = 0;
    L.scale = scale;
}

// FP64 vertex v of the polytope
__device__ __forceinline__ d3 refine_vertex(const Slot& s, int v, const Col<double>& c1, const Col<double>& c2,
                                            const d3d_store& st, const double* simplex) {
    float4 d = s.vd[v];
    if (d.w >= 0.f) {
        int r = (int)d.w;
        return mk(simplex[3 * r], simplex[3 * r + 1], simplex[3 * r + 2]);
    }
    d3 dir = mk((double)d.x, (double)d.y, (double)d.z);
    return RefineSupport::eval(c1, st, dir) - RefineSupport::eval(c2, st, -dir);
}

// FP64 refinement of the closest face (see the file comment)
__device__ __forceinline__ d3 mepa_refine(const MixedEpa& L, const Slot& s, const d3d_store& st, int a, int b,
                                          const double* simplex) {
    const int4 f = s.fi[L.closest];
    if (L.nf == 0 || L.closest >= L.nf || f.x < 0 || f.x >= L.nv || f.y < 0 || f.y >= L.nv || f.z < 0 ||
        f.z >= L.nv)
        return mk(double(NAN), double(NAN), double(NAN));
    Col<double> c1, c2;
    load_col(st, a, c1);
    load_col(st, b, c2);
    d3 y0 = refine_vertex(s, f.x, c1, c2, st, simplex);
    d3 y1 = refine_vertex(s, f.y, c1, c2, st, simplex);
    d3 y2 = refine_vertex(s, f.z, c1, c2, st, simplex);
    // the face keeps the polytope's outward winding, so the FP64 normal of
    // the same vertex order points the way of the FP32 normal
    const float4 fn = s.fn[L.closest];
    const d3 n32 = mk((double)fn.x, (double)fn.y, (double)fn.z);
    d3 n = cross(y1 - y0, y2 - y0);
    double l = sqrt(dot(n, n));
    if (!(l > 0.0) || dot(n, n32) <= 0.0) {
        n = n32;
        l = sqrt(dot(n, n));
    }
    n = n * (1.0 / l);
    d3 w = RefineSupport::eval(c1, st, n) - RefineSupport::eval(c2, st, -n);
    return n * dot(w, n);
}

// one iteration of the FP32 search; -1 while running, else a status
__device__ __forceinline__ int mepa_step(MixedEpa& L, const Slot& s, const Col<float>& c1, const Col<float>& c2,
                                         const d3d_store& st, const d3d_epa_options& o) {
    if (L.it >= o.max_iterations) return D3D_STATUS_EPA_NOT_CONVERGED;
    ++L.it;
    const int nf = L.nf;
    if (nf == 0) return D3D_STATUS_EPA_DEGENERATE;
    float md = 0.f;
    int closest = 0;
    for (int i = 0; i < nf; ++i) {
        float d = s.fn[i].w;
        if (i == 0 || d < md) {
            md = d;
            closest = i;
        }
    }
    L.closest = closest;
    const float4 cn = s.fn[closest];
    const f3 sd = mk(cn.x, cn.y, cn.z);
    const f3 w = FastSupport::eval(c1, st, sd) - FastSupport::eval(c2, st, -sd);
    const float pd = dot(w, sd);
    const float wl = sqrtf(dot(w, w));
    L.scale = fmaxf(L.scale, wl);
    const float eps = fmaxf((float)o.epsilon, (float)kSearchUlps * FLT_EPSILON * L.scale);
    if (pd - md < eps) return D3D_STATUS_OK;
    if (L.nv >= o.max_iterations + 4) return D3D_STATUS_EPA_NOT_CONVERGED;
    const int nv = L.nv++;
    s.vy[nv] = make_float4(w.x, w.y, w.z, 0.f);
    s.vd[nv] = make_float4(sd.x, sd.y, sd.z, -1.f);
    // The faces that see w (epa.py:157-165), grown by flood fill from the
    // closest face (which sees w by the test above) across shared edges, so
    // that FP32 noise on far, nearly coplanar faces cannot make the visible
    // set disconnected.  Neighbours are found by vertex ids: the face across
    // edge (u, v) is the one holding (v, u).
    // visibility uses the reference's epsilon (epa.py:122-124); the FP32
    // noise floor above only decides convergence
    const float vis_eps = (float)o.epsilon;
    const int stamp = L.it;
    s.fi[closest].w = stamp;
    s.queue[0] = closest;
    int qt = 1;
    for (int qh = 0; qh < qt; ++qh) {
        const int4 f = s.fi[s.queue[qh]];
        const int v[3] = {f.x, f.y, f.z};
        for (int j = 0; j < 3; ++j) {
            const int u = v[j], x = v[(j + 1) % 3];
            for (int g = 0; g < nf; ++g) {
                const int4 gi = s.fi[g];
                if ((gi.x == x && gi.y == u) || (gi.y == x && gi.z == u) || (gi.z == x && gi.x == u)) {
                    if (gi.w != stamp) {
                        const float4 gn = s.fn[g];
                        if (dot(mk(gn.x, gn.y, gn.z), w - y_of(s, gi.x)) > vis_eps) {
                            s.fi[g].w = stamp;
                            s.queue[qt++] = g;
                        }
                    }
                    break;
                }
            }
        }
    }
    // horizon: the edges of visible faces not shared with another visible
    // face (epa.py:167-187, by vertex ids), then remove the visible faces
    int ne = 0;
    for (int q = 0; q < qt; ++q) {
        const int4 f = s.fi[s.queue[q]];
        const int v[3] = {f.x, f.y, f.z};
        for (int j = 0; j < 3; ++j) {
            const int e0 = v[j], e1 = v[(j + 1) % 3];
            bool found = false;
            for (int k = 0; k < ne; ++k) {
                const int2 e = s.edges[k];
                if (e.x == e1 && e.y == e0) {
                    s.edges[k] = s.edges[ne - 1];
                    --ne;
                    found = true;
                    break;
                }
            }
            if (!found) {
                if (ne >= o.max_loose_edges) return kEpaFallback;
                s.edges[ne++] = make_int2(e0, e1);
            }
        }
    }
    int m = 0;
    for (int i = 0; i < nf; ++i) {
        if (s.fi[i].w == stamp) continue;
        if (m != i) {
            s.fi[m] = s.fi[i];
            s.fn[m] = s.fn[i];
        }
        ++m;
    }
    // The visible faces must form a disk, i.e. the horizon one closed loop; an
    // invisible face enclosed by visible ones would break that, and such
    // pairs go to the FP64 EPA instead of growing a polytope with holes.
    if (ne < 3) return kEpaFallback;
    {
        int cur = s.edges[0].y, steps = 1;
        while (cur != s.edges[0].x && steps <= ne) {
            int next = -1;
            for (int k = 1; k < ne; ++k)
                if (s.edges[k].x == cur) {
                    next = s.edges[k].y;
                    break;
                }
            if (next < 0) return kEpaFallback;
            cur = next;
            ++steps;
        }
        if (steps != ne) return kEpaFallback;
    }
    // new faces (edge, w) (epa.py:126-146)
    for (int k = 0; k < ne; ++k) {
        if (m >= o.max_faces) {
            L.nf = m;
            return D3D_STATUS_EPA_FACE_OVERFLOW;
        }
        const int a = s.edges[k].x, b = s.edges[k].y;
        float4 pl;
        if (!face_plane(s, a, b, nv, pl)) return kEpaFallback;
        s.fi[m] = make_int4(a, b, nv, 0);
        s.fn[m] = pl;
        ++m;
    }
    L.nf = m;
    return -1;
}

}  // namespace d3d
