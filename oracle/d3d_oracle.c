/*
 * d3d_oracle.c -- CPU restatement of distance3d's collision hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA kernels of
 * distance3d_gb300 are checked against; it is also the timed CPU baseline
 * ("port").  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it.  The product never links or calls it.
 *
 * Every function restates one function of the reference (distance3d 0.9.0);
 * the citations are path:line inside that project.  Arithmetic is IEEE
 * double, compiled with -ffp-contract=off so that no multiply-add is fused
 * unless written as fma().  The reference evaluates its small products through
 * NumPy, whose BLAS (OpenBLAS) rounds them as fused multiply-add chains in a
 * fixed order; the two orders it uses are restated as dot012 / dot102 below and
 * used exactly where the reference calls np.dot / .dot / np.linalg.norm.
 * Element-wise NumPy arithmetic, np.cross, np.sum and Python scalar
 * arithmetic are unfused and written as plain C expressions.  With this the
 * oracle reproduces the reference bit for bit on the golden vectors
 * (tests/golden/make_golden.py); see tests/test_oracle_golden.py.
 *
 * Collider record layout (shared with the product's host store):
 *   pose   : 12 doubles, R row-major (9) then t (3)
 *   types  : type code, or-ed with T_MARGIN for a Margin wrapper
 *   params : 4 doubles  (sphere r | capsule r,h | box size xyz (full edge
 *            lengths) | cylinder r,L | ellipsoid radii xyz | hull unused |
 *            disk r | ellipse radii (2) | cone r,h | mesh links offset,
 *            start vertex; params[3] the margin)
 *            A disk's normal is R column 2; an ellipse's axes are R columns
 *            0 and 1.
 *   hull vertices: (V,4) doubles, xyz + pad, world space.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define T_SPHERE 0
#define T_CAPSULE 1
#define T_BOX 2
#define T_CYLINDER 3
#define T_ELLIPSOID 4
#define T_HULL 5
#define T_DISK 6
#define T_ELLIPSE 7
#define T_CONE 8
#define T_MESH 9        /* MeshGraph: vertices in the mesh frame, links block */
#define T_MARGIN 0x100  /* flag: wrapped in Margin, margin = params[3] */

#define ST_OK 0
#define ST_CLIPPED 1
#define ST_SANITY 2
#define ST_MAX_ITER 3
#define ST_EPA_NOT_CONVERGED 4
#define ST_EPA_FACE_OVERFLOW 5
#define ST_EPA_DEGENERATE 6

/* utils.py:7-8 */
static const double EPS = DBL_EPSILON;
static const double MAXF = DBL_MAX;

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
/* np.dot(a, b) of two 3-vectors, np.linalg.norm(v)^2, and the (8,3)x(3,3)
 * and (3,3)x(3,3) products of geometry.py:157 / containment.py:147:
 * fma(a2,b2, fma(a1,b1, a0*b0)). */
static inline double dot012(double a0, double a1, double a2, double b0, double b1, double b2) {
    return fma(a2, b2, fma(a1, b1, a0 * b0));
}
/* matrix (>= 2 rows) times vector through BLAS gemv: the pose products of
 * utils.py:143 / geometry.py:198,245,281 and the hull support
 * vertices.dot(d) of colliders.py:132: fma(a2,b2, fma(a0,b0, a1*b1)). */
static inline double dot102(double a0, double a1, double a2, double b0, double b1, double b2) {
    return fma(a2, b2, fma(a0, b0, a1 * b1));
}
static inline double dot(v3 a, v3 b) { return dot012(a.x, a.y, a.z, b.x, b.y, b.z); }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

typedef struct {
    int type;
    int wrapped;   /* Margin wrapper */
    double margin;
    double R[9];
    double t[3];
    double p[3];
    const double* verts; /* (n,4) */
    int nverts;
    const int32_t* links; /* mesh: links block (shortcuts, offsets, neighbour lists) */
    int start;            /* mesh: start vertex of the hill climb */
    int* cache;           /* mesh: the support object's vertex cache (mesh.py:30, 85), or NULL
                             to start every climb at `start` */
    double box[8 * 4];   /* box vertices, geometry.py:138-157 */
} collider;

/* geometry.py:135,138-157: t + (BOX_COORDS * size) . R^T, BOX_COORDS in
 * itertools.product([-.5,.5], repeat=3) order (x slowest). */
static void box_vertices(const double* R, const double* t, const double* size, double* out) {
    for (int k = 0; k < 8; ++k) {
        double c0 = ((k >> 2) & 1) ? 0.5 : -0.5;
        double c1 = ((k >> 1) & 1) ? 0.5 : -0.5;
        double c2 = (k & 1) ? 0.5 : -0.5;
        double a0 = c0 * size[0], a1 = c1 * size[1], a2 = c2 * size[2];
        for (int i = 0; i < 3; ++i)
            out[k * 4 + i] = t[i] + dot012(a0, a1, a2, R[i * 3 + 0], R[i * 3 + 1], R[i * 3 + 2]);
        out[k * 4 + 3] = 0.0;
    }
}

/* utils.py:78-122 plane_basis_from_normal (unfused scalar arithmetic) */
static void plane_basis(const double* n, double* x, double* y) {
    if (fabs(n[0]) >= fabs(n[1])) {
        double len = sqrt(n[0] * n[0] + n[2] * n[2]);
        x[0] = -n[2] / len; x[1] = 0.0; x[2] = n[0] / len;
        y[0] = n[1] * x[2]; y[1] = n[2] * x[0] - n[0] * x[2]; y[2] = -n[1] * x[0];
    } else {
        double len = sqrt(n[1] * n[1] + n[2] * n[2]);
        x[0] = 0.0; x[1] = n[2] / len; x[2] = -n[1] / len;
        y[0] = n[1] * x[2] - n[2] * x[1]; y[1] = -n[0] * x[2]; y[2] = n[0] * x[1];
    }
}

static void load_collider(collider* c, int idx, const int32_t* types, const double* poses,
                          const double* params, const int64_t* hull_offset,
                          const int32_t* hull_count, const double* vertices, const int32_t* links) {
    c->type = types[idx] & ~T_MARGIN;
    c->wrapped = (types[idx] & T_MARGIN) != 0;
    c->margin = params[(int64_t)idx * 4 + 3];
    memcpy(c->R, poses + (int64_t)idx * 12, 9 * sizeof(double));
    memcpy(c->t, poses + (int64_t)idx * 12 + 9, 3 * sizeof(double));
    memcpy(c->p, params + (int64_t)idx * 4, 3 * sizeof(double));
    if (c->type == T_DISK) {
        /* R = column_stack(x, y, normal), geometry.py:375-376 */
        double n[3] = {c->R[2], c->R[5], c->R[8]}, x[3], y[3];
        plane_basis(n, x, y);
        for (int i = 0; i < 3; ++i) { c->R[i * 3] = x[i]; c->R[i * 3 + 1] = y[i]; }
    }
    c->verts = NULL;
    c->nverts = 0;
    if (c->type == T_BOX) {
        box_vertices(c->R, c->t, c->p, c->box);
        c->verts = c->box;
        c->nverts = 8;
    } else if (c->type == T_HULL || c->type == T_MESH) {
        c->verts = vertices + hull_offset[idx] * 4;
        c->nverts = hull_count[idx];
    }
    c->links = NULL;
    c->start = 0;
    c->cache = NULL;
    if (c->type == T_MESH) {
        c->links = links + (int64_t)c->p[0];
        c->start = (int)c->p[1];
    }
}

/* R^T d, as np.dot(pose[:3, :3].T, d) (geometry.py:198,245,281) */
static inline v3 rt_mul(const double* R, v3 d) {
    return mk(dot102(R[0], R[3], R[6], d.x, d.y, d.z),
              dot102(R[1], R[4], R[7], d.x, d.y, d.z),
              dot102(R[2], R[5], R[8], d.x, d.y, d.z));
}

/* utils.py:125-143 transform_point: t + R v */
static inline v3 xform(const double* R, const double* t, v3 v) {
    return mk(t[0] + dot102(R[0], R[1], R[2], v.x, v.y, v.z),
              t[1] + dot102(R[3], R[4], R[5], v.x, v.y, v.z),
              t[2] + dot102(R[6], R[7], R[8], v.x, v.y, v.z));
}

/* Support functions: colliders.py:131-132 (hull/box argmax, first max),
 * geometry.py:314-346 sphere, :209-256 capsule, :160-206 cylinder,
 * :259-284 ellipsoid, :353-387 disk, :390-418 ellipse, :421-455 cone. */
static v3 base_support(const collider* c, v3 d) {
    switch (c->type) {
    case T_SPHERE: {
        double n = sqrt(dot(d, d));
        v3 ctr = mk(c->t[0], c->t[1], c->t[2]);
        if (n == 0.0) return add(ctr, mk(0.0, 0.0, c->p[0]));
        return add(ctr, mk(d.x / n * c->p[0], d.y / n * c->p[0], d.z / n * c->p[0]));
    }
    case T_CAPSULE: {
        double r = c->p[0], h = c->p[1];
        v3 l = rt_mul(c->R, d);
        double s = sqrt(l.x * l.x + l.y * l.y + l.z * l.z);
        v3 v;
        if (s == 0.0) v = mk(r, 0.0, 0.0);
        else { double f = r / s; v = mk(l.x * f, l.y * f, l.z * f); }
        if (l.z > 0.0) v.z += 0.5 * h; else v.z -= 0.5 * h;
        return xform(c->R, c->t, v);
    }
    case T_CYLINDER: {
        double r = c->p[0], L = c->p[1];
        v3 l = rt_mul(c->R, d);
        double s = sqrt(l.x * l.x + l.y * l.y);
        double z = (l.z < 0.0) ? -0.5 * L : 0.5 * L;
        v3 v;
        if (s == 0.0) v = mk(r, 0.0, z);
        else { double f = r / s; v = mk(l.x * f, l.y * f, z); }
        return xform(c->R, c->t, v);
    }
    case T_ELLIPSOID: {
        v3 l = rt_mul(c->R, d);
        v3 a = mk(l.x * c->p[0], l.y * c->p[1], l.z * c->p[2]);
        double n = sqrt(dot(a, a));
        if (n != 0.0) a = mk(a.x / n, a.y / n, a.z / n);  /* utils.py:26-30 */
        a = mk(a.x * c->p[0], a.y * c->p[1], a.z * c->p[2]);
        return xform(c->R, c->t, a);
    }
    case T_DISK: {
        const double* R = c->R;
        /* point = np.dot(R.T, d), R from np.column_stack: ddot over columns */
        double p0 = dot012(R[0], R[3], R[6], d.x, d.y, d.z);
        double p1 = dot012(R[1], R[4], R[7], d.x, d.y, d.z);
        double p2 = 0.0;  /* point[2] = 0.0 */
        double n = sqrt(dot012(p0, p1, p2, p0, p1, p2));
        if (n == 0.0) return mk(c->t[0], c->t[1], c->t[2]);
        double f = c->p[0] / n;
        p0 *= f; p1 *= f; p2 *= f;
        /* center + np.dot(R, point), R C-contiguous: gemv */
        return mk(c->t[0] + dot102(R[0], R[1], R[2], p0, p1, p2),
                  c->t[1] + dot102(R[3], R[4], R[5], p0, p1, p2),
                  c->t[2] + dot102(R[6], R[7], R[8], p0, p1, p2));
    }
    case T_ELLIPSE: {
        const double* R = c->R;
        /* local_dir = axes.dot(d): gemv over the axis rows (R columns 0, 1) */
        double l0 = dot102(R[0], R[3], R[6], d.x, d.y, d.z);
        double l1 = dot102(R[1], R[4], R[7], d.x, d.y, d.z);
        double v0 = c->p[0] * l0, v1 = c->p[1] * l1;
        double n = sqrt(fma(v1, v1, v0 * v0));  /* np.linalg.norm of 2 values */
        if (n != 0.0) { v0 = v0 / n; v1 = v1 / n; }
        v0 = v0 * c->p[0]; v1 = v1 * c->p[1];
        /* center + np.dot(local_vertex, axes) */
        return mk(c->t[0] + fma(v1, R[1], v0 * R[0]),
                  c->t[1] + fma(v1, R[4], v0 * R[3]),
                  c->t[2] + fma(v1, R[7], v0 * R[6]));
    }
    case T_CONE: {
        double r = c->p[0], h = c->p[1];
        v3 l = rt_mul(c->R, d);
        v3 q = mk(l.x, l.y, 0.0);
        double n = sqrt(dot(q, q));
        if (n == 0.0) q = mk(0.0, 0.0, 0.0);
        else q = scl(q, r / n);
        if (!(dot(l, q) >= l.z * h)) q = mk(0.0, 0.0, h);
        return xform(c->R, c->t, q);
    }
    case T_MESH: {
        /* mesh.py:77-85, 88-127: direction into the mesh frame, hill climb
         * from the cached vertex (mesh.py:82-85; without a cache each call
         * starts at the start vertex), posed vertex */
        v3 l = rt_mul(c->R, d);
        const int32_t* blk = c->links;
        const double eps = 10.0 * EPS;  /* PROJECTION_LENGTH_EPSILON */
        int best = (c->cache && *c->cache >= 0 && *c->cache < c->nverts) ? *c->cache : c->start;
        for (int k = 0; k < 6; ++k) {
            int cand = blk[k];
            const double* a = c->verts + (int64_t)cand * 4;
            const double* b = c->verts + (int64_t)best * 4;
            if (dot(l, mk(a[0] - b[0], a[1] - b[1], a[2] - b[2])) > eps) best = cand;
        }
        int converged = 0;
        while (!converged) {
            converged = 1;
            int lo = blk[6 + best], hi = blk[7 + best];
            for (int e = lo; e < hi; ++e) {
                int cand = blk[e];
                const double* a = c->verts + (int64_t)cand * 4;
                const double* b = c->verts + (int64_t)best * 4;
                if (dot(l, mk(a[0] - b[0], a[1] - b[1], a[2] - b[2])) > eps) { best = cand; converged = 0; }
            }
        }
        if (c->cache) *c->cache = best;  /* vertex caching, mesh.py:85 */
        const double* v = c->verts + (int64_t)best * 4;
        return xform(c->R, c->t, mk(v[0], v[1], v[2]));
    }
    default: { /* box and hull */
        int best = 0;
        double bd = 0.0;
        for (int k = 0; k < c->nverts; ++k) {
            const double* v = c->verts + (int64_t)k * 4;
            /* a one-row matrix goes through ddot instead of gemv */
            double s = c->nverts == 1 ? dot012(v[0], v[1], v[2], d.x, d.y, d.z)
                                      : dot102(v[0], v[1], v[2], d.x, d.y, d.z);
            if (k == 0 || s > bd) { bd = s; best = k; }  /* np.argmax: first max */
        }
        const double* v = c->verts + (int64_t)best * 4;
        return mk(v[0], v[1], v[2]);
    }
    }
}

/* colliders.py:629-631 Margin: s + margin * norm_vector(d) (utils.py:12-30) */
static v3 support(const collider* c, v3 d) {
    v3 s = base_support(c, d);
    if (!c->wrapped) return s;
    double n = sqrt(dot(d, d));
    v3 u = n == 0.0 ? d : mk(d.x / n, d.y / n, d.z / n);
    return mk(s.x + c->margin * u.x, s.y + c->margin * u.y, s.z + c->margin * u.z);
}

/* ---------------- Jolt GJK sub-algorithms: gjk/_gjk_jolt.py --------------- */

/* :292-312 */
static void bary_line(v3 a, v3 b, double* u, double* v) {
    v3 ab = sub(b, a);
    double den = dot(ab, ab);
    if (den < EPS * EPS) {
        if (dot(a, a) < dot(b, b)) { *u = 1.0; *v = 0.0; }
        else { *u = 0.0; *v = 1.0; }
    } else {
        *v = -dot(a, ab) / den;
        *u = 1.0 - *v;
    }
}

/* :316-372 */
static void bary_plane(v3 a, v3 b, v3 c, double* u, double* v, double* w) {
    v3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(c, b);
    double d00 = dot(v0, v0), d11 = dot(v1, v1), d22 = dot(v2, v2);
    if (d00 <= d22) {
        double d01 = dot(v0, v1);
        double den = d00 * d11 - d01 * d01;
        if (fabs(den) < EPS) {
            if (d00 > d11) { bary_line(a, b, u, v); *w = 0.0; }
            else { bary_line(a, c, u, w); *v = 0.0; }
        } else {
            double a0 = dot(a, v0), a1 = dot(a, v1);
            *v = (d01 * a1 - d11 * a0) / den;
            *w = (d01 * a0 - d00 * a1) / den;
            *u = 1.0 - *v - *w;
        }
    } else {
        double d12 = dot(v1, v2);
        double den = d11 * d22 - d12 * d12;
        if (fabs(den) < EPS) {
            if (d11 > d22) { bary_line(a, c, u, w); *v = 0.0; }
            else { bary_line(b, c, v, w); *u = 0.0; }
        } else {
            double c1 = dot(c, v1), c2 = dot(c, v2);
            *u = (d22 * c1 - d12 * c2) / den;
            *v = (d11 * c2 - d12 * c1) / den;
            *w = 1.0 - *u - *v;
        }
    }
}

/* utils.py:33-73 scalar_triple_product a.(b x c) */
static inline double stp(v3 a, v3 b, v3 c) { return dot(a, cross(b, c)); }

/* :376-390 */
static void bary_tetra(v3 a, v3 b, v3 c, v3 d, double* o) {
    v3 vab = sub(b, a), vac = sub(c, a), vad = sub(d, a);
    double va6 = -stp(b, sub(d, b), sub(c, b));
    double vb6 = -stp(a, vac, vad);
    double vc6 = -stp(a, vad, vab);
    double vd6 = -stp(a, vab, vac);
    double v6 = 1.0 / stp(vab, vac, vad);
    o[0] = va6 * v6; o[1] = vb6 * v6; o[2] = vc6 * v6; o[3] = vd6 * v6;
}

/* :394-412 */
static v3 cp_line(v3 a, v3 b, int* set) {
    double u, v;
    bary_line(a, b, &u, &v);
    if (v <= 0.0) { *set = 1; return a; }
    if (u <= 0.0) { *set = 2; return b; }
    *set = 3;
    return add(scl(a, u), scl(b, v));
}

/* :416-523 */
static v3 cp_triangle(v3 a, v3 b, v3 c, int* set) {
    v3 ab = sub(b, a), ac = sub(c, a), bc = sub(c, b);
    v3 n = (dot(bc, bc) < dot(ac, ac)) ? cross(ab, bc) : cross(ab, ac);
    double nl = dot(n, n);
    if (nl < EPS * EPS) {
        int s, ns;
        v3 cp = cp_line(a, b, &s);
        double best = dot(cp, cp);
        v3 q = cp_line(a, c, &ns);
        double d2 = dot(q, q);
        if (d2 < best) { cp = q; best = d2; s = (ns & 1) + ((ns & 2) << 1); }
        q = cp_line(b, c, &ns);
        d2 = dot(q, q);
        if (d2 < best) { cp = q; s = ns << 1; }
        *set = s;
        return cp;
    }
    v3 ap = neg(a);
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) { *set = 1; return a; }
    v3 bp = neg(b);
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) { *set = 2; return b; }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && 0.0 <= d1 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        *set = 3;
        return add(a, scl(ab, v));
    }
    v3 cpp = neg(c);
    double d5 = dot(ab, cpp), d6 = dot(ac, cpp);
    if (d6 >= 0.0 && d5 <= d6) { *set = 4; return c; }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && 0.0 <= d2 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        *set = 5;
        return add(a, scl(ac, w));
    }
    double va = d3 * d6 - d5 * d4;
    double d43 = d4 - d3, d56 = d5 - d6;
    if (va <= 0.0 && 0.0 <= d43 && d56 >= 0.0) {
        double w = d43 / (d43 + d56);
        *set = 6;
        return add(b, scl(bc, w));
    }
    *set = 7;
    /* n * (a + b + c).dot(n) / (3.0 * n_len_sq), evaluated left to right */
    double s = dot(add(add(a, b), c), n);
    double den = 3.0 * nl;
    return mk(n.x * s / den, n.y * s / den, n.z * s / den);
}

/* :527-570 */
static void outside_planes(v3 a, v3 b, v3 c, v3 d, int* o) {
    v3 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a), bd = sub(d, b), bc = sub(c, b);
    v3 abac = cross(ab, ac), acad = cross(ac, ad), adab = cross(ad, ab), bdbc = cross(bd, bc);
    double sp[4] = {dot(a, abac), dot(a, acad), dot(a, adab), dot(b, bdbc)};
    double sd[4] = {dot(ad, abac), dot(ab, acad), dot(ac, adab), -dot(ab, bdbc)};
    int allpos = sd[0] > 0.0 && sd[1] > 0.0 && sd[2] > 0.0 && sd[3] > 0.0;
    int allneg = sd[0] < 0.0 && sd[1] < 0.0 && sd[2] < 0.0 && sd[3] < 0.0;
    for (int i = 0; i < 4; ++i) {
        if (allpos) o[i] = sp[i] >= -EPS;
        else if (allneg) o[i] = sp[i] <= EPS;
        else o[i] = 1;
    }
}

/* :574-631 */
static v3 cp_tetra(v3 a, v3 b, v3 c, v3 d, int* set) {
    int s = 15, ns;
    v3 cp = mk(0.0, 0.0, 0.0);
    double best = MAXF;
    int o[4];
    outside_planes(a, b, c, d, o);
    if (o[0]) { cp = cp_triangle(a, b, c, &s); best = dot(cp, cp); }
    if (o[1]) {
        v3 q = cp_triangle(a, c, d, &ns);
        double d2 = dot(q, q);
        if (d2 < best) { best = d2; cp = q; s = (ns & 1) + ((ns & 6) << 1); }
    }
    if (o[2]) {
        v3 q = cp_triangle(a, d, b, &ns);
        double d2 = dot(q, q);
        if (d2 < best) { best = d2; cp = q; s = (ns & 1) + ((ns & 2) << 2) + ((ns & 4) >> 1); }
    }
    if (o[3]) {
        v3 q = cp_triangle(b, d, c, &ns);
        double d2 = dot(q, q);
        if (d2 < best) { cp = q; s = ((ns & 1) << 1) + ((ns & 2) << 2) + (ns & 4); }
    }
    *set = s;
    return cp;
}

/* :691-711; returns 1 on success */
static int closest_to_origin(const v3* Y, int n, double prev, v3* v, double* vl, int* set) {
    v3 r;
    int s;
    if (n == 1) { s = 1; r = Y[0]; }
    else if (n == 2) r = cp_line(Y[0], Y[1], &s);
    else if (n == 3) r = cp_triangle(Y[0], Y[1], Y[2], &s);
    else r = cp_tetra(Y[0], Y[1], Y[2], Y[3], &s);
    double l = dot(r, r);
    if (l < prev) { *v = r; *vl = l; *set = s; return 1; }
    return 0;
}

/* :635-640 */
static double max_y_len_sq(const v3* Y, int n) {
    double m = dot(Y[0], Y[0]);
    for (int i = 1; i < n; ++i) { double l = dot(Y[i], Y[i]); if (l > m) m = l; }
    return m;
}

/* :655-664 (and :644-651 when P, Q are NULL) */
static int compact(v3* Y, v3* P, v3* Q, int n, int set) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        if (set & (1 << i)) {
            Y[m] = Y[i];
            if (P) { P[m] = P[i]; Q[m] = Q[i]; }
            ++m;
        }
    }
    return m;
}

/* :668-687 */
static void closest_points(const v3* Y, const v3* P, const v3* Q, int n, v3* a, v3* b) {
    if (n == 1) { *a = P[0]; *b = Q[0]; }
    else if (n == 2) {
        double u, v;
        bary_line(Y[0], Y[1], &u, &v);
        *a = add(scl(P[0], u), scl(P[1], v));
        *b = add(scl(Q[0], u), scl(Q[1], v));
    } else if (n == 3) {
        double u, v, w;
        bary_plane(Y[0], Y[1], Y[2], &u, &v, &w);
        *a = add(add(scl(P[0], u), scl(P[1], v)), scl(P[2], w));
        *b = add(add(scl(Q[0], u), scl(Q[1], v)), scl(Q[2], w));
    } else {
        double o[4];
        bary_tetra(Y[0], Y[1], Y[2], Y[3], o);
        *a = add(add(add(scl(P[0], o[0]), scl(P[1], o[1])), scl(P[2], o[2])), scl(P[3], o[3]));
        *b = add(add(add(scl(Q[0], o[0]), scl(Q[1], o[1])), scl(Q[2], o[2])), scl(Q[3], o[3]));
    }
}

typedef struct {
    double dist;
    v3 cp1, cp2;
    v3 Y[4];
    int n;
    int status;
    int iters;
} gjk_result;

/* :138-221 gjk_distance_jolt with :224-288 _distance_loop inlined.
 * max_iter bounds the loop (the reference has no bound); reaching it sets
 * ST_MAX_ITER. */
static void gjk_distance(const collider* c1, const collider* c2, double tol, double max_d2,
                         double sanity, int max_iter, gjk_result* out) {
    v3 Y[4], P[4], Q[4];
    memset(Y, 0, sizeof(Y)); memset(P, 0, sizeof(P)); memset(Q, 0, sizeof(Q));
    int n = 0;
    double tol2 = tol * tol;
    v3 dir = mk(1.0, 0.0, 0.0);
    double vl = dot(dir, dir);
    double prev = MAXF;
    int it = 0, state = -1;
    out->status = ST_OK;
    while (1) {
        if (it >= max_iter) { state = 0; out->status = ST_MAX_ITER; break; }
        ++it;
        v3 p = support(c1, dir);
        v3 q = support(c2, neg(dir));
        v3 w = sub(p, q);
        double dd = dot(dir, w);
        if (dd < 0.0 && dd * dd > vl * max_d2) { state = 3; break; }
        Y[n] = w; P[n] = p; Q[n] = q; ++n;
        v3 nv; double nl; int set;
        if (closest_to_origin(Y, n, prev, &nv, &nl, &set)) {
            dir = nv; vl = nl;
        } else {
            --n;
            set = 0;
            for (int i = 0; i < n; ++i) set |= 1 << i;
        }
        if (set == 15) { vl = 0.0; state = 1; break; }
        n = compact(Y, P, Q, n, set);
        if (vl <= tol2) { vl = 0.0; state = 1; break; }
        if (vl <= EPS * max_y_len_sq(Y, n)) { vl = 0.0; state = 1; break; }
        dir = neg(dir);
        if (prev - vl <= EPS * prev) { state = 0; break; }
        prev = vl;
    }
    out->iters = it;
    memcpy(out->Y, Y, sizeof(Y));
    out->n = n;
    if (state == 3) {
        out->status = ST_CLIPPED;
        out->dist = MAXF;
        out->cp1 = out->cp2 = mk(NAN, NAN, NAN);
        return;
    }
    v3 a, b;
    closest_points(Y, P, Q, n, &a, &b);
    double check = fabs(dot(dir, dir) - vl);
    if (!(check < sanity) && out->status == ST_OK) out->status = ST_SANITY;
    double dist = sqrt(vl);
    if (dist < EPS) { v3 m = scl(add(a, b), 0.5); a = b = m; }
    out->dist = dist;
    out->cp1 = a;
    out->cp2 = b;
}

/* :29-135 gjk_intersection_jolt.  Returns 1 on intersection; *status is
 * ST_MAX_ITER when the iteration bound was reached (result 0). */
static int gjk_intersection(const collider* c1, const collider* c2, double tol, int max_iter,
                            int* status, int* iters) {
    v3 Y[4];
    memset(Y, 0, sizeof(Y));
    int n = 0;
    double tol2 = tol * tol;
    double prev = MAXF;
    v3 dir = mk(1.0, 0.0, 0.0);
    *status = ST_OK;
    for (int it = 1; ; ++it) {
        if (it > max_iter) { *status = ST_MAX_ITER; *iters = it - 1; return 0; }
        *iters = it;
        v3 p = support(c1, dir);
        v3 q = support(c2, neg(dir));
        v3 w = sub(p, q);
        if (dot(dir, w) < -EPS) return 0;
        Y[n++] = w;
        v3 nv; double vl; int set;
        if (!closest_to_origin(Y, n, prev, &nv, &vl, &set)) return 0;
        dir = nv;
        if (set == 15) return 1;
        if (vl <= tol2) return 1;
        if (vl <= EPS * max_y_len_sq(Y, n)) return 1;
        dir = neg(dir);
        if (prev - vl <= EPS * prev) return 0;
        prev = vl;
        n = compact(Y, NULL, NULL, n, set);
    }
}

/* ------------------------------- EPA: epa.py ------------------------------ */

typedef struct { v3 v[3]; v3 n; } face;

/* utils.py:12-30 norm_vector */
static inline v3 norm_vec(v3 v) {
    double n = sqrt(dot(v, v));
    if (n == 0.0) return v;
    return mk(v.x / n, v.y / n, v.z / n);
}

/* epa.py:99-102 */
static inline void face_normal(face* f) {
    f->n = norm_vec(cross(sub(f->v[1], f->v[0]), sub(f->v[2], f->v[0])));
}

static inline double vlen(v3 v) { return sqrt(dot(v, v)); }

/* epa.py:9-78 with Polytope :81-146 and LooseEdges :149-202.
 * faces: scratch of max_faces faces; edges: scratch of 2*max_loose_edges v3.
 * Returns status; writes mtv and the final face count. */
static int epa(const v3* simplex, const collider* c1, const collider* c2, int max_iter,
               int max_edges, int max_faces, double eps, face* F, v3* E, v3* mtv, int* n_faces_out) {
    /* :89-97 */
    static const int init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    int nf = 4;
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 3; ++j) F[i].v[j] = simplex[init[i][j]];
        face_normal(&F[i]);
    }
    int closest = 0;
    for (int it = 0; it < max_iter; ++it) {
        /* :104-109 find_face_closest_to_origin (np.argmin: first min) */
        if (nf == 0) { *n_faces_out = 0; *mtv = mk(NAN, NAN, NAN); return ST_EPA_DEGENERATE; }
        double md = 0.0;
        closest = 0;
        for (int i = 0; i < nf; ++i) {
            double d = F[i].v[0].x * F[i].n.x + F[i].v[0].y * F[i].n.y + F[i].v[0].z * F[i].n.z;
            if (i == 0 || d < md) { md = d; closest = i; }
        }
        v3 sd = F[closest].n;
        v3 np_ = sub(support(c1, sd), support(c2, neg(sd)));
        double pd = dot(np_, sd);
        if (pd - md < eps) {  /* :67-70 */
            *mtv = scl(sd, pd);
            *n_faces_out = nf;
            return ST_OK;
        }
        /* :157-165 find_triangles_facing_point_and_store_loose_edges */
        int ne = 0;
        int i = 0;
        while (i < nf) {
            if (dot(F[i].n, sub(np_, F[i].v[0])) > eps) {  /* :122-124 */
                /* :167-187 */
                for (int j = 0; j < 3; ++j) {
                    v3 e0 = F[i].v[j], e1 = F[i].v[(j + 1) % 3];
                    int found = 0;
                    for (int k = 0; k < ne; ++k) {
                        if (vlen(sub(E[2 * k + 1], e0)) < eps && vlen(sub(E[2 * k], e1)) < eps) {
                            E[2 * k] = E[2 * (ne - 1)];
                            E[2 * k + 1] = E[2 * (ne - 1) + 1];
                            --ne;
                            found = 1;
                            break;
                        }
                    }
                    if (!found) {
                        if (ne >= max_edges) break;  /* :193-198 */
                        E[2 * ne] = e0; E[2 * ne + 1] = e1; ++ne;
                    }
                }
                F[i] = F[nf - 1];  /* :118-120 */
                --nf;
                --i;
            }
            ++i;
        }
        /* :126-137 extend_with_point */
        for (int k = 0; k < ne; ++k) {
            if (!(nf < max_faces)) { *n_faces_out = nf; *mtv = mk(NAN, NAN, NAN); return ST_EPA_FACE_OVERFLOW; }
            face* f = &F[nf];
            f->v[0] = E[2 * k]; f->v[1] = E[2 * k + 1]; f->v[2] = np_;
            face_normal(f);
            if (vlen(f->n) < 0.5) continue;
            /* :139-146 fix_ccw_normal_direction, bias 1e-6.  The reference
             * keeps `temp` as a NumPy view of row 0, so after
             * faces[i,0] = faces[i,1] the write-back faces[i,1] = temp
             * stores row 1 again: the net effect is v0 := v1, v1 unchanged,
             * normal negated.  Restated as observed. */
            if (dot(f->v[0], f->n) + 1e-6 < 0.0) {
                f->v[0] = f->v[1];
                f->n = neg(f->n);
            }
            ++nf;
        }
    }
    /* :77: closest_face is a view into the face array, read after the last
     * iteration's edits. */
    *mtv = scl(F[closest].n, dot(F[closest].v[0], F[closest].n));
    *n_faces_out = nf;
    return ST_EPA_NOT_CONVERGED;
}

/* ------------------------- MPR: mpr.py ----------------------------------- */

/* ConvexCollider.center (colliders.py): the pose translation, a hull's
 * vertex mean (np.mean(axis=0): rows summed in order, then divided), a
 * cone's mid-axis point :582-584; Margin passes through :633-634. */
static v3 collider_center(const collider* c) {
    if (c->type == T_HULL || c->type == T_MESH) {
        v3 s = mk(c->verts[0], c->verts[1], c->verts[2]);
        for (int k = 1; k < c->nverts; ++k)
            s = add(s, mk(c->verts[k * 4], c->verts[k * 4 + 1], c->verts[k * 4 + 2]));
        double n = (double)c->nverts;
        v3 m = mk(s.x / n, s.y / n, s.z / n);
        return c->type == T_MESH ? xform(c->R, c->t, m) : m;  /* colliders.py:224-226 */
    }
    v3 t = mk(c->t[0], c->t[1], c->t[2]);
    if (c->type == T_CONE) {
        double f = 0.5 * c->p[1];
        return add(t, mk(f * c->R[2], f * c->R[5], f * c->R[8]));
    }
    return t;
}

enum { PORTAL_CONTINUE = -2, PORTAL_OUTSIDE = -1, PORTAL_BUILT = 0, PORTAL_ON_V1 = 1, PORTAL_ON_SEGMENT = 2 };

/* portal rows: v (Minkowski difference), a (collider 1), b (collider 2) */
typedef struct { v3 v[4], a[4], b[4]; } portal;

static void portal_support(const collider* c1, const collider* c2, v3 d, portal* P, int i) {
    P->a[i] = support(c1, d);
    P->b[i] = support(c2, neg(d));
    P->v[i] = sub(P->a[i], P->b[i]);  /* minkowski.py:23-55 */
}

static void portal_copy(portal* P, int dst, int src) {
    P->v[dst] = P->v[src]; P->a[dst] = P->a[src]; P->b[dst] = P->b[src];
}

static inline int all_zero(v3 v) { return v.x == 0.0 && v.y == 0.0 && v.z == 0.0; }

/* :123-158 _discover_portal with :161-240 */
static int mpr_discover(const collider* c1, const collider* c2, int max_iter, portal* P) {
    /* :161-174 origin ray from the centers */
    P->a[0] = collider_center(c1);
    P->b[0] = collider_center(c2);
    P->v[0] = sub(P->a[0], P->b[0]);
    if (all_zero(P->v[0])) P->v[0].x += EPS * 10.0;
    /* :177-185 */
    v3 d = norm_vec(neg(P->v[0]));
    portal_support(c1, c2, d, P, 1);
    if (!all_zero(P->v[1]) && dot(P->v[1], d) < EPS) return PORTAL_OUTSIDE;
    /* :188-201 */
    d = cross(P->v[0], P->v[1]);
    if (dot(d, d) < EPS) return all_zero(P->v[1]) ? PORTAL_ON_V1 : PORTAL_ON_SEGMENT;
    d = norm_vec(d);
    portal_support(c1, c2, d, P, 2);
    if (dot(P->v[2], d) < EPS) return PORTAL_OUTSIDE;
    /* :204-210 */
    d = norm_vec(cross(sub(P->v[1], P->v[0]), sub(P->v[2], P->v[0])));
    if (dot(d, P->v[0]) > 0.0) {
        /* :232-240 _swap_vertices keeps row idx1 as a NumPy view, so after
         * row idx1 = row idx2 the "swap" writes row idx2 back onto itself:
         * both rows end up holding the old row 2 */
        portal_copy(P, 1, 2);
        d = scl(d, -1.0);
    }
    int n_points = 3, it = 0;
    while (n_points < 4) {
        portal_support(c1, c2, d, P, 3);
        if (dot(P->v[3], d) < EPS) return PORTAL_OUTSIDE;
        /* :213-229 _iterate_discover_portal */
        int cont = 0;
        if (dot(cross(P->v[1], P->v[3]), P->v[0]) < EPS) {
            portal_copy(P, 2, 3);
            cont = 1;
        }
        if (!cont && dot(cross(P->v[3], P->v[2]), P->v[0]) < EPS) {
            portal_copy(P, 1, 3);
            cont = 1;
        }
        if (cont) d = norm_vec(cross(sub(P->v[1], P->v[0]), sub(P->v[2], P->v[0])));
        else n_points = 4;
        if (++it >= max_iter) break;
    }
    return PORTAL_BUILT;
}

/* :276-281 */
static inline v3 portal_direction(const portal* P) {
    return norm_vec(cross(sub(P->v[2], P->v[1]), sub(P->v[3], P->v[1])));
}

/* :290-299: min over the three portal vertices of (v4 - v_i) . d, with
 * v[1:].dot(d) through gemv */
static int portal_reach_tolerance(const portal* P, v3 v4, v3 d, double tol) {
    double s4 = dot(v4, d);
    double m = 0.0;
    for (int i = 1; i < 4; ++i) {
        double e = s4 - dot102(P->v[i].x, P->v[i].y, P->v[i].z, d.x, d.y, d.z);
        if (i == 1 || e < m) m = e;
    }
    return m < tol + EPS;
}

/* :302-317 */
static void expand_portal(portal* P, v3 v4, v3 a4, v3 b4) {
    v3 c = cross(v4, P->v[0]);
    int idx;
    if (dot(P->v[1], c) > 0.0) idx = dot(P->v[2], c) > 0.0 ? 1 : 3;
    else idx = dot(P->v[3], c) > 0.0 ? 2 : 1;
    P->v[idx] = v4; P->a[idx] = a4; P->b[idx] = b4;
}

/* :243-273 _refine_portal.  The reference loops until it decides; here at
 * most `limit` expansions, then *status = ST_MAX_ITER. */
static int mpr_refine(const collider* c1, const collider* c2, portal* P, double tol, int limit, int* status) {
    for (int it = 0;; ++it) {
        v3 d = portal_direction(P);
        if (dot(P->v[1], d) > -10.0 * EPS) return 1;
        v3 a4 = support(c1, d), b4 = support(c2, neg(d)), v4 = sub(a4, b4);
        if (!(dot(v4, d) > -10.0 * EPS) || portal_reach_tolerance(P, v4, d, tol)) return 0;
        if (it >= limit) { *status = ST_MAX_ITER; return 0; }
        expand_portal(P, v4, a4, b4);
    }
}

/* distance/_triangle.py:12-89 point_to_triangle for the origin:
 * returns the distance, *cp the closest point */
static double origin_to_triangle(v3 A, v3 B, v3 C, v3* cp) {
    const v3 o = mk(0.0, 0.0, 0.0);
    v3 ab = sub(B, A), ac = sub(C, A);
    v3 ap = sub(o, A);
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) { *cp = A; return sqrt(dot(sub(o, A), sub(o, A))); }
    v3 bp = sub(o, B);
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { *cp = B; return sqrt(dot(sub(o, B), sub(o, B))); }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && 0.0 <= d1 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        *cp = add(A, scl(ab, v));
    } else {
        v3 cpt = sub(o, C);
        double d5 = dot(ab, cpt), d6 = dot(ac, cpt);
        if (d6 >= 0.0 && d5 <= d6) { *cp = C; return sqrt(dot(sub(o, C), sub(o, C))); }
        double vb = d5 * d2 - d1 * d6;
        if (vb <= 0.0 && 0.0 <= d2 && d6 <= 0.0) {
            double w = d2 / (d2 - d6);
            *cp = add(A, scl(ac, w));
        } else {
            double va = d3 * d6 - d5 * d4;
            if (va <= 0.0 && 0.0 <= d4 - d3 && d5 - d6 >= 0.0) {
                double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
                *cp = add(B, scl(sub(C, B), w));
            } else {
                double denom = 1.0 / ((va + vb) + vc);
                double v = vb * denom, w = vc * denom;
                *cp = add(add(A, scl(ab, v)), scl(ac, w));
            }
        }
    }
    v3 r = sub(o, *cp);
    return sqrt(dot(r, r));
}

/* :372-393 _contact_position: barycentric weights of the origin in the
 * portal (np.sum in order, b.dot(V) through gemv as
 * fma(b0,V0,b1*V1) + fma(b2,V2,b3*V3)) */
static v3 contact_position(const portal* P, v3 d) {
    const v3* v = P->v;
    double w[4];
    w[0] = dot(cross(v[1], v[2]), v[3]);
    w[1] = dot(cross(v[3], v[2]), v[0]);
    w[2] = dot(cross(v[0], v[1]), v[3]);
    w[3] = dot(cross(v[2], v[1]), v[0]);
    double sum = ((w[0] + w[1]) + w[2]) + w[3];
    if (sum < EPS) {
        w[0] = 0.0;
        w[1] = dot(cross(v[2], v[3]), d);
        w[2] = dot(cross(v[3], v[1]), d);
        w[3] = dot(cross(v[1], v[2]), d);
        sum = ((w[0] + w[1]) + w[2]) + w[3];
    }
    for (int i = 0; i < 4; ++i) w[i] = w[i] / sum;
    double p1[3], p2[3];
    for (int j = 0; j < 3; ++j) {
        const double* A0 = &P->a[0].x; const double* A1 = &P->a[1].x;
        const double* A2 = &P->a[2].x; const double* A3 = &P->a[3].x;
        const double* B0 = &P->b[0].x; const double* B1 = &P->b[1].x;
        const double* B2 = &P->b[2].x; const double* B3 = &P->b[3].x;
        p1[j] = fma(w[0], A0[j], w[1] * A1[j]) + fma(w[2], A2[j], w[3] * A3[j]);
        p2[j] = fma(w[0], B0[j], w[1] * B1[j]) + fma(w[2], B2[j], w[3] * B3[j]);
    }
    return mk(0.5 * (p1[0] + p2[0]), 0.5 * (p1[1] + p2[1]), 0.5 * (p1[2] + p2[2]));
}

typedef struct { int hit, status; double depth; v3 dir, pos; } mpr_result;

/* :21-110 mpr_intersection (penetration = 0) and mpr_penetration; depth,
 * dir and pos are NaN where the reference returns None. */
static void mpr(const collider* c1, const collider* c2, double tol, int max_iter, int limit, int penetration,
                mpr_result* r) {
    portal P;
    memset(&P, 0, sizeof(P));
    r->status = ST_OK;
    r->depth = NAN;
    r->dir = r->pos = mk(NAN, NAN, NAN);
    int res = mpr_discover(c1, c2, max_iter, &P);
    if (res == PORTAL_OUTSIDE) { r->hit = 0; return; }
    if (res == PORTAL_ON_V1 || res == PORTAL_ON_SEGMENT) {
        r->hit = 1;
        if (!penetration) return;
        r->pos = scl(add(P.a[1], P.b[1]), 0.5);  /* :337-352 */
        if (res == PORTAL_ON_V1) {
            r->depth = 0.0;
            r->dir = mk(0.0, 0.0, 0.0);
        } else {
            r->depth = sqrt(dot(P.v[1], P.v[1]));
            r->dir = norm_vec(P.v[1]);
        }
        return;
    }
    r->hit = mpr_refine(c1, c2, &P, tol, limit, &r->status);
    if (!r->hit || !penetration) return;
    /* :320-334 _find_penetration_info, :355-362 _penetration_info */
    for (int it = 0;; ++it) {
        v3 d = portal_direction(&P);
        v3 a4 = support(c1, d), b4 = support(c2, neg(d)), v4 = sub(a4, b4);
        if (portal_reach_tolerance(&P, v4, d, tol) || it > max_iter) {
            v3 cp;
            double depth = origin_to_triangle(P.v[1], P.v[2], P.v[3], &cp);
            if (fabs(depth) < EPS) cp = mk(0.0, 0.0, 0.0);
            r->depth = depth;
            r->pos = contact_position(&P, portal_direction(&P));
            r->dir = norm_vec(cp);
            return;
        }
        expand_portal(&P, v4, a4, b4);
    }
}

/* ---------------------- AABBs: containment.py ---------------------------- */

/* np.minimum / np.maximum: a NaN operand gives NaN */
static inline double np_min(double a, double b) { return (a != a || a < b) ? a : b; }
static inline double np_max(double a, double b) { return (a != a || a > b) ? a : b; }

static void base_aabb(const collider* c, double* o);

/* writes (3,2) [axis][min,max]; Margin colliders.py:639-643 */
static void collider_aabb(const collider* c, double* o) {
    base_aabb(c, o);
    if (c->wrapped)
        for (int i = 0; i < 3; ++i) { o[2 * i] = o[2 * i] - c->margin; o[2 * i + 1] = o[2 * i + 1] + c->margin; }
}

static void base_aabb(const collider* c, double* o) {
    const double* R = c->R;
    const double* t = c->t;
    switch (c->type) {
    case T_SPHERE:  /* :25-44 */
        for (int i = 0; i < 3; ++i) { o[2 * i] = t[i] - c->p[0]; o[2 * i + 1] = t[i] + c->p[0]; }
        return;
    case T_CAPSULE:  /* :99-122 */
        for (int i = 0; i < 3; ++i) {
            double e = 0.5 * c->p[1] * fabs(R[i * 3 + 2]) + c->p[0];
            o[2 * i] = t[i] - e; o[2 * i + 1] = t[i] + e;
        }
        return;
    case T_CYLINDER:  /* :70-96 */
        for (int i = 0; i < 3; ++i) {
            double a = R[i * 3 + 2];
            double e = 0.5 * c->p[1] * fabs(a) + c->p[0] * sqrt(1.0 - a * a);
            o[2 * i] = t[i] - e; o[2 * i + 1] = t[i] + e;
        }
        return;
    case T_ELLIPSOID: {  /* :125-148 */
        double E[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) E[i * 3 + j] = R[i * 3 + j] * c->p[j];
        for (int j = 0; j < 3; ++j) {
            double nn = sqrt(E[0 * 3 + j] * E[0 * 3 + j] + E[1 * 3 + j] * E[1 * 3 + j] + E[2 * 3 + j] * E[2 * 3 + j]);
            for (int i = 0; i < 3; ++i) E[i * 3 + j] = E[i * 3 + j] / nn;
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) E[i * 3 + j] = E[i * 3 + j] * c->p[j];
        for (int k = 0; k < 3; ++k) {
            double m = 0.0;
            for (int i = 0; i < 3; ++i) {
                double s = dot012(R[i * 3 + 0], R[i * 3 + 1], R[i * 3 + 2], E[k * 3 + 0], E[k * 3 + 1], E[k * 3 + 2]);
                if (i == 0 || s > m) m = s;
            }
            o[2 * k] = t[k] - m; o[2 * k + 1] = t[k] + m;
        }
        return;
    }
    case T_DISK:  /* :151-174 */
        for (int i = 0; i < 3; ++i) {
            double n = R[i * 3 + 2];
            double e = c->p[0] * sqrt(1.0 - n * n);
            o[2 * i] = t[i] - e; o[2 * i + 1] = t[i] + e;
        }
        return;
    case T_ELLIPSE:  /* :206-229 */
        for (int i = 0; i < 3; ++i) {
            double a = c->p[0] * R[i * 3], b = c->p[1] * R[i * 3 + 1];
            double e = sqrt(a * a + b * b);
            o[2 * i] = t[i] - e; o[2 * i + 1] = t[i] + e;
        }
        return;
    case T_MESH:  /* colliders.py:234-237: t + V R^T (dgemm: dot012 order), min / max */
        for (int i = 0; i < 3; ++i) {
            double lo = 0.0, hi = 0.0;
            for (int k = 0; k < c->nverts; ++k) {
                const double* v = c->verts + (int64_t)k * 4;
                double w = t[i] + dot012(v[0], v[1], v[2], R[i * 3], R[i * 3 + 1], R[i * 3 + 2]);
                if (k == 0 || w < lo) lo = w;
                if (k == 0 || w > hi) hi = w;
            }
            o[2 * i] = lo; o[2 * i + 1] = hi;
        }
        return;
    case T_CONE:  /* :177-203 */
        for (int i = 0; i < 3; ++i) {
            double pb = t[i] + c->p[1] * R[i * 3 + 2];
            double a = pb - t[i];
            double e = sqrt(1.0 - a * a / (c->p[1] * c->p[1]));
            o[2 * i] = np_min(t[i] - e * c->p[0], pb);
            o[2 * i + 1] = np_max(t[i] + e * c->p[0], pb);
        }
        return;
    default: {  /* box :47-67 and hull :6-22 (min/max of vertices) */
        for (int i = 0; i < 3; ++i) {
            double lo = c->verts[i], hi = c->verts[i];
            for (int k = 1; k < c->nverts; ++k) {
                double v = c->verts[(int64_t)k * 4 + i];
                if (v < lo) lo = v;
                if (v > hi) hi = v;
            }
            o[2 * i] = lo; o[2 * i + 1] = hi;
        }
        return;
    }
    }
}

/* ---------------------------- exported batch API -------------------------- */

#define SET_ARGS const int32_t* types, const double* poses, const double* params, \
    const int64_t* hull_offset, const int32_t* hull_count, const double* vertices, const int32_t* links
#define SET_PASS types, poses, params, hull_offset, hull_count, vertices, links

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_support(SET_ARGS, int idx, const double* d, double* out) {
    collider c;
    load_collider(&c, idx, SET_PASS);
    v3 r = support(&c, mk(d[0], d[1], d[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void orc_box_vertices(const double* pose, const double* size, double* out) {
    box_vertices(pose, pose + 9, size, out);
}

void orc_gjk_distance(SET_ARGS, const int32_t* i1, const int32_t* i2, int64_t n,
                      double tol, double max_d2, double sanity, int max_iter,
                      double* dist, double* cp1, double* cp2, double* simplex,
                      int8_t* n_simplex, int8_t* status, int32_t* iters, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < n; ++k) {
        collider a, b;
        load_collider(&a, i1[k], SET_PASS);
        load_collider(&b, i2[k], SET_PASS);
        gjk_result r;
        gjk_distance(&a, &b, tol, max_d2, sanity, max_iter, &r);
        dist[k] = r.dist;
        cp1[3 * k] = r.cp1.x; cp1[3 * k + 1] = r.cp1.y; cp1[3 * k + 2] = r.cp1.z;
        cp2[3 * k] = r.cp2.x; cp2[3 * k + 1] = r.cp2.y; cp2[3 * k + 2] = r.cp2.z;
        for (int j = 0; j < 4; ++j) {
            simplex[12 * k + 3 * j] = r.Y[j].x;
            simplex[12 * k + 3 * j + 1] = r.Y[j].y;
            simplex[12 * k + 3 * j + 2] = r.Y[j].z;
        }
        n_simplex[k] = (int8_t)r.n;
        status[k] = (int8_t)r.status;
        if (iters) iters[k] = r.iters;
    }
}

/* orc_gjk_distance with the MeshGraph vertex cache: pair k's mesh supports
 * start their climbs at cache[2k] (collider i1[k]) and cache[2k+1] (i2[k]),
 * -1 meaning the mesh's start vertex, and leave their last answer there --
 * one support object per pair side, as a reference MeshGraph object carries
 * its first_idx from call to call (mesh.py:30, 82-85). */
void orc_gjk_distance_cached(SET_ARGS, const int32_t* i1, const int32_t* i2, int64_t n,
                             double tol, double max_d2, double sanity, int max_iter, int32_t* cache,
                             double* dist, double* cp1, double* cp2, double* simplex,
                             int8_t* n_simplex, int8_t* status, int32_t* iters, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < n; ++k) {
        collider a, b;
        load_collider(&a, i1[k], SET_PASS);
        load_collider(&b, i2[k], SET_PASS);
        a.cache = cache + 2 * k;
        b.cache = cache + 2 * k + 1;
        gjk_result r;
        gjk_distance(&a, &b, tol, max_d2, sanity, max_iter, &r);
        dist[k] = r.dist;
        cp1[3 * k] = r.cp1.x; cp1[3 * k + 1] = r.cp1.y; cp1[3 * k + 2] = r.cp1.z;
        cp2[3 * k] = r.cp2.x; cp2[3 * k + 1] = r.cp2.y; cp2[3 * k + 2] = r.cp2.z;
        for (int j = 0; j < 4; ++j) {
            simplex[12 * k + 3 * j] = r.Y[j].x;
            simplex[12 * k + 3 * j + 1] = r.Y[j].y;
            simplex[12 * k + 3 * j + 2] = r.Y[j].z;
        }
        n_simplex[k] = (int8_t)r.n;
        status[k] = (int8_t)r.status;
        if (iters) iters[k] = r.iters;
    }
}

void orc_gjk_intersection(SET_ARGS, const int32_t* i1, const int32_t* i2, int64_t n,
                          double tol, int max_iter, int8_t* hit, int8_t* status,
                          int32_t* iters, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < n; ++k) {
        collider a, b;
        load_collider(&a, i1[k], SET_PASS);
        load_collider(&b, i2[k], SET_PASS);
        int st, it;
        hit[k] = (int8_t)gjk_intersection(&a, &b, tol, max_iter, &st, &it);
        status[k] = (int8_t)st;
        if (iters) iters[k] = it;
    }
}

/* EPA on given simplices (n,4,3).  faces_out (optional): (n,max_faces,4,3). */
void orc_epa(SET_ARGS, const int32_t* i1, const int32_t* i2, int64_t n, const double* simplices,
             int max_iter, int max_edges, int max_faces, double eps,
             double* mtv, int8_t* status, int32_t* n_faces, double* faces_out, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel
    {
        face* F = (face*)malloc(sizeof(face) * (size_t)(max_faces + 1));
        v3* E = (v3*)malloc(sizeof(v3) * 2 * (size_t)(max_edges + 1));
#pragma omp for schedule(dynamic, 16)
        for (int64_t k = 0; k < n; ++k) {
            collider a, b;
            load_collider(&a, i1[k], SET_PASS);
            load_collider(&b, i2[k], SET_PASS);
            v3 s[4];
            for (int j = 0; j < 4; ++j)
                s[j] = mk(simplices[12 * k + 3 * j], simplices[12 * k + 3 * j + 1], simplices[12 * k + 3 * j + 2]);
            v3 m;
            int nf;
            status[k] = (int8_t)epa(s, &a, &b, max_iter, max_edges, max_faces, eps, F, E, &m, &nf);
            mtv[3 * k] = m.x; mtv[3 * k + 1] = m.y; mtv[3 * k + 2] = m.z;
            n_faces[k] = nf;
            if (faces_out) {
                double* fo = faces_out + (int64_t)k * max_faces * 12;
                for (int f = 0; f < nf && f < max_faces; ++f) {
                    const v3* vv = F[f].v;
                    double row[12] = {vv[0].x, vv[0].y, vv[0].z, vv[1].x, vv[1].y, vv[1].z,
                                      vv[2].x, vv[2].y, vv[2].z, F[f].n.x, F[f].n.y, F[f].n.z};
                    memcpy(fo + f * 12, row, sizeof(row));
                }
            }
        }
        free(F);
        free(E);
    }
}

/* AABBs of all colliders, (n,3,2) */
void orc_aabbs(SET_ARGS, int64_t n, double* out, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        collider c;
        load_collider(&c, (int)k, SET_PASS);
        collider_aabb(&c, out + 6 * k);
    }
}

/* aabb_tree.py:504-527 closed-interval overlap */
static inline int aabb_overlap(const double* a, const double* b) {
    return a[0] <= b[1] && a[1] >= b[0] && a[2] <= b[3] && a[3] >= b[2] && a[4] <= b[5] && a[5] >= b[4];
}

/* aabb_tree.py:466-500 all_aabbs_overlap restricted to i<j over one set:
 * counts (out == NULL) or writes sorted (i,j) pairs, row-major by i then j. */
int64_t orc_self_pairs(const double* aabbs, int64_t n, int32_t* out, int64_t cap) {
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j)
            if (aabb_overlap(aabbs + 6 * i, aabbs + 6 * j)) {
                if (out && m < cap) { out[2 * m] = (int32_t)i; out[2 * m + 1] = (int32_t)j; }
                ++m;
            }
    return m;
}

/* all_aabbs_overlap between two sets (every (i,j), i in a, j in b) */
int64_t orc_cross_pairs(const double* a, int64_t na, const double* b, int64_t nb, int32_t* out, int64_t cap) {
    int64_t m = 0;
    for (int64_t i = 0; i < na; ++i)
        for (int64_t j = 0; j < nb; ++j)
            if (aabb_overlap(a + 6 * i, b + 6 * j)) {
                if (out && m < cap) { out[2 * m] = (int32_t)i; out[2 * m + 1] = (int32_t)j; }
                ++m;
            }
    return m;
}

/* Sort-and-sweep restatement of all_aabbs_overlap restricted to i < j
 * (aabb_tree.py:466-527): the same closed-interval pair set as the brute
 * force, in O(n log n + candidates).  Pairs come out unsorted; count is
 * returned, at most cap are written. */
typedef struct { double lo; int64_t i; } sweep_key;

static int sweep_cmp(const void* a, const void* b) {
    const sweep_key* x = (const sweep_key*)a;
    const sweep_key* y = (const sweep_key*)b;
    if (x->lo < y->lo) return -1;
    if (x->lo > y->lo) return 1;
    return (x->i > y->i) - (x->i < y->i);
}

int64_t orc_self_pairs_sweep(const double* aabbs, int64_t n, int32_t* out, int64_t cap) {
    sweep_key* k = (sweep_key*)malloc(sizeof(sweep_key) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) { k[i].lo = aabbs[6 * i]; k[i].i = i; }
    qsort(k, (size_t)n, sizeof(sweep_key), sweep_cmp);
    int64_t m = 0;
    for (int64_t a = 0; a < n; ++a) {
        const int64_t i = k[a].i;
        const double hx = aabbs[6 * i + 1];
        for (int64_t b = a + 1; b < n && k[b].lo <= hx; ++b) {
            const int64_t j = k[b].i;
            if (aabb_overlap(aabbs + 6 * i, aabbs + 6 * j)) {
                if (out && m < cap) {
                    out[2 * m] = (int32_t)(i < j ? i : j);
                    out[2 * m + 1] = (int32_t)(i < j ? j : i);
                }
                ++m;
            }
        }
    }
    free(k);
    return m;
}

/* Support points of colliders idx[k] along dirs[k] (FP64, the reference's
 * support functions), in parallel. */
void orc_support_batch(SET_ARGS, const int32_t* idx, const double* dirs, int64_t n, double* out, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        collider c;
        load_collider(&c, idx[k], SET_PASS);
        v3 r = support(&c, mk(dirs[3 * k], dirs[3 * k + 1], dirs[3 * k + 2]));
        out[3 * k] = r.x; out[3 * k + 1] = r.y; out[3 * k + 2] = r.z;
    }
}

/* MPR for pairs (i1[k], i2[k]): hit[k], depth[k], dir[k][3], pos[k][3],
 * status[k] (mpr.py:21-110) */
void orc_mpr(SET_ARGS, const int32_t* i1, const int32_t* i2, int64_t n, double tol, int max_iter, int limit,
             int penetration, int8_t* hit, double* depth, double* dir, double* pos, int8_t* status, int nthreads) {
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < n; ++k) {
        collider a, b;
        load_collider(&a, i1[k], SET_PASS);
        load_collider(&b, i2[k], SET_PASS);
        mpr_result r;
        mpr(&a, &b, tol, max_iter, limit, penetration, &r);
        hit[k] = (int8_t)r.hit;
        status[k] = (int8_t)r.status;
        depth[k] = r.depth;
        dir[3 * k] = r.dir.x; dir[3 * k + 1] = r.dir.y; dir[3 * k + 2] = r.dir.z;
        pos[3 * k] = r.pos.x; pos[3 * k + 1] = r.pos.y; pos[3 * k + 2] = r.pos.z;
    }
}
