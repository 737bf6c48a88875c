"""Generate the golden fixtures in this folder from the distance3d reference.

Run from the repository root, in a container where the reference source tree
is available (it is NOT needed at test time):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/distance3d [mixed6 scb all9 mesh10 edge tree mesh_cached]

(no names: every fixture).
The reference is imported with its JIT disabled -- the mode its own CI uses --
through the inert stand-ins in ``_standins/`` (numba: ``njit`` returns the
function unchanged; pytransform3d: only names imported at module load).
NumPy 2 removed ``np.row_stack``; it is aliased to ``np.vstack`` for the
reference's libccd module, which is imported but not used here.

Inputs come from ``distance3d_gb300.workloads`` (seeded).  Outputs:

* ``gjk_mixed6.npz``  -- 1,000 six-type pairs, centers in [-w,w]^3 with w
  calibrated to ~30% intersecting pairs: reference ``gjk_distance_jolt``
  (dist, closest points, simplex, number of valid simplex rows, iterations)
  and ``gjk_intersection_jolt`` flags, plus every collider's ``aabb()``.
* ``gjk_scb.npz``     -- 1,000 Sphere/Capsule/Box pairs, centers in [-1,1]^3.
* ``epa_mixed6.npz``  -- reference ``epa.epa`` on the intersecting pairs of
  gjk_mixed6 whose four simplex rows were all written by GJK, at the default
  limits (64 faces; AssertionError -> face overflow) and at 256 faces / 128
  loose edges.
* ``gjk_all9.npz``    -- 1,000 pairs of the nine types (``pairs_all_types``: adds
  Disk, Ellipse and Cone, a quarter of the colliders wrapped in Margin), as
  gjk_mixed6, plus every collider's ``support_function`` along six
  directions (three random, +/- its local z axis, zero).
* ``epa_all9.npz``    -- reference ``epa.epa`` on the intersecting pairs of
  gjk_all9, as epa_mixed6.
* ``mpr_all9.npz``    -- reference ``mpr.mpr_penetration`` (flag, depth,
  direction, contact position; NaN for None) and ``mpr.mpr_intersection`` on
  every gjk_all9 pair, at the default tolerance and iteration limit.
* ``gjk_mesh10.npz``, ``epa_mesh10.npz``, ``mpr_mesh10.npz`` -- the same for
  1,000 pairs of the ten types (MeshGraph included).  The reference's
  MeshGraph support starts from its previous answer (the object caches it);
  here every support call restarts from the mesh's start vertex, the
  semantics of the GPU path, so that the fixture does not depend on the
  order of the calls.
* ``edge.npz``        -- degenerate and boundary colliders built one by one
  (zero radii and lengths, flat boxes, axis-aligned and tied disk normals, a
  zero normal, a zero-height cone, point / segment / coplanar hulls, a
  tetrahedron and a cube MeshGraph with tied vertices, margins of 0): their
  supports along axis, diagonal, tiny and zero directions, their AABBs, and
  GJK, EPA and MPR on every pair of the colliders whose supports are finite.
  Calls on which the reference raises its sanity assertion are recorded as
  such (status 2).
* ``gjk_mesh_cached.npz`` -- the stock reference MeshGraph with its vertex
  caching: 600 pairs over 21 shared colliders (axis-aligned and rotated
  cube MeshGraphs, whose tied vertices make the answer depend on the start
  vertex, random hull MeshGraphs, a MeshGraph in a Margin, spheres, boxes)
  run through the stock ``gjk_distance_jolt`` in a fixed order; per pair
  the two sides' caches (``first_idx``, -1 for no MeshGraph) before and
  after the call, and the outputs.  Also the triangles, for rebuilding the
  colliders.
* ``aabb_tree.npz``   -- a 400-collider scene: reference AabbTree self overlap
  (both orders, i == j dropped, reduced to i < j), brute force
  ``all_aabbs_overlap``, BoundingVolumeHierarchy.aabb_overlapping_with_self on
  the first 150 colliders, and AabbTree.overlaps_aabb for 20 query boxes.

Simplex rows that GJK never wrote are NaN here (the reference leaves
``np.empty`` memory there).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def import_reference(ref_root):
    sys.path[:0] = [os.path.join(HERE, "_standins"), ref_root, ROOT]
    np.row_stack = np.vstack
    import distance3d  # noqa: F401
    from distance3d import gjk, epa, colliders, aabb_tree, broad_phase
    return gjk, epa, colliders, aabb_tree, broad_phase


def import_mpr():
    from distance3d import mpr
    return mpr


def make_ref_colliders(colliders, cs):
    out = []
    for i in range(len(cs)):
        t = int(cs.types[i]) & 0xff
        pose = np.eye(4)
        pose[:3, :3] = cs.poses[i, :9].reshape(3, 3)
        pose[:3, 3] = cs.poses[i, 9:]
        p = cs.params[i]
        if t == 0:
            out.append(colliders.Sphere(pose[:3, 3].copy(), float(p[0])))
        elif t == 1:
            out.append(colliders.Capsule(pose, float(p[0]), float(p[1])))
        elif t == 2:
            out.append(colliders.Box(pose, p[:3].copy()))
        elif t == 3:
            out.append(colliders.Cylinder(pose, float(p[0]), float(p[1])))
        elif t == 4:
            out.append(colliders.Ellipsoid(pose, p[:3].copy()))
        elif t == 5:
            o, c = int(cs.hull_offset[i]), int(cs.hull_count[i])
            out.append(colliders.ConvexHullVertices(np.ascontiguousarray(cs.vertices[o:o + c, :3])))
        elif t == 6:
            out.append(colliders.Disk(pose[:3, 3].copy(), float(p[0]), pose[:3, 2].copy()))
        elif t == 7:
            out.append(colliders.Ellipse(pose[:3, 3].copy(), np.ascontiguousarray(pose[:3, :2].T), p[:2].copy()))
        elif t == 8:
            out.append(colliders.Cone(pose, float(p[0]), float(p[1])))
        else:
            out.append(fresh_mesh_graph(colliders, cs, i, pose))
        if int(cs.types[i]) & 0x100:
            out[-1] = colliders.Margin(out[-1], float(p[3]))
    return out


def fresh_mesh_graph(colliders, cs, i, pose):
    """The reference's MeshGraph for collider i, its triangles recomputed by
    scipy's ConvexHull as the workload made them (checked against the packed
    links), and its support restarted from the first vertex of the
    triangles in every call: the reference caches the last answer in the
    object (mesh.py:84), the GPU path starts every call afresh."""
    from scipy.spatial import ConvexHull
    from distance3d_gb300.collider_set import mesh_links
    o, c = int(cs.hull_offset[i]), int(cs.hull_count[i])
    v = np.ascontiguousarray(cs.vertices[o:o + c, :3])
    tri = ConvexHull(v).simplices
    blk = mesh_links(v, tri)
    b = int(cs.params[i, 0])
    assert np.array_equal(cs.links[b:b + len(blk)], blk) and cs.params[i, 1] == np.min(tri)
    m = colliders.MeshGraph(pose, v, tri)
    start = np.min(tri)

    def support_function(d, m=m, start=start):
        m._support_function.first_idx = start
        return m._support_function(d)[1]
    m.support_function = support_function
    return m


def support_fixture(cols, cs, seed=11):
    """Every collider's support_function along three random directions,
    +/- its local z axis and the zero vector."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = len(cols)
    dirs = np.zeros((n, 6, 3))
    dirs[:, :3] = rng.standard_normal((n, 3, 3))
    z = cs.poses[:, [2, 5, 8]]
    dirs[:, 3] = z
    dirs[:, 4] = -z
    out = np.empty_like(dirs)
    for i, c in enumerate(cols):
        for k in range(6):
            out[i, k] = c.support_function(dirs[i, k].copy())
    return dict(support_dirs=dirs, supports=out)


def ref_distance(gjk_mod, c1, c2, tolerance=1e-10, max_distance_squared=100000.0):
    """The outer loop of gjk_distance_jolt (_gjk_jolt.py:189-221) around the
    reference's own _distance_loop, exposing n_points and the iteration count."""
    J = sys.modules["distance3d.gjk._gjk_jolt"]
    Y = np.full((4, 3), np.nan)
    P = np.full((4, 3), np.nan)
    Q = np.full((4, 3), np.nan)
    n_points = 0
    tol2 = tolerance * tolerance
    d = np.array([1.0, 0.0, 0.0])
    v_len_sq = np.dot(d, d)
    prev = J.MAX_FLOAT
    it = 0
    while True:
        it += 1
        p = c1.support_function(d)
        q = c2.support_function(-d)
        state, n_new, prev, v_len_sq = J._distance_loop(
            p, q, Y, P, Q, n_points, tol2, prev, v_len_sq, d, max_distance_squared)
        if state == J.GjkState.Unknown:
            n_points = n_new
            continue
        if state == J.GjkState.Clipped:
            return J.MAX_FLOAT, None, None, Y, -1, it
        n_points = n_new
        a, b = J.calculate_closest_points(Y, P, Q, n_points)
        dist = np.sqrt(v_len_sq)
        if dist < J.EPSILON:
            a = b = 0.5 * (a + b)
        return float(dist), a, b, Y, n_points, it


GJK_SETTINGS = (("clip", dict(max_distance_squared=0.01)), ("coarse", dict(tolerance=1e-3)))


def gjk_fixture(mods, cs, i1, i2):
    gjk, epa, colliders, _, _ = mods
    cols = make_ref_colliders(colliders, cs)
    n = len(i1)
    dist = np.empty(n)
    cp1 = np.full((n, 3), np.nan)
    cp2 = np.full((n, 3), np.nan)
    simplex = np.full((n, 4, 3), np.nan)
    n_simplex = np.empty(n, np.int8)
    iters = np.empty(n, np.int32)
    hit = np.empty(n, bool)
    t0 = time.time()
    for k in range(n):
        c1, c2 = cols[i1[k]], cols[i2[k]]
        d, a, b, Y, m, it = ref_distance(gjk, c1, c2)
        d0, a0, b0, Y0 = gjk.gjk_distance_jolt(c1, c2)
        assert d == d0
        if a is not None:
            assert np.array_equal(a, a0) and np.array_equal(b, b0)
            assert np.array_equal(Y[:m], Y0[:m])
            cp1[k], cp2[k] = a, b
        dist[k] = d
        simplex[k] = Y
        n_simplex[k] = m
        iters[k] = it
        hit[k] = gjk.gjk_intersection_jolt(c1, c2)
    dt = time.time() - t0
    aabbs = np.stack([c.aabb() for c in cols])
    print(f"  gjk: {n} pairs in {dt:.1f}s ({n / dt:.0f} pairs/s incl. intersection)")
    # other options: a clipping distance some pairs exceed (_gjk_jolt.py:209-210
    # returns MAX_FLOAT and no points), and a coarse tolerance
    extra = {}
    for tag, kw in GJK_SETTINGS:
        dk = np.full(n, np.nan)
        ck = np.full((n, 3), np.nan)
        sk = np.zeros(n, np.int8)  # 0 ok, 1 clipped, 2 the sanity assertion (_gjk_jolt.py:216)
        for k in range(n):
            try:
                d, a, _, _ = gjk.gjk_distance_jolt(cols[i1[k]], cols[i2[k]], **kw)
            except AssertionError:
                sk[k] = 2
                continue
            dk[k] = d
            if a is None:
                sk[k] = 1
            else:
                ck[k] = a
        extra[f"dist_{tag}"] = dk
        extra[f"cp1_{tag}"] = ck
        extra[f"status_{tag}"] = sk
        print(f"  gjk[{tag}]: status counts {np.bincount(sk, minlength=3)}")
    return dict(types=cs.types, poses=cs.poses, params=cs.params, hull_offset=cs.hull_offset,
                hull_count=cs.hull_count, vertices=cs.vertices[:, :3].copy(), links=cs.links, i1=i1, i2=i2, **extra,
                dist=dist, cp1=cp1, cp2=cp2, simplex=simplex, n_simplex=n_simplex,
                iterations=iters, intersect=hit, aabbs=aabbs), cols


# EPA limit settings of the fixtures: the reference's defaults, the bench's
# polytope, limits under which the face buffer (tight), the iteration bound
# (short) and the loose-edge list (edges) run out on some pairs, and a coarser
# epsilon (convergence, visibility and edge matching)
EPA_SETTINGS = (("default", {}), ("large", dict(max_faces=256, max_loose_edges=128)),
                ("tight", dict(max_iter=20, max_faces=24, max_loose_edges=6)),
                ("short", dict(max_iter=6, max_faces=256, max_loose_edges=128)),
                ("edges", dict(max_faces=256, max_loose_edges=4)),
                ("eps", dict(max_faces=256, max_loose_edges=128, epsilon=1e-4)))


def epa_fixture(mods, cols, gf):
    _, epa, _, _, _ = mods
    sel = np.flatnonzero((gf["dist"] == 0.0) & ~np.isnan(gf["simplex"]).any(axis=(1, 2)))
    n = len(sel)
    out = {"pair": sel.astype(np.int32)}
    for tag, kw in EPA_SETTINGS:
        mtv = np.full((n, 3), np.nan)
        status = np.zeros(n, np.int8)   # 0 converged, 4 max_iter, 5 face overflow, 6 other error
        nfaces = np.zeros(n, np.int32)
        t0 = time.time()
        for k, p in enumerate(sel):
            c1, c2 = cols[gf["i1"][p]], cols[gf["i2"][p]]
            try:
                m, faces, ok = epa.epa(gf["simplex"][p].copy(), c1, c2, **kw)
                mtv[k] = m
                nfaces[k] = len(faces)
                status[k] = 0 if ok else 4
            except AssertionError:
                status[k] = 5
            except Exception:  # noqa: BLE001 - recorded as a distinct outcome
                status[k] = 6
        dt = time.time() - t0
        print(f"  epa[{tag}]: {n} pairs in {dt:.1f}s; status counts {np.bincount(status, minlength=7)}")
        out[f"mtv_{tag}"] = mtv
        out[f"status_{tag}"] = status
        out[f"n_faces_{tag}"] = nfaces
    return out


def mpr_fixture(cols, gf):
    mpr = import_mpr()
    n = len(gf["i1"])
    hit = np.zeros(n, bool)
    hit_i = np.zeros(n, bool)
    depth = np.full(n, np.nan)
    pdir = np.full((n, 3), np.nan)
    pos = np.full((n, 3), np.nan)
    t0 = time.time()
    for k in range(n):
        c1, c2 = cols[gf["i1"][k]], cols[gf["i2"][k]]
        h, d, p, c = mpr.mpr_penetration(c1, c2)
        hit[k] = h
        if d is not None:
            depth[k], pdir[k], pos[k] = d, p, c
        hit_i[k] = mpr.mpr_intersection(c1, c2)
    print(f"  mpr: {n} pairs in {time.time() - t0:.1f}s, {hit.sum()} intersecting")
    out = dict(i1=gf["i1"], i2=gf["i2"], hit=hit, depth=depth, dir=pdir, pos=pos, hit_intersection=hit_i)
    # other options: a coarse tolerance, and an iteration bound that the
    # portal discovery and refinement run into
    for tag, kw in MPR_SETTINGS:
        h2 = np.zeros(n, bool)
        d2 = np.full(n, np.nan)
        for k in range(n):
            h, d, _, _ = mpr.mpr_penetration(cols[gf["i1"][k]], cols[gf["i2"][k]], **kw)
            h2[k] = h
            if d is not None:
                d2[k] = d
        out[f"hit_{tag}"] = h2
        out[f"depth_{tag}"] = d2
        print(f"  mpr[{tag}]: {h2.sum()} intersecting")
    return out


MPR_SETTINGS = (("coarse", dict(mpr_tolerance=1e-2)), ("short", dict(max_iterations=3)))


class _FakeTM:
    def __init__(self):
        self.T = {}

    def add_transform(self, a, b, A2B):
        self.T[(a, b)] = A2B

    def get_transform(self, a, b):
        return self.T[(a, b)]


def tree_fixture(mods, cs, n_bvh=150, n_queries=20, seed=7):
    _, _, colliders, aabb_tree, broad_phase = mods
    cols = make_ref_colliders(colliders, cs)
    aabbs = np.stack([c.aabb() for c in cols])
    tree = aabb_tree.AabbTree()
    tree.insert_aabbs(aabbs)
    _, _, _, pairs = tree.overlaps_aabb_tree(tree)
    tp = {(min(a, b), max(a, b)) for a, b in pairs if a != b}
    tree_pairs = np.array(sorted(tp), dtype=np.int32).reshape(-1, 2)
    _, _, brute = aabb_tree.all_aabbs_overlap(aabbs, aabbs)
    bp = {(a, b) for a, b in brute if a < b}
    assert bp == tp, "reference tree and brute force disagree"
    # incremental BVH (broad_phase.py:129-142, 229-252)
    bvh = broad_phase.BoundingVolumeHierarchy(_FakeTM(), "base")
    for i in range(n_bvh):
        bvh.add_collider(i, cols[i])
    dp = bvh.aabb_overlapping_with_self()
    bvh_pairs = np.array(sorted((a[0], b[0]) for a, b in dp), dtype=np.int32).reshape(-1, 2)
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = rng.uniform(-3.5, 3.0, size=(n_queries, 3))
    hi = lo + rng.uniform(0.05, 1.5, size=(n_queries, 3))
    queries = np.stack([lo, hi], axis=2)
    q_idx, q_ptr = [], [0]
    for q in queries:
        _, ov = tree.overlaps_aabb(q)
        q_idx.extend(sorted(int(x) for x in ov))
        q_ptr.append(len(q_idx))
    print(f"  tree: {len(tree_pairs)} pairs (i<j), bvh[{n_bvh}]: {len(bvh_pairs)} ordered pairs")
    return dict(types=cs.types, poses=cs.poses, params=cs.params, hull_offset=cs.hull_offset,
                hull_count=cs.hull_count, vertices=cs.vertices[:, :3].copy(), aabbs=aabbs,
                tree_pairs=tree_pairs, bvh_n=np.int32(n_bvh), bvh_pairs=bvh_pairs,
                queries=queries, query_idx=np.array(q_idx, np.int32), query_ptr=np.array(q_ptr, np.int64))


def make_mixed6(mods, workloads):
    print("mixed six-type pairs (calibrated ~30% intersecting)")
    cs, i1, i2 = workloads.pairs_mixed_six(1000, seed=1234, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    gf, cols = gjk_fixture(mods, cs, i1, i2)
    print(f"  intersecting fraction {np.mean(gf['dist'] == 0.0):.3f}")
    np.savez_compressed(os.path.join(HERE, "gjk_mixed6.npz"), **gf)
    np.savez_compressed(os.path.join(HERE, "epa_mixed6.npz"), **epa_fixture(mods, cols, gf))


def make_scb(mods, workloads):
    print("sphere/capsule/box pairs")
    cs, i1, i2 = workloads.pairs_sphere_capsule_box(1000, seed=99)
    gf, _ = gjk_fixture(mods, cs, i1, i2)
    print(f"  intersecting fraction {np.mean(gf['dist'] == 0.0):.3f}")
    np.savez_compressed(os.path.join(HERE, "gjk_scb.npz"), **gf)


def make_all9(mods, workloads):
    print("nine-type pairs with margins")
    cs, i1, i2 = workloads.pairs_all_types(1000, seed=2024)
    gf, cols = gjk_fixture(mods, cs, i1, i2)
    gf.update(support_fixture(cols, cs))
    print(f"  intersecting fraction {np.mean(gf['dist'] == 0.0):.3f}")
    np.savez_compressed(os.path.join(HERE, "gjk_all9.npz"), **gf)
    np.savez_compressed(os.path.join(HERE, "epa_all9.npz"), **epa_fixture(mods, cols, gf))
    np.savez_compressed(os.path.join(HERE, "mpr_all9.npz"), **mpr_fixture(cols, gf))


def make_mesh(mods, workloads):
    print("ten-type pairs (MeshGraph included) with margins")
    cs, i1, i2 = workloads.pairs_all_types(1000, seed=2025, types=workloads.ALL_TYPES_MESH)
    gf, cols = gjk_fixture(mods, cs, i1, i2)
    gf.update(support_fixture(cols, cs))
    print(f"  intersecting fraction {np.mean(gf['dist'] == 0.0):.3f}")
    np.savez_compressed(os.path.join(HERE, "gjk_mesh10.npz"), **gf)
    np.savez_compressed(os.path.join(HERE, "epa_mesh10.npz"), **epa_fixture(mods, cols, gf))
    np.savez_compressed(os.path.join(HERE, "mpr_mesh10.npz"), **mpr_fixture(cols, gf))


def edge_colliders(colliders):
    """(reference collider objects, mask of those with finite supports)."""
    def pose(t=(0.0, 0.0, 0.0), axis=None, angle=0.0):
        m = np.eye(4)
        if axis is not None:
            a = np.asarray(axis, dtype=float) / np.linalg.norm(axis)
            K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
            m[:3, :3] = np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K
        m[:3, 3] = t
        return m
    C = colliders
    cube_v = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)])
    cube_t = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1],
                       [2, 3, 7], [2, 7, 6], [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]])
    tet_v = np.array([[0.0, 0.0, 0.0], [0.4, 0.0, 0.0], [0.0, 0.4, 0.0], [0.0, 0.0, 0.4]])
    tet_t = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]])
    finite = []
    out = []

    def add(c, ok=True):
        out.append(c)
        finite.append(ok)
    add(C.Sphere(np.zeros(3), 0.0))
    add(C.Sphere(np.array([0.2, -0.1, 0.3]), 0.5))
    add(C.Capsule(pose((0.1, 0.0, 0.0)), 0.2, 0.0))
    add(C.Capsule(pose((0.0, 0.3, 0.0), (1, 0, 0), 0.7), 0.0, 0.6))
    add(C.Cylinder(pose((0.0, 0.0, 0.2)), 0.0, 0.5))
    add(C.Cylinder(pose((-0.2, 0.0, 0.0), (0, 1, 0), 1.1), 0.3, 0.0))
    add(C.Box(pose((0.0, 0.1, 0.0)), np.array([0.6, 0.0, 0.4])))
    add(C.Box(pose((0.3, 0.3, 0.3), (1, 1, 1), 0.5), np.array([0.2, 0.2, 0.2])))
    add(C.Ellipsoid(pose((0.0, -0.2, 0.1), (0, 0, 1), 0.3), np.array([0.3, 0.0, 0.2])))
    for n in ((0, 0, 1), (1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, -1), (-1, 0, 0), (1, -1, 1)):
        nn = np.asarray(n, dtype=float)
        add(C.Disk(np.array([0.05, 0.1, -0.05]), 0.35, nn / np.linalg.norm(nn)))
    add(C.Disk(np.zeros(3), 0.0, np.array([0.0, 0.0, 1.0])))
    add(C.Disk(np.zeros(3), 0.3, np.zeros(3)), ok=False)
    add(C.Ellipse(np.array([0.1, 0.0, 0.0]), np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]), np.array([0.3, 0.0])))
    add(C.Ellipse(np.zeros(3), np.array([[0.6, 0.8, 0.0], [0.0, 0.0, 1.0]]), np.array([0.25, 0.4])))
    add(C.Cone(pose((0.0, 0.0, -0.3)), 0.0, 0.5))
    add(C.Cone(pose((0.1, 0.1, 0.0), (1, 0, 0), 3.0), 0.3, 0.0))
    add(C.Cone(pose((0.0, 0.0, 0.0), (0, 1, 1), 0.4), 0.25, 0.6))
    add(C.ConvexHullVertices(np.array([[0.1, 0.2, 0.3]])))
    add(C.ConvexHullVertices(np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])))
    add(C.ConvexHullVertices(np.array([[0.0, 0.0, 0.1], [0.4, 0.0, 0.1], [0.0, 0.4, 0.1], [0.4, 0.4, 0.1]])))
    add(C.MeshGraph(pose((0.0, 0.0, 0.0)), tet_v, tet_t))
    add(C.MeshGraph(pose((0.1, -0.1, 0.2), (0, 0, 1), 0.25), cube_v * 0.6, cube_t))
    add(C.Margin(C.Sphere(np.zeros(3), 0.2), 0.0))
    add(C.Margin(C.Box(pose(), np.array([0.3, 0.3, 0.3])), 0.2))
    add(C.Margin(C.ConvexHullVertices(np.array([[0.0, 0.0, 0.0]])), 0.5))
    add(C.Margin(C.Disk(np.zeros(3), 0.3, np.array([0.0, 1.0, 0.0])), 0.1))
    add(C.Margin(C.MeshGraph(pose((0.0, 0.2, 0.0)), tet_v, tet_t), 0.05))
    add(C.Margin(C.Cone(pose(), 0.2, 0.4), 0.0))
    for c in out:  # MeshGraph supports restart from the start vertex in every call
        inner = c.collider if type(c).__name__ == "Margin" else c
        if type(inner).__name__ == "MeshGraph":
            m, start = inner, np.min(inner.triangles)

            def support_function(d, m=m, start=start):
                m._support_function.first_idx = start
                return m._support_function(d)[1]
            m.support_function = support_function
    return out, np.array(finite)


def make_edge(mods, workloads):
    import signal
    from distance3d_gb300.collider_set import ColliderSet
    gjk, epa, colliders, _, _ = mods
    mpr = import_mpr()
    cols, finite = edge_colliders(colliders)
    cs = ColliderSet.from_colliders(cols)
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 1],
                     [-1, 1, 0], [0.3, -0.4, 1.2], [1e-300, 0, 0], [0, 0, 0], [2.5, 1.0, -0.5],
                     [0, 1, 1], [1, 1, 0]], dtype=float)
    supports = np.array([[c.support_function(d.copy()) for d in dirs] for c in cols])
    aabbs = np.stack([c.aabb() for c in cols])
    ok = np.flatnonzero(finite)
    i1, i2 = np.triu_indices(len(ok), k=1)
    i1, i2 = ok[i1].astype(np.int32), ok[i2].astype(np.int32)

    def timeout(signum, frame):
        raise TimeoutError()
    signal.signal(signal.SIGALRM, timeout)
    n = len(i1)
    keep = np.ones(n, bool)
    sanity = np.zeros(n, bool)
    dist = np.full(n, np.nan)
    cp1 = np.full((n, 3), np.nan)
    cp2 = np.full((n, 3), np.nan)
    simplex = np.full((n, 4, 3), np.nan)
    n_simplex = np.zeros(n, np.int8)
    iters = np.zeros(n, np.int32)
    hit = np.zeros(n, bool)
    mhit = np.zeros(n, bool)
    mhit_i = np.zeros(n, bool)
    mdepth = np.full(n, np.nan)
    mdir = np.full((n, 3), np.nan)
    mpos = np.full((n, 3), np.nan)
    for k in range(n):
        c1, c2 = cols[i1[k]], cols[i2[k]]
        signal.alarm(5)
        try:
            d, a, b, Y, m, it = ref_distance(gjk, c1, c2)
            try:
                gjk.gjk_distance_jolt(c1, c2)
            except AssertionError:
                sanity[k] = True
            dist[k], simplex[k], n_simplex[k], iters[k] = d, Y, m, it
            if a is not None:
                cp1[k], cp2[k] = a, b
            hit[k] = gjk.gjk_intersection_jolt(c1, c2)
            h, dd, p, c = mpr.mpr_penetration(c1, c2)
            mhit[k] = h
            if dd is not None:
                mdepth[k], mdir[k], mpos[k] = dd, p, c
            mhit_i[k] = mpr.mpr_intersection(c1, c2)
        except TimeoutError:
            keep[k] = False
        finally:
            signal.alarm(0)
    print(f"  edge: {len(cols)} colliders, {n} pairs, {np.sum(~keep)} dropped (reference did not return in 5 s), "
          f"{sanity.sum()} sanity assertions, {hit.sum()} intersecting")
    i1, i2 = i1[keep], i2[keep]
    gf = dict(types=cs.types, poses=cs.poses, params=cs.params, hull_offset=cs.hull_offset,
              hull_count=cs.hull_count, vertices=cs.vertices[:, :3].copy(), links=cs.links, i1=i1, i2=i2,
              dist=dist[keep], cp1=cp1[keep], cp2=cp2[keep], simplex=simplex[keep], n_simplex=n_simplex[keep],
              iterations=iters[keep], intersect=hit[keep], sanity=sanity[keep], aabbs=aabbs,
              support_dirs=dirs, supports=supports, finite=finite,
              mpr_hit=mhit[keep], mpr_depth=mdepth[keep], mpr_dir=mdir[keep], mpr_pos=mpos[keep],
              mpr_hit_intersection=mhit_i[keep])
    ef = epa_fixture(mods, cols, gf)
    gf.update({"epa_" + key: v for key, v in ef.items()})
    np.savez_compressed(os.path.join(HERE, "edge.npz"), **gf)


def mesh_cached_colliders(colliders, seed=77):
    """Stock reference colliders for the vertex-cache fixture: axis-aligned
    cube MeshGraphs (GJK's first search direction, +x, and many later ones
    tie four cube vertices within 10 EPSILON, so the vertex a climb returns
    depends on where it starts), rotated cubes, random hull MeshGraphs, a
    MeshGraph in a Margin, and spheres and boxes as partners.  Returns the
    objects and each one's triangles (None for other types)."""
    from scipy.spatial import ConvexHull
    C = colliders
    rng = np.random.Generator(np.random.PCG64(seed))
    cube_v = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)])
    cube_t = ConvexHull(cube_v).simplices

    def pose(rotate=False):
        m = np.eye(4)
        if rotate:
            q = rng.standard_normal(4)
            q /= np.linalg.norm(q)
            w, x, y, z = q
            m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
        m[:3, 3] = np.round(rng.uniform(-0.6, 0.6, 3), 2)
        return m
    cols, tris = [], []
    for k in range(8):
        s = np.round(rng.uniform(0.3, 0.7), 2)
        cols.append(C.MeshGraph(pose(rotate=k >= 6), cube_v * s, cube_t))
        tris.append(cube_t)
    for k in range(6):
        u = rng.standard_normal((int(rng.integers(8, 40)), 3))
        v = u / np.linalg.norm(u, axis=1, keepdims=True) * rng.uniform(0.15, 0.4)
        t = ConvexHull(v).simplices
        cols.append(C.MeshGraph(pose(rotate=True), v, t))
        tris.append(t)
    cols.append(C.Margin(C.MeshGraph(pose(), cube_v * 0.4, cube_t), 0.05))
    tris.append(cube_t)
    for k in range(3):
        cols.append(C.Sphere(np.round(rng.uniform(-0.6, 0.6, 3), 2), float(np.round(rng.uniform(0.1, 0.4), 2))))
        tris.append(None)
        cols.append(C.Box(pose(), np.round(rng.uniform(0.2, 0.8, 3), 2)))
        tris.append(None)
    return cols, tris


def make_mesh_cached(mods, workloads, n=600, seed=78):
    """The stock reference MeshGraph's vertex caching (mesh.py:30, 82-85):
    every collider object is shared by all the pairs that name it, and the
    pairs run through the stock gjk_distance_jolt one after another in this
    fixed order, so each climb starts where the object's previous climb
    stopped.  Records per pair the caches of both sides before and after the
    call (-1 for colliders without one) and the outputs."""
    from distance3d_gb300.collider_set import ColliderSet
    gjk, _, colliders, _, _ = mods
    print("MeshGraph vertex cache (stock objects, fixed call order)")
    cols, tris = mesh_cached_colliders(colliders)
    cs = ColliderSet.from_colliders(cols)
    rng = np.random.Generator(np.random.PCG64(seed))
    i1 = rng.integers(0, len(cols), n).astype(np.int32)
    i2 = ((i1 + rng.integers(1, len(cols), n)) % len(cols)).astype(np.int32)

    def holder(c):
        inner = c.collider if type(c).__name__ == "Margin" else c
        return inner._support_function if type(inner).__name__ == "MeshGraph" else None

    def caches(c1, c2):
        return [int(h.first_idx) if h is not None else -1 for h in (holder(c1), holder(c2))]
    before = np.empty((n, 2), np.int32)
    after = np.empty((n, 2), np.int32)
    dist = np.empty(n)
    cp1 = np.full((n, 3), np.nan)
    cp2 = np.full((n, 3), np.nan)
    simplex = np.full((n, 4, 3), np.nan)
    n_simplex = np.empty(n, np.int8)
    iters = np.empty(n, np.int32)
    sanity = np.zeros(n, bool)
    for k in range(n):
        c1, c2 = cols[i1[k]], cols[i2[k]]
        before[k] = caches(c1, c2)
        d, a, b, Y, m, it = ref_distance(gjk, c1, c2)
        after[k] = caches(c1, c2)
        # the stock call from the same caches: same outputs, same caches after
        for h, v in zip((holder(c1), holder(c2)), before[k]):
            if h is not None:
                h.first_idx = int(v)
        try:
            d0, a0, b0, Y0 = gjk.gjk_distance_jolt(c1, c2)
            assert d == d0
            if a is not None:
                assert np.array_equal(a, a0) and np.array_equal(b, b0) and np.array_equal(Y[:m], Y0[:m])
        except AssertionError:
            sanity[k] = True  # the reference's sanity check (_gjk_jolt.py:215-216) or a mismatch
        assert caches(c1, c2) == list(after[k])
        dist[k], simplex[k], n_simplex[k], iters[k] = d, Y, m, it
        if a is not None:
            cp1[k], cp2[k] = a, b
    moved = np.sum(np.any(before != after, axis=1))
    print(f"  {n} pairs over {len(cols)} colliders: {moved} calls moved a cache, {sanity.sum()} sanity assertions, "
          f"{np.sum(dist == 0.0)} intersecting")
    assert not sanity.any()
    tri_ptr = np.zeros(len(cols) + 1, np.int64)
    for j, t in enumerate(tris):
        tri_ptr[j + 1] = tri_ptr[j] + (0 if t is None else len(t))
    tri_all = np.concatenate([t for t in tris if t is not None]).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "gjk_mesh_cached.npz"), types=cs.types, poses=cs.poses, params=cs.params,
                        hull_offset=cs.hull_offset, hull_count=cs.hull_count, vertices=cs.vertices[:, :3].copy(),
                        links=cs.links, triangles=tri_all, triangle_ptr=tri_ptr, i1=i1, i2=i2,
                        cache_before=before, cache_after=after, dist=dist, cp1=cp1, cp2=cp2, simplex=simplex,
                        n_simplex=n_simplex, iterations=iters)


def make_tree(mods, workloads):
    print("aabb tree scene")
    scene = workloads.scene_mixed_six(400, seed=4321, half_width=3.0)
    np.savez_compressed(os.path.join(HERE, "aabb_tree.npz"), **tree_fixture(mods, scene))


FIXTURES = {"mixed6": make_mixed6, "scb": make_scb, "all9": make_all9, "mesh10": make_mesh, "edge": make_edge,
            "tree": make_tree, "mesh_cached": make_mesh_cached}


def main(ref_root, names):
    mods = import_reference(ref_root)
    from distance3d_gb300 import workloads
    for name in names or FIXTURES:
        FIXTURES[name](mods, workloads)


if __name__ == "__main__":
    if len(sys.argv) < 2 or any(a not in FIXTURES for a in sys.argv[2:]):
        sys.exit(__doc__)
    main(sys.argv[1], sys.argv[2:])
