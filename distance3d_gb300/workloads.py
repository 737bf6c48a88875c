"""Seeded synthetic workloads for the benchmark configurations.

All inputs come from ``numpy.random.Generator(PCG64(seed))``; nothing is read
from disk.  Rotations are quaternions drawn from a normalised 4-D Gaussian.

* ``pairs_sphere_capsule_box``: plain GJK distance workload, types uniform
  over {Sphere, Capsule, Box}, centers U[-1,1]^3, sphere/capsule radius
  U[0.05,0.3], capsule height U[0.1,0.5], box half-extents U[0.05,0.3] per
  axis (the box collider takes full edge lengths, so size = 2 * half).
* ``pairs_mixed_six``: batched mixed-type workload, types uniform over the six
  supported colliders.  Hulls are N points on the unit sphere (every point is
  a hull vertex), N = floor(exp(U[ln 8, ln 256])), scaled by U[0.05,0.3].
  Cylinder radius U[0.05,0.3] and length U[0.1,0.5], ellipsoid radii
  U[0.05,0.3] per axis (the same ranges as the capsule, since the workload
  names no other).  ``center_half_width`` sets the center box
  [-w, w]^3: w = 1 as literally specified gives ~3% intersecting pairs;
  ``INTERSECT30_HALF_WIDTH`` is calibrated to ~30% intersecting pairs.
* ``scene_mixed_six``: broad-phase scene, the same type/size distributions
  placed uniformly in [-20,20]^3.
* ``pairs_all_types``: the nine collider types, disk radius U[0.05,0.3],
  ellipse radii U[0.05,0.3] per axis, cone radius U[0.05,0.3] and height
  U[0.1,0.5] (the capsule's ranges), and a fraction of the colliders wrapped
  in Margin with margin U[0.01,0.05].  With ``types=ALL_TYPES_MESH`` also
  MeshGraphs: N points on the unit sphere in the mesh frame,
  N = floor(exp(U[ln 8, ln 64])), scaled by U[0.05,0.3], triangulated by
  their convex hull (scipy), posed by the collider's rotation and center.
"""
import numpy as np

from .collider_set import (ColliderSet, SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL, DISK, ELLIPSE, CONE,
                           MESH, MARGIN, mesh_links)

ALL_TYPES = (SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL, DISK, ELLIPSE, CONE)
ALL_TYPES_MESH = ALL_TYPES + (MESH,)

# center half-width for which ~30% of mixed six-type pairs intersect
# (calibrated with the oracle on 200k pairs, seed 0; see tests/test_workloads.py)
INTERSECT30_HALF_WIDTH = 0.38


def random_rotations(rng, n):
    """Rotation matrices (n,3,3) from normalised 4-D Gaussian quaternions."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def random_colliders(rng, n, type_choices, center_half_width=1.0, hull_n_range=(8, 256), margin_fraction=0.0):
    """n colliders with types drawn uniformly from ``type_choices``; with
    ``margin_fraction`` > 0 that fraction is wrapped in Margin (the draws for
    it come last, so the colliders themselves do not depend on it)."""
    types = rng.choice(np.asarray(type_choices, dtype=np.int32), size=n).astype(np.int32)
    R = random_rotations(rng, n)
    t = rng.uniform(-center_half_width, center_half_width, size=(n, 3))
    params = np.zeros((n, 4))
    u = rng.uniform(0.05, 0.3, size=(n, 3))
    h = rng.uniform(0.1, 0.5, size=n)
    m = types == SPHERE
    params[m, 0] = u[m, 0]
    m = types == CAPSULE
    params[m, 0] = u[m, 0]
    params[m, 1] = h[m]
    m = types == BOX
    params[m, :3] = 2.0 * u[m]
    m = types == CYLINDER
    params[m, 0] = u[m, 0]
    params[m, 1] = h[m]
    m = types == ELLIPSOID
    params[m, :3] = u[m]
    m = types == DISK
    params[m, 0] = u[m, 0]
    m = types == ELLIPSE
    params[m, :2] = u[m, :2]
    m = types == CONE
    params[m, 0] = u[m, 0]
    params[m, 1] = h[m]
    hulls = np.flatnonzero(types == HULL)
    counts = np.zeros(n, np.int32)
    offsets = np.full(n, -1, np.int64)
    lo, hi = hull_n_range
    nh = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), size=len(hulls)))).astype(np.int64)
    nh = np.clip(nh, lo, hi)
    counts[hulls] = nh
    starts = np.concatenate([[0], np.cumsum(nh)[:-1]]).astype(np.int64)
    offsets[hulls] = starts
    total = int(nh.sum())
    pts = rng.standard_normal((total, 3))
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    owner = np.repeat(hulls, nh)
    pts *= u[owner, 0:1]
    pts += t[owner]
    verts = np.zeros((total, 4))
    verts[:, :3] = pts
    R[hulls] = np.eye(3)
    t[hulls] = 0.0
    R[types == SPHERE] = np.eye(3)
    links = np.zeros(0, np.int32)
    meshes = np.flatnonzero(types == MESH)
    if len(meshes):
        from scipy.spatial import ConvexHull
        nm = np.floor(np.exp(rng.uniform(np.log(8), np.log(64), size=len(meshes)))).astype(np.int64)
        blocks, mverts = [], []
        nl = 0
        for k, i in enumerate(meshes):
            p = rng.standard_normal((nm[k], 3))
            p /= np.linalg.norm(p, axis=1, keepdims=True)
            p *= u[i, 0]
            tri = ConvexHull(p).simplices
            blk = mesh_links(p, tri)
            offsets[i] = total + sum(len(m) for m in mverts)
            counts[i] = len(p)
            params[i, :2] = (nl, float(np.min(tri)))
            blocks.append(blk)
            nl += len(blk)
            mverts.append(p)
        links = np.concatenate(blocks)
        mv = np.zeros((sum(len(m) for m in mverts), 4))
        mv[:, :3] = np.concatenate(mverts)
        verts = np.concatenate([verts, mv])
    poses = np.concatenate([R.reshape(n, 9), t], axis=1)
    if margin_fraction > 0:
        wrap = rng.uniform(size=n) < margin_fraction
        params[wrap, 3] = rng.uniform(0.01, 0.05, size=int(wrap.sum()))
        types = types | np.where(wrap, MARGIN, 0).astype(np.int32)
    return ColliderSet(types, poses, params, offsets, counts, verts, links)


def pairs_sphere_capsule_box(n_pairs, seed=0):
    """(ColliderSet with 2*n_pairs colliders, i1, i2) for the plain GJK workload."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = random_colliders(rng, 2 * n_pairs, [SPHERE, CAPSULE, BOX], 1.0)
    idx = np.arange(n_pairs, dtype=np.int32)
    return cs, 2 * idx, 2 * idx + 1


def pairs_mixed_six(n_pairs, seed=0, center_half_width=1.0):
    """(ColliderSet with 2*n_pairs colliders, i1, i2) for the mixed six-type workload."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = random_colliders(rng, 2 * n_pairs, [SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL],
                          center_half_width)
    idx = np.arange(n_pairs, dtype=np.int32)
    return cs, 2 * idx, 2 * idx + 1


def pairs_all_types(n_pairs, seed=0, center_half_width=INTERSECT30_HALF_WIDTH, margin_fraction=0.25,
                    types=ALL_TYPES):
    """(ColliderSet with 2*n_pairs colliders, i1, i2): the nine types (ten
    with ``types=ALL_TYPES_MESH``), a fraction wrapped in Margin."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = random_colliders(rng, 2 * n_pairs, types, center_half_width, margin_fraction=margin_fraction)
    idx = np.arange(n_pairs, dtype=np.int32)
    return cs, 2 * idx, 2 * idx + 1


def scene_mixed_six(n_colliders, seed=0, half_width=20.0):
    """ColliderSet of n colliders in [-half_width, half_width]^3 for the broad phase."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return random_colliders(rng, n_colliders, [SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL],
                            half_width)
