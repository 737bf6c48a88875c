"""Host-side packed collider set: the flat format every C-ABI entry point and
the device store are built from.

One row per collider:

* ``types``       int32 (n,)     SPHERE=0 CAPSULE=1 BOX=2 CYLINDER=3 ELLIPSOID=4 HULL=5
                                 DISK=6 ELLIPSE=7 CONE=8 MESH=9 (MeshGraph), or-ed with
                                 MARGIN (0x100) for a collider wrapped in distance3d's
                                 Margin
* ``poses``       float64 (n,12) rotation R row-major (9 values) then translation t (3)
* ``params``      float64 (n,4)  sphere (r) | capsule (r, h) | box (size xyz, full edge
                                 lengths as in distance3d colliders.py:147-184) |
                                 cylinder (r, L) | ellipsoid (radii xyz) | hull (unused) |
                                 disk (r) | ellipse (radii, 2) | cone (r, height) |
                                 mesh (links offset, start vertex); params[3] is the
                                 margin of a Margin wrapper
* ``hull_offset`` int64 (n,)     first row of the collider in ``vertices`` (-1: none)
* ``hull_count``  int32 (n,)     number of hull vertices
* ``vertices``    float64 (V,4)  world-space hull vertices (mesh-frame vertices for a
                                 mesh), xyz plus a zero pad so a vertex is 32 B (FP64) /
                                 16 B (FP32) and loads as aligned 128-bit words
* ``links``       int32 (L,)     MeshGraph adjacency blocks (``mesh_links``)

A sphere keeps its center in ``t`` (its rotation is unused, distance3d
colliders.py:243-287); a ConvexHullVertices has the identity pose
(colliders.py:143-144).  A disk keeps its normal in R column 2 (columns 0 and
1 are derived from it on the device, utils.py:78-122); an ellipse keeps its
two axes in R columns 0 and 1 and their cross product in column 2
(colliders.py:546-551).  A Margin (colliders.py:606-647) wraps one collider
of any other type; Margin of a Margin is not representable.  A MeshGraph
keeps its pose (mesh2origin) and its vertices in the mesh frame; its links
block holds the hill climb's shortcut vertices and vertex neighbours in the
reference's order (mesh.py:26-52).  Boxes carry no
vertices here: the device store derives their 8 vertices from pose and size
(geometry.py:135-157).
"""
import numpy as np

SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL, DISK, ELLIPSE, CONE, MESH = range(10)
MARGIN = 0x100
TYPE_NAMES = ("Sphere", "Capsule", "Box", "Cylinder", "Ellipsoid", "ConvexHullVertices", "Disk", "Ellipse",
              "Cone", "MeshGraph")


def mesh_links(vertices, triangles):
    """The links block of a MeshGraph (see module docstring): shortcut
    vertices (argmax x, y, z, argmin x, y, z), nv + 1 neighbour-list offsets
    relative to the block, the neighbour lists.  The neighbour sets are built
    and iterated as mesh.py:26-52 builds and iterates them, so the hill climb
    visits neighbours in the reference's order."""
    v = np.asarray(vertices, dtype=np.float64).reshape(-1, 3)
    triangles = np.asarray(triangles)
    connections = {}
    for i, j, k in triangles:
        if i not in connections:
            connections[i] = set()
        if j not in connections:
            connections[j] = set()
        if k not in connections:
            connections[k] = set()
        connections[i].update((j, k))
        connections[j].update((i, k))
        connections[k].update((i, j))
    nv = len(v)
    shortcut = [np.argmax(v[:, 0]), np.argmax(v[:, 1]), np.argmax(v[:, 2]),
                np.argmin(v[:, 0]), np.argmin(v[:, 1]), np.argmin(v[:, 2])]
    lists = []
    offsets = np.zeros(nv + 1, dtype=np.int64)
    pos = 6 + nv + 1
    for idx in range(nv):
        offsets[idx] = pos
        if idx in connections:
            nb = np.fromiter(connections[idx], dtype=int, count=len(connections[idx]))
            lists.append(nb)
            pos += len(nb)
    offsets[nv] = pos
    out = np.concatenate([np.asarray(shortcut, dtype=np.int64), offsets] + lists).astype(np.int32)
    return out


class ColliderSet:
    """Packed host arrays for a batch of colliders (see module docstring)."""

    def __init__(self, types, poses, params, hull_offset, hull_count, vertices, links=None):
        self.types = np.ascontiguousarray(types, dtype=np.int32)
        n = len(self.types)
        self.poses = np.ascontiguousarray(poses, dtype=np.float64).reshape(n, 12)
        self.params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, 4)
        self.hull_offset = np.ascontiguousarray(hull_offset, dtype=np.int64)
        self.hull_count = np.ascontiguousarray(hull_count, dtype=np.int32)
        v = np.asarray(vertices, dtype=np.float64)
        if v.ndim == 2 and v.shape[1] == 3:
            v = np.concatenate([v, np.zeros((len(v), 1))], axis=1)
        self.vertices = np.ascontiguousarray(v.reshape(-1, 4))
        self.links = np.ascontiguousarray(np.zeros(0, np.int32) if links is None else links, dtype=np.int32)
        self.validate()

    def __len__(self):
        return len(self.types)

    @property
    def n_vertices(self):
        return len(self.vertices)

    @property
    def base_types(self):
        """Type codes without the Margin flag."""
        return self.types & ~MARGIN

    @property
    def wrapped(self):
        """True where the collider is wrapped in Margin."""
        return (self.types & MARGIN) != 0

    def validate(self):
        n = len(self.types)
        for name in ("poses", "params", "hull_offset", "hull_count"):
            if len(getattr(self, name)) != n:
                raise ValueError(f"ColliderSet.{name} has {len(getattr(self, name))} rows, expected {n}")
        base = self.base_types
        if n and (base.min() < 0 or base.max() > MESH):
            raise ValueError("ColliderSet.types holds an unknown collider type")
        hulls = (base == HULL) | (base == MESH)
        if np.any(self.hull_count[hulls] < 1):
            raise ValueError("ConvexHullVertices needs at least one vertex")
        if np.any(self.hull_offset[hulls] < 0) or np.any(
                self.hull_offset[hulls] + self.hull_count[hulls] > len(self.vertices)):
            raise ValueError("hull vertex range outside the vertex pool")
        if len(self.vertices) + 8 * int(np.count_nonzero(base == BOX)) >= 2 ** 31:
            raise ValueError("vertex pool larger than 2^31 rows")
        for i in np.flatnonzero(base == MESH):
            nv, off = int(self.hull_count[i]), int(self.params[i, 0])
            if off != self.params[i, 0] or off < 0 or off + 7 + nv > len(self.links):
                raise ValueError("MeshGraph links block outside the links array")
            blk = self.links[off:]
            lo, hi = int(blk[6]), int(blk[6 + nv])
            if (np.any(blk[:6] < 0) or np.any(blk[:6] >= nv) or lo != 7 + nv or hi < lo
                    or off + hi > len(self.links) or np.any(np.diff(blk[6:7 + nv]) < 0)
                    or np.any(blk[lo:hi] < 0) or np.any(blk[lo:hi] >= nv)):
                raise ValueError("MeshGraph links block is inconsistent")
            start = self.params[i, 1]
            if start != int(start) or not 0 <= start < nv:
                raise ValueError("MeshGraph start vertex outside the mesh")

    @staticmethod
    def concatenate(sets):
        types = np.concatenate([s.types for s in sets])
        poses = np.concatenate([s.poses for s in sets])
        params = np.concatenate([s.params for s in sets])
        counts = np.concatenate([s.hull_count for s in sets])
        offs, base = [], 0
        for s in sets:
            o = s.hull_offset.copy()
            o[o >= 0] += base
            offs.append(o)
            base += len(s.vertices)
        verts = np.concatenate([s.vertices for s in sets]) if sets else np.zeros((0, 4))
        params = params.copy()
        row, link_base, links = 0, 0, []
        for s in sets:
            mesh = np.flatnonzero(s.base_types == MESH) + row
            params[mesh, 0] += link_base
            row += len(s)
            link_base += len(s.links)
            links.append(s.links)
        links = np.concatenate(links) if links else np.zeros(0, np.int32)
        return ColliderSet(types, poses, params, np.concatenate(offs), counts, verts, links)

    @staticmethod
    def from_colliders(colliders):
        """Pack collider objects with distance3d's attribute names.

        Accepts this package's colliders and distance3d's own (the class name,
        searched along the MRO, selects the type; the attributes read are the
        ones distance3d's constructors set, colliders.py:109-647).
        """
        n = len(colliders)
        types = np.zeros(n, np.int32)
        poses = np.zeros((n, 12))
        params = np.zeros((n, 4))
        offs = np.full(n, -1, np.int64)
        counts = np.zeros(n, np.int32)
        verts = []
        links = []
        nv = 0
        nl = 0
        for i, c in enumerate(colliders):
            if _is_margin(c):
                inner = c.collider
                if _is_margin(inner):
                    raise TypeError("Margin of a Margin is not supported on the GPU path")
                params[i, 3] = float(c.margin)
                flag = MARGIN
                c = inner
            else:
                flag = 0
            t = collider_type(c)
            types[i] = t | flag
            if t == SPHERE:
                pose = np.eye(4)
                pose[:3, 3] = np.asarray(c.c, dtype=float)
                params[i, 0] = float(c.radius)
            elif t == CAPSULE:
                pose = np.asarray(c.capsule2origin, dtype=float)
                params[i, :2] = (float(c.radius), float(c.height))
            elif t == BOX:
                pose = np.asarray(c.box2origin, dtype=float)
                params[i, :3] = np.asarray(c.size, dtype=float).reshape(-1)[:3] * np.ones(3)
            elif t == CYLINDER:
                pose = np.asarray(c.cylinder2origin, dtype=float)
                params[i, :2] = (float(c.radius), float(c.length))
            elif t == ELLIPSOID:
                pose = np.asarray(c.ellipsoid2origin, dtype=float)
                params[i, :3] = np.asarray(c.radii, dtype=float)
            elif t == DISK:
                pose = np.eye(4)
                pose[:3, 2] = np.asarray(c.normal, dtype=float)
                pose[:3, 3] = np.asarray(c.c, dtype=float)
                params[i, 0] = float(c.radius)
            elif t == ELLIPSE:
                axes = np.asarray(c.axes, dtype=float).reshape(2, 3)
                pose = np.eye(4)
                pose[:3, :2] = axes.T
                pose[:3, 2] = np.cross(axes[0], axes[1])
                pose[:3, 3] = np.asarray(c.c, dtype=float)
                params[i, :2] = np.asarray(c.radii, dtype=float).reshape(-1)[:2]
            elif t == CONE:
                pose = np.asarray(c.cone2origin, dtype=float)
                params[i, :2] = (float(c.radius), float(c.height))
            elif t == MESH:
                pose = np.asarray(c.mesh2origin, dtype=float)
                v = np.asarray(c.vertices, dtype=float).reshape(-1, 3)
                tri = np.asarray(c.triangles)
                blk = mesh_links(v, tri)
                params[i, :2] = (nl, float(np.min(tri)))
                links.append(blk)
                nl += len(blk)
                offs[i] = nv
                counts[i] = len(v)
                verts.append(v)
                nv += len(v)
            else:
                pose = np.eye(4)
                v = np.asarray(c.vertices, dtype=float).reshape(-1, 3)
                offs[i] = nv
                counts[i] = len(v)
                verts.append(v)
                nv += len(v)
            poses[i, :9] = pose[:3, :3].reshape(-1)
            poses[i, 9:] = pose[:3, 3]
        v = np.concatenate(verts) if verts else np.zeros((0, 3))
        links = np.concatenate(links) if links else np.zeros(0, np.int32)
        return ColliderSet(types, poses, params, offs, counts, v, links)


def _is_margin(c):
    return any(k.__name__ == "Margin" for k in type(c).__mro__)


def collider_type(c):
    """Type code of a collider object, from its class name along the MRO."""
    for klass in type(c).__mro__:
        name = klass.__name__
        if name in TYPE_NAMES:
            return TYPE_NAMES.index(name)
    raise TypeError(
        f"{type(c).__name__} is not supported on the GPU path (supported: "
        + ", ".join(TYPE_NAMES) + ")")
