"""Colliders with distance3d's constructors and attributes.

Mirrors distance3d colliders.py:17-647 for the types on the GPU path:
``ConvexHullVertices``, ``Box``, ``Sphere``, ``Capsule``, ``Ellipsoid``,
``Cylinder``, ``Disk``, ``Ellipse``, ``Cone``, ``MeshGraph`` and the
``Margin`` wrapper.  Attributes carry the reference's names
(``c``/``radius``, ``capsule2origin``/``radius``/``height``,
``box2origin``/``size``, ...), so
``ColliderSet.from_colliders`` packs these and the reference's own objects
alike.  ``support_function`` and ``aabb`` run on the GPU (one-collider store,
cached until ``update_pose``); ``make_artist`` is not provided (no
visualisation on this path).
"""
import abc

import numpy as np

from .collider_set import ColliderSet


class ConvexCollider(abc.ABC):
    """Convex collider base class (colliders.py:17-106)."""

    def __init__(self, artist=None):
        self.artist_ = artist
        self._store = None

    def make_artist(self, c=None):
        raise NotImplementedError("distance3d_gb300 has no visualisation")

    def _device_store(self):
        if self._store is None:
            from .store import ColliderStore
            self._store = ColliderStore(ColliderSet.from_colliders([self]))
        return self._store

    def _invalidate(self):
        self._store = None

    def support_function(self, search_direction):
        """Extreme point along ``search_direction`` (FP64, on the GPU)."""
        d = np.asarray(search_direction, dtype=np.float64).reshape(1, 3)
        return self._device_store().support([0], d)[0].cpu().numpy()

    def aabb(self):
        """(3,2) axis-aligned bounding box ([axis][min,max], on the GPU)."""
        return self._device_store().aabbs()[0].cpu().numpy()

    @abc.abstractmethod
    def first_vertex(self):
        """Vertex with index 0."""

    @abc.abstractmethod
    def center(self):
        """(Approximate) center."""

    @abc.abstractmethod
    def update_pose(self, pose):
        """Set a new 4x4 pose."""

    @abc.abstractmethod
    def collider2origin(self):
        """4x4 pose."""


class ConvexHullVertices(ConvexCollider):
    """Convex hull of a set of vertices (colliders.py:109-144)."""

    def __init__(self, vertices, artist=None):
        super().__init__(artist)
        self.vertices = vertices

    def first_vertex(self):
        return self.vertices[0]

    def center(self):
        return np.mean(self.vertices, axis=0)

    def update_pose(self, pose):
        raise NotImplementedError("update_pose is not implemented!")

    def collider2origin(self):
        return np.eye(4)


class Box(ConvexHullVertices):
    """Box collider (colliders.py:147-184); ``size`` is the full edge lengths."""

    def __init__(self, box2origin, size, artist=None):
        ConvexCollider.__init__(self, artist)
        self.box2origin = box2origin
        self.size = size

    @property
    def vertices(self):
        """The 8 vertices (geometry.py:138-157), derived on the GPU."""
        st = self._device_store()
        return st.verts64[:8, :3].cpu().numpy()

    @vertices.setter
    def vertices(self, value):  # ConvexHullVertices.__init__ is bypassed; kept for symmetry
        raise AttributeError("Box vertices are derived from box2origin and size")

    def first_vertex(self):
        return self.vertices[0]

    def center(self):
        return self.box2origin[:3, 3]

    def update_pose(self, pose):
        self.box2origin = pose
        self._invalidate()

    def collider2origin(self):
        return self.box2origin


class Sphere(ConvexCollider):
    """Sphere collider (colliders.py:243-287)."""

    def __init__(self, center, radius, artist=None):
        super().__init__(artist)
        self.c = center
        self.radius = radius

    def center(self):
        return self.c

    def first_vertex(self):
        return self.c + np.array([0, 0, self.radius], dtype=float)

    def update_pose(self, pose):
        self.c = pose[:3, 3]
        self._invalidate()

    def collider2origin(self):
        m = np.eye(4)
        m[:3, 3] = self.c
        return m


class Capsule(ConvexCollider):
    """Capsule collider (colliders.py:290-340)."""

    def __init__(self, capsule2origin, radius, height, artist=None):
        super().__init__(artist)
        self.capsule2origin = capsule2origin
        self.radius = radius
        self.height = height

    def center(self):
        return self.capsule2origin[:3, 3]

    def first_vertex(self):
        return self.capsule2origin[:3, 3] - (self.radius + 0.5 * self.height) * self.capsule2origin[:3, 2]

    def update_pose(self, pose):
        self.capsule2origin = pose
        self._invalidate()

    def collider2origin(self):
        return self.capsule2origin


class Ellipsoid(ConvexCollider):
    """Ellipsoid collider (colliders.py:343-387)."""

    def __init__(self, ellipsoid2origin, radii, artist=None):
        super().__init__(artist)
        self.ellipsoid2origin = ellipsoid2origin
        self.radii = radii

    def center(self):
        return self.ellipsoid2origin[:3, 3]

    def first_vertex(self):
        return self.ellipsoid2origin[:3, 3] + self.radii[2] * self.ellipsoid2origin[:3, 2]

    def update_pose(self, pose):
        self.ellipsoid2origin = pose
        self._invalidate()

    def collider2origin(self):
        return self.ellipsoid2origin


class Cylinder(ConvexCollider):
    """Cylinder collider (colliders.py:390-440)."""

    def __init__(self, cylinder2origin, radius, length, artist=None):
        super().__init__(artist)
        self.cylinder2origin = cylinder2origin
        self.radius = radius
        self.length = length

    def center(self):
        return self.cylinder2origin[:3, 3]

    def first_vertex(self):
        return self.cylinder2origin[:3, 3] + 0.5 * self.length * self.cylinder2origin[:3, 2]

    def update_pose(self, pose):
        self.cylinder2origin = pose
        self._invalidate()

    def collider2origin(self):
        return self.cylinder2origin


def _plane_basis(n):
    """utils.py:78-122 plane_basis_from_normal."""
    if abs(n[0]) >= abs(n[1]):
        length = np.sqrt(n[0] * n[0] + n[2] * n[2])
        x = np.array([-n[2] / length, 0.0, n[0] / length])
        y = np.array([n[1] * x[2], n[2] * x[0] - n[0] * x[2], -n[1] * x[0]])
    else:
        length = np.sqrt(n[1] * n[1] + n[2] * n[2])
        x = np.array([0.0, n[2] / length, -n[1] / length])
        y = np.array([n[1] * x[2] - n[2] * x[1], -n[0] * x[2], n[0] * x[1]])
    return x, y


class Disk(ConvexCollider):
    """Disk collider (colliders.py:443-497)."""

    def __init__(self, center, radius, normal, artist=None):
        super().__init__(artist)
        self.c = center
        self.radius = radius
        self.normal = normal

    def center(self):
        return self.c

    def first_vertex(self):
        x, _ = _plane_basis(np.asarray(self.normal, dtype=float))
        return self.c + self.radius * x

    def update_pose(self, pose):
        self.c = pose[:3, 3]
        self.normal = pose[:3, 2]
        self._invalidate()

    def collider2origin(self):
        x, y = _plane_basis(np.asarray(self.normal, dtype=float))
        m = np.eye(4)
        m[:3, :3] = np.column_stack((x, y, self.normal))
        m[:3, 3] = self.c
        return m


class Ellipse(ConvexCollider):
    """Ellipse collider (colliders.py:500-551); ``axes`` (2,3), ``radii`` (2,)."""

    def __init__(self, center, axes, radii, artist=None):
        super().__init__(artist)
        self.c = center
        self.axes = axes
        self.radii = radii

    def center(self):
        return self.c

    def first_vertex(self):
        return self.c + self.axes[0] * self.radii[0]

    def update_pose(self, pose):
        self.c = pose[:3, 3]
        self.axes = pose[:3, :2].T
        self._invalidate()

    def collider2origin(self):
        m = np.eye(4)
        m[:3, :2] = self.axes.T
        m[:3, 2] = np.cross(self.axes[0], self.axes[1])
        m[:3, 3] = self.c
        return m


class Cone(ConvexCollider):
    """Cone collider (colliders.py:554-603): base disk at the origin of
    ``cone2origin``, tip at ``height`` along its z axis."""

    def __init__(self, cone2origin, radius, height, artist=None):
        super().__init__(artist)
        self.cone2origin = cone2origin
        self.radius = radius
        self.height = height

    def center(self):
        return self.cone2origin[:3, 3] + 0.5 * self.height * self.cone2origin[:3, 2]

    def first_vertex(self):
        return self.cone2origin[:3, 3] + self.height * self.cone2origin[:3, 2]

    def update_pose(self, pose):
        self.cone2origin = pose
        self._invalidate()

    def collider2origin(self):
        return self.cone2origin


class MeshGraph(ConvexCollider):
    """Convex mesh with hill-climbing support (colliders.py:187-240):
    ``vertices`` (n,3) in the mesh frame, ``triangles`` (m,3) vertex
    indices.  ``first_idx`` is the reference's vertex cache
    (mesh.py:30, 85): the hill climbs of ``gjk.gjk_distance`` on this
    collider start from it and leave their last answer in it, as the
    reference's support object does.  ``support_function`` climbs from the
    mesh's start vertex (the smallest index in ``triangles``) and leaves the
    cache alone; that gives the same vertex unless the climb can stop within
    10 EPSILON of the maximum."""

    def __init__(self, mesh2origin, vertices, triangles, artist=None):
        super().__init__(artist)
        self.mesh2origin = mesh2origin
        self.vertices = vertices
        self.triangles = triangles
        self.first_idx = int(np.min(triangles))

    def first_vertex(self):
        return self.mesh2origin[:3, 3] + np.dot(self.mesh2origin[:3, :3], self.vertices[0])

    def center(self):
        return self.mesh2origin[:3, 3] + np.dot(self.mesh2origin[:3, :3], np.mean(self.vertices, axis=0))

    def update_pose(self, mesh2origin):
        self.mesh2origin = mesh2origin
        self._invalidate()

    def collider2origin(self):
        return self.mesh2origin


class Margin(ConvexCollider):
    """Margin around another collider (colliders.py:606-647): its support
    point moved by ``margin`` along the unit search direction, its box grown
    by ``margin``."""

    def __init__(self, collider, margin):
        super().__init__(getattr(collider, "artist_", None))
        self.collider = collider
        self.margin = margin

    def first_vertex(self):
        return self.collider.first_vertex()

    def center(self):
        return self.collider.center()

    def update_pose(self, pose):
        self.collider.update_pose(pose)
        self._invalidate()

    def collider2origin(self):
        return self.collider.collider2origin()


COLLIDERS = {
    "sphere": Sphere,
    "ellipsoid": Ellipsoid,
    "capsule": Capsule,
    "cylinder": Cylinder,
    "box": Box,
    "convex": ConvexHullVertices,
    "disk": Disk,
    "ellipse": Ellipse,
    "cone": Cone,
    "mesh": MeshGraph,
}
