"""distance3d_gb300: distance3d's narrow and broad phase on one GB300.

Batched Jolt GJK distance and intersection, EPA, the Sphere / Capsule / Box /
Cylinder / Ellipsoid / ConvexHullVertices / Disk / Ellipse / Cone support
functions (each optionally wrapped in Margin) and AABB queries,
as hand-written sm_103a CUDA kernels behind the C ABI of libd3d_gb300.so
(include/d3d_gb300.h).  The modules mirror distance3d's call surface:

* ``distance3d_gb300.colliders``  -- collider classes (colliders.py)
* ``distance3d_gb300.gjk``        -- gjk, gjk_distance, gjk_intersection, batched forms
* ``distance3d_gb300.epa``        -- epa, epa_batch
* ``distance3d_gb300.store``      -- ColliderStore, the device-resident collider batch
* ``distance3d_gb300.collider_set`` -- the packed host format
"""
from ._lib import (STATUS_OK, STATUS_CLIPPED, STATUS_SANITY, STATUS_MAX_ITER,  # noqa: F401
                   STATUS_EPA_NOT_CONVERGED, STATUS_EPA_FACE_OVERFLOW, STATUS_EPA_DEGENERATE,
                   STATUS_BAD_INDEX, D3DError)
from .collider_set import (ColliderSet, SPHERE, CAPSULE, BOX, CYLINDER, ELLIPSOID, HULL,  # noqa: F401
                           DISK, ELLIPSE, CONE, MARGIN)

__version__ = "0.1.0"
