"""ctypes binding of libd3d_gb300.so (the C ABI declared in include/d3d_gb300.h).

The library is built in-tree (distance3d_gb300/_build/) by
``distance3d_gb300.build.build()``.  Loading fails loudly when it is missing:
there is no CPU fallback for any entry point.
"""
import ctypes
import os
import threading

from . import build as _build

c_int64, c_int32, c_double, c_void_p, c_size_t = (
    ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t)
c_int = ctypes.c_int

D3D_SUCCESS, D3D_ERR_INVALID, D3D_ERR_CAPACITY, D3D_ERR_CUDA = 0, 1, 2, 3
STATUS_OK, STATUS_CLIPPED, STATUS_SANITY, STATUS_MAX_ITER = 0, 1, 2, 3
STATUS_EPA_NOT_CONVERGED, STATUS_EPA_FACE_OVERFLOW, STATUS_EPA_DEGENERATE = 4, 5, 6
STATUS_BAD_INDEX = 7
PRECISION_FP64, PRECISION_MIXED = 0, 1


class D3DStore(ctypes.Structure):
    _fields_ = [("n_colliders", c_int64), ("n_vertices", c_int64), ("rec64", c_void_p),
                ("rec32", c_void_p), ("meta", c_void_p), ("verts64", c_void_p), ("verts32", c_void_p),
                ("links", c_void_p), ("n_links", c_int64)]


class GjkOptions(ctypes.Structure):
    _fields_ = [("tolerance", c_double), ("max_distance_squared", c_double),
                ("sanity_check", c_double), ("max_iterations", c_int32), ("precision", c_int32)]


class EpaOptions(ctypes.Structure):
    _fields_ = [("max_iterations", c_int32), ("max_loose_edges", c_int32), ("max_faces", c_int32),
                ("precision", c_int32), ("epsilon", c_double)]


class MprOptions(ctypes.Structure):
    _fields_ = [("tolerance", c_double), ("max_iterations", c_int32), ("refine_limit", c_int32),
                ("penetration", c_int32), ("precision", c_int32)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_int64), ("slots", ctypes.c_int32), ("use_graphs", ctypes.c_int32),
                ("hbm_budget", ctypes.c_int64), ("worker_priority", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class PairResults(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("dist", "cp1", "cp2", "simplex", "n_simplex", "status",
                                               "iterations", "mtv", "epa_status", "n_faces")]


class ServerStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_int64), ("max_batch_s", ctypes.c_double), ("max_enqueue_s", ctypes.c_double),
                ("max_loop_gap_s", ctypes.c_double), ("worker_realtime", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("gjk_block", ctypes.c_int32), ("gjk_warps_per_sm", ctypes.c_int32), ("epa_warps", ctypes.c_int32),
                ("sort_min", ctypes.c_int32)]


class Chain(ctypes.Structure):
    _fields_ = [("n_joints", ctypes.c_int32), ("n_bodies", ctypes.c_int32), ("joint_axis", ctypes.c_void_p),
                ("joint_origin", ctypes.c_void_p), ("body_link", ctypes.c_void_p), ("body_origin", ctypes.c_void_p)]


class D3DError(RuntimeError):
    """A libd3d_gb300 entry point returned an error code."""

    def __init__(self, code, message):
        super().__init__(f"libd3d_gb300 error {code}: {message}")
        self.code = code


# (name, restype, argtypes) for every entry point declared in include/d3d_gb300.h
_SP = ctypes.POINTER(D3DStore)
SIGNATURES = [
    ("d3d_abi_version", c_int, []),
    ("d3d_last_error", ctypes.c_char_p, []),
    ("d3d_graph_kernel_nodes", c_int, [c_void_p, ctypes.POINTER(c_int64), ctypes.POINTER(c_int64)]),
    ("d3d_store_pack", c_int, [_SP, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    ("d3d_store_set_poses", c_int, [_SP, c_void_p, c_void_p, c_int64, c_void_p]),
    ("d3d_support", c_int, [_SP, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    ("d3d_aabbs", c_int, [_SP, c_void_p, c_int64, c_void_p, c_void_p]),
    ("d3d_gjk_distance", c_int, [_SP, c_void_p, c_void_p, c_int64, ctypes.POINTER(GjkOptions),
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    ("d3d_gjk_distance_cached", c_int, [_SP, c_void_p, c_void_p, c_int64, ctypes.POINTER(GjkOptions),
                                        c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
    ("d3d_gjk_intersection", c_int, [_SP, c_void_p, c_void_p, c_int64, c_double, c_int32, c_void_p,
                                     c_void_p, c_void_p]),
    ("d3d_epa_scratch_bytes", c_size_t, [c_int64, ctypes.POINTER(EpaOptions)]),
    ("d3d_epa", c_int, [_SP, c_void_p, c_void_p, c_int64, c_void_p, ctypes.POINTER(EpaOptions),
                        c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    ("d3d_epa_noalloc", c_int, [_SP, c_void_p, c_void_p, c_int64, c_void_p, ctypes.POINTER(EpaOptions),
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("d3d_collide_scratch_bytes", c_size_t, [c_int64, ctypes.POINTER(GjkOptions), ctypes.POINTER(EpaOptions)]),
    ("d3d_collide", c_int, [_SP, c_void_p, c_void_p, c_int64, c_void_p, ctypes.POINTER(GjkOptions),
                            ctypes.POINTER(EpaOptions)] + [c_void_p] * 11 + [c_size_t, c_void_p]),
    ("d3d_mpr", c_int, [_SP, c_void_p, c_void_p, c_int64, ctypes.POINTER(MprOptions), c_void_p, c_void_p,
                        c_void_p, c_void_p, c_void_p, c_void_p]),
    ("d3d_chain_fk", c_int, [ctypes.POINTER(Chain), c_void_p, c_int64, c_void_p, c_void_p]),
    ("d3d_get_tuning", c_int, [ctypes.POINTER(Tuning)]),
    ("d3d_set_tuning", c_int, [ctypes.POINTER(Tuning)]),
    ("d3d_autotune", c_int, [_SP, c_void_p, c_void_p, c_int64, ctypes.POINTER(GjkOptions), ctypes.POINTER(EpaOptions),
                             ctypes.POINTER(Tuning), c_void_p]),
    ("d3d_server_create", c_int, [_SP, ctypes.POINTER(GjkOptions), ctypes.POINTER(EpaOptions),
                                  ctypes.POINTER(ServerOptions), ctypes.POINTER(c_void_p)]),
    ("d3d_server_destroy", None, [c_void_p]),
    ("d3d_server_submit", c_int, [c_void_p, c_void_p, c_void_p, c_int64, ctypes.POINTER(c_int64)]),
    ("d3d_server_wait", c_int, [c_void_p, c_int64, c_double]),
    ("d3d_server_result", c_int, [c_void_p, c_int64, ctypes.POINTER(PairResults), ctypes.POINTER(c_double)]),
    ("d3d_server_stats_read", c_int, [c_void_p, ctypes.POINTER(ServerStats), c_int]),
    ("d3d_server_replay", c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                  ctypes.POINTER(c_double)]),
    ("d3d_bvh_bytes", c_size_t, [c_int64]),
    ("d3d_bvh_build", c_int, [c_void_p, c_int64, c_void_p, c_size_t, c_void_p]),
    ("d3d_bvh_refit", c_int, [c_void_p, c_int64, c_void_p, c_size_t, c_void_p]),
    ("d3d_bvh_query_bytes", c_size_t, [c_int64]),
    ("d3d_bvh_self_pairs", c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_int64, ctypes.POINTER(c_int64),
                                   c_void_p, c_size_t, c_void_p]),
    ("d3d_bvh_query", c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_int64,
                              ctypes.POINTER(c_int64), c_void_p, c_size_t, c_void_p]),
]

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.LIB


def load(build_if_missing=False):
    """The loaded library.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if build_if_missing:
                path = _build.build()
            if not os.path.exists(path):
                raise ImportError(
                    f"{path} is missing: build the CUDA library first "
                    "(python -m distance3d_gb300.build, or __graft_entry__.build())")
            lib = ctypes.CDLL(path)
            for name, res, args in SIGNATURES:
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(rc):
    if rc != D3D_SUCCESS:
        msg = load().d3d_last_error().decode(errors="replace")
        raise D3DError(rc, msg)
