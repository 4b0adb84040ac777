"""ctypes binding of libmcl_gb300.so (the C ABI declared in include/mcl_gb300.h).

The shared library is the engine: there is no Python or CPU fallback.  Loading
fails loudly when the library has not been built (``python -m
mcleap_gb300.build``) or when no CUDA device is present for device calls.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcl_gb300.so")

MCL_OK = 0
MCL_ERR_INVALID_ARGUMENT = 1
MCL_ERR_CUDA = 2
MCL_ERR_OUT_OF_MEMORY = 3
MCL_ERR_NO_CONVERGENCE = 4
MCL_ERR_CAPACITY = 5
MCL_ERR_DEGENERATE_INPUT = 6
MCL_ERR_PREDICATE = 7
MCL_ERR_NO_DEVICE = 8

LAYOUT_COLUMN = 0
LAYOUT_ROW = 1
GRID_PERIODIC = 1

EXPORTS = [
    "mcl_status_string", "mcl_last_error", "mcl_version",
    "mcl_mesh_create_from_aos", "mcl_mesh_build", "mcl_mesh_destroy", "mcl_mesh_sizes",
    "mcl_mesh_download_aos", "mcl_mesh_upload_aos", "mcl_mesh_positions", "mcl_mesh_copy_positions", "mcl_move", "mcl_integrate",
    "mcl_untangle", "mcl_delaunay_restore", "mcl_step", "mcl_step_host", "mcl_step_host_async", "mcl_mesh_last_status", "mcl_mesh_totals",
    "mcl_one_ring", "mcl_closest_neighbors", "mcl_mesh_frnn",
    "mcl_grid_create", "mcl_grid_destroy", "mcl_grid_update", "mcl_grid_tables", "mcl_grid_describe", "mcl_grid_frnn",
    "mcl_grid_build", "mcl_grid_frnn_ids",
    "mcl_batch_create", "mcl_batch_count", "mcl_batch_range", "mcl_batch_vertex_mesh", "mcl_batch_download_aos",
    "mcl_batch_frnn", "mcl_mesh_clone", "mcl_mesh_set_tuning", "mcl_mesh_get_tuning", "mcl_mesh_set_substeps", "mcl_walk",
    "mcl_settle_moves", "mcl_dla_freeze", "mcl_batch_frnn_list", "mcl_one_ring_list", "mcl_batch_set_active", "mcl_batch_frnn_grid",
    "mcl_grid_mean_occupancy", "mcl_debug_predicates_host", "mcl_debug_predicates_device", "mcl_mesh_validate", "mcl_debug_state", "mcl_debug_timeline", "mcl_grid_frnn_noalloc", "mcl_debug_counters",
    "mcl_debug_insert_timeline", "mcl_debug_remove_timeline", "mcl_mesh_export_aos", "mcl_walk_seeded",
    "mcl_mesh_set_removal_tile", "mcl_mesh_get_removal_tile",
    "mcl_periodic_build", "mcl_periodic_create", "mcl_periodic_destroy", "mcl_periodic_sizes", "mcl_periodic_download",
    "mcl_periodic_positions", "mcl_periodic_step", "mcl_periodic_from_planar", "mcl_periodic_one_ring",
    "mcl_periodic_closest", "mcl_periodic_frnn", "mcl_periodic_step_host", "mcl_periodic_debug_timeline",
]


class McleapError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mcl error {code}: {msg}")
        self.code = code


class AosView(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("v", C.c_void_p), ("he", C.c_void_p), ("t", C.c_void_p),
                ("V", C.c_int64), ("HE", C.c_int64), ("T", C.c_int64)]


STAT_FIELDS = ["inverted_faces", "reverted_vertices", "removed_vertices", "lawson_flips", "lawson_rounds",
               "removal_flips", "insert_rounds", "incircle_tests", "incircle_fp64", "incircle_exact",
               "orient_fp64", "orient_exact", "sos_decisions", "status", "error_site", "failed_launches",
               "substep_vertices"]


class StepStats(C.Structure):
    _fields_ = [(f, C.c_int64) for f in STAT_FIELDS]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f in STAT_FIELDS}


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m mcleap_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp, i64, i32, f32 = C.c_void_p, C.c_int64, C.c_int, C.c_float
        sig = {
            "mcl_status_string": ([i32], C.c_char_p),
            "mcl_last_error": ([], C.c_char_p),
            "mcl_version": ([], i32),
            "mcl_mesh_create_from_aos": ([C.POINTER(AosView), C.POINTER(vp)], i32),
            "mcl_mesh_build": ([vp, i64, C.POINTER(vp)], i32),
            "mcl_mesh_destroy": ([vp], i32),
            "mcl_mesh_sizes": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], i32),
            "mcl_mesh_download_aos": ([vp, vp, vp, vp, vp], i32),
            "mcl_mesh_upload_aos": ([vp, C.POINTER(AosView)], i32),
            "mcl_mesh_positions": ([vp, C.POINTER(vp)], i32),
            "mcl_mesh_copy_positions": ([vp, vp, i32, vp], i32),
            "mcl_move": ([vp, vp, vp], i32),
            "mcl_integrate": ([vp, vp, vp, vp], i32),
            "mcl_untangle": ([vp, vp, C.POINTER(StepStats)], i32),
            "mcl_delaunay_restore": ([vp, vp, C.POINTER(StepStats)], i32),
            "mcl_step": ([vp, vp, vp, C.POINTER(StepStats)], i32),
            "mcl_step_host": ([vp, vp, vp, C.POINTER(StepStats)], i32),
            "mcl_step_host_async": ([vp, vp, vp, vp], i32),
            "mcl_mesh_last_status": ([vp, vp, C.POINTER(StepStats)], i32),
            "mcl_mesh_totals": ([vp, C.POINTER(StepStats), C.POINTER(i64)], i32),
            "mcl_one_ring": ([vp, i32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_closest_neighbors": ([vp, i32, i32, vp, vp, vp], i32),
            "mcl_mesh_frnn": ([vp, f32, i32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_grid_create": ([i64, f32, f32, f32, f32, i32, i32, i32, C.POINTER(vp)], i32),
            "mcl_grid_destroy": ([vp], i32),
            "mcl_grid_update": ([vp, vp, vp, vp], i32),
            "mcl_grid_tables": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(i32), C.POINTER(i32)], i32),
            "mcl_grid_frnn": ([vp, vp, f32, i32, vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_grid_describe": ([vp, vp], i32),
            "mcl_grid_build": ([vp, vp, vp], i32),
            "mcl_grid_frnn_ids": ([vp, f32, i32, vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_grid_mean_occupancy": ([vp, C.POINTER(f32)], i32),
            "mcl_debug_predicates_host": ([i32, vp, vp, i64, vp, vp], i32),
            "mcl_mesh_validate": ([vp, vp], i32),
            "mcl_debug_state": ([vp, vp], i32),
            "mcl_debug_timeline": ([vp, vp], i32),
            "mcl_debug_counters": ([vp, vp, i32], i32),
            "mcl_debug_insert_timeline": ([vp, vp], i32),
            "mcl_debug_remove_timeline": ([vp, vp], i32),
            "mcl_mesh_export_aos": ([vp, vp, vp, vp, vp], i32),
            "mcl_walk_seeded": ([vp, vp, vp, vp, vp, f32, f32, vp, vp], i32),
            "mcl_mesh_set_removal_tile": ([vp, i32], i32),
            "mcl_mesh_get_removal_tile": ([vp, C.POINTER(i32)], i32),
            "mcl_grid_frnn_noalloc": ([vp, i64, f32, f32, f32, f32, i32, i32, i32, f32, i32, vp, vp, vp, vp, vp,
                                       C.POINTER(i64)], i32),
            "mcl_debug_predicates_device": ([i32, vp, vp, i64, vp, vp, vp], i32),
            "mcl_batch_create": ([vp, i64, C.POINTER(vp)], i32),
            "mcl_batch_count": ([vp, C.POINTER(i64)], i32),
            "mcl_batch_range": ([vp, i64, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], i32),
            "mcl_batch_vertex_mesh": ([vp, C.POINTER(vp)], i32),
            "mcl_batch_download_aos": ([vp, i64, vp, vp, vp, vp], i32),
            "mcl_batch_frnn": ([vp, vp, i32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_mesh_clone": ([vp, C.POINTER(vp)], i32),
            "mcl_mesh_set_tuning": ([vp, i32, i32], i32),
            "mcl_mesh_set_substeps": ([vp, i32], i32),
            "mcl_mesh_get_tuning": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32),
            "mcl_walk": ([vp, vp, vp, C.c_uint64, vp, f32, f32, vp, vp], i32),
            "mcl_settle_moves": ([vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_dla_freeze": ([vp, vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_batch_frnn_list": ([vp, vp, vp, i64, i32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_one_ring_list": ([vp, vp, i64, i32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_batch_set_active": ([vp, vp, i64, vp], i32),
            "mcl_batch_frnn_grid": ([vp, vp, vp, f32, f32, i32, vp, vp, C.POINTER(i64)], i32),
            "mcl_periodic_build": ([vp, i64, f32, C.POINTER(vp)], i32),
            "mcl_periodic_create": ([vp, i64, f32, vp, vp, vp, C.POINTER(vp)], i32),
            "mcl_periodic_destroy": ([vp], i32),
            "mcl_periodic_sizes": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(f32)], i32),
            "mcl_periodic_download": ([vp, vp, vp, vp, vp], i32),
            "mcl_periodic_positions": ([vp, C.POINTER(vp)], i32),
            "mcl_periodic_step": ([vp, vp, vp, C.POINTER(StepStats), C.POINTER(i64)], i32),
            "mcl_periodic_from_planar": ([C.POINTER(AosView), vp, vp, i64, vp, vp, vp], i32),
            "mcl_periodic_one_ring": ([vp, i32, i32, vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_periodic_closest": ([vp, i32, i32, vp, vp, vp, vp], i32),
            "mcl_periodic_frnn": ([vp, f32, i32, i32, vp, vp, vp, C.POINTER(i64)], i32),
            "mcl_periodic_step_host": ([vp, vp, vp, C.POINTER(StepStats), C.POINTER(i64)], i32),
            "mcl_periodic_debug_timeline": ([vp, vp, C.POINTER(i64)], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def check(rc):
    if rc != MCL_OK:
        L = lib()
        msg = L.mcl_last_error().decode() or L.mcl_status_string(rc).decode()
        raise McleapError(rc, msg)
    return rc


def ptr(x):
    """Address of a numpy array, a torch tensor, or an int; None -> NULL."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        assert x.flags["C_CONTIGUOUS"]
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        assert x.is_contiguous()
        return x.data_ptr()
    raise TypeError(f"cannot take the address of {type(x)}")


def predicates_host(kind, pts, ids=None):
    """The device predicate ladder run on the host CPU (same source)."""
    pts = np.ascontiguousarray(pts, np.float32)
    n = len(pts)
    sign = np.zeros(n, np.int32)
    stage = np.zeros(n, np.int32)
    idsa = None if ids is None else np.ascontiguousarray(ids, np.int32)
    check(lib().mcl_debug_predicates_host(kind, ptr(pts), ptr(idsa), n, ptr(sign), ptr(stage)))
    return sign, stage
