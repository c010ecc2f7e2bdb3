"""ctypes binding of ``libthea_gpu.so`` (the C ABI declared in ``include/thea_gpu.h``).

Loading fails loudly: there is no fallback implementation of any entry point.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libthea_gpu.so")

THEA_OK = 0
STATUS_NAMES = {0: "THEA_OK", 1: "THEA_ERR_INVALID_ARGUMENT", 2: "THEA_ERR_OUT_OF_MEMORY",
                3: "THEA_ERR_ADMISSION_REFUSED", 4: "THEA_ERR_DEVICE_TIMEOUT", 5: "THEA_ERR_CUDA",
                6: "THEA_ERR_INTERNAL", 7: "THEA_ERR_NOT_SUPPORTED", 8: "THEA_ERR_CANCELLED",
                9: "THEA_ERR_WAIT_TIMEOUT"}
THEA_ERR_INVALID_ARGUMENT = 1
THEA_ERR_ADMISSION_REFUSED = 3
THEA_ERR_DEVICE_TIMEOUT = 4
THEA_ERR_INTERNAL = 6
THEA_ERR_CANCELLED = 8
THEA_ERR_WAIT_TIMEOUT = 9

LAYOUT_CLOSEST = 1
LAYOUT_RAY = 2
RNG_THEA_MT = 0
RNG_COUNTER = 1

# Every symbol the header declares, with (restype, argtypes)
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u32 = ctypes.c_uint32
_f32 = ctypes.c_float
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


class BuildConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("max_leaf_size", ctypes.c_int32), ("layouts", ctypes.c_uint32),
                ("query_order", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


class BvhInfo(ctypes.Structure):
    _fields_ = [("num_elements", ctypes.c_int64), ("num_nodes", ctypes.c_int64), ("width", ctypes.c_int32),
                ("max_leaf_size", ctypes.c_int32), ("is_mesh", ctypes.c_int32), ("depth", ctypes.c_int32),
                ("device_bytes", ctypes.c_int64), ("bounds_lo", ctypes.c_float * 3), ("bounds_hi", ctypes.c_float * 3),
                ("device_error_bits", ctypes.c_uint32), ("num_segments", ctypes.c_int32)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_int64), ("num_triangles", ctypes.c_int64), ("num_faces", ctypes.c_int64),
                ("num_submeshes", ctypes.c_int64)]


class Tuning(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("max_leaf_size", ctypes.c_int32), ("queries_per_warp", ctypes.c_int32),
                ("milliseconds", ctypes.c_float), ("candidates", ctypes.c_int32),
                ("hard_query_budget", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_int64), ("slots", ctypes.c_int32),
                ("max_batch_queries", ctypes.c_int32), ("max_piece_queries", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("width", ctypes.c_int32), ("max_leaf_size", ctypes.c_int32),
                ("small_request_queries", ctypes.c_int32), ("max_wait_ms", ctypes.c_int32),
                ("test_executor", ctypes.c_int32), ("test_ns_per_query", ctypes.c_int32),
                ("hard_query_budget", ctypes.c_int32), ("reserved", ctypes.c_int32 * 5)]


class Request(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("mesh", ctypes.c_int32), ("num_queries", ctypes.c_int64),
                ("queries", ctypes.c_void_p), ("directions", ctypes.c_void_p), ("bound", ctypes.c_float),
                ("k", ctypes.c_int32), ("out_index", ctypes.c_void_p), ("out_value", ctypes.c_void_p),
                ("out_point", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "cancelled", "refused",
                                              "queries_completed", "batches", "resident_meshes", "resident_bytes",
                                              "inflight_bytes", "pending_requests")] + \
               [(n, ctypes.c_double) for n in ("p50_ms", "p99_ms", "max_ms", "small_p50_ms", "small_p99_ms",
                                               "busy_seconds", "queries_per_second")]


KNN_CANDIDATES_TRAVERSAL = 0
KNN_CANDIDATES_GRAM = 1

REQUEST_CLOSEST = 0
REQUEST_RAY = 1
REQUEST_KNN = 2

SIGNATURES = {
    "thea_abi_version": (ctypes.c_int, []),
    "thea_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "thea_last_error_message": (ctypes.c_char_p, []),
    "thea_launch_count": (ctypes.c_int64, []),
    "thea_allocation_count": (ctypes.c_int64, []),
    "thea_profiling_enable": (ctypes.c_int, [ctypes.c_int]),
    "thea_profiling_reset": (ctypes.c_int, []),
    "thea_profiling_read": (ctypes.c_int, [ctypes.c_char_p, _f64p, _i64p]),
    "thea_mesh_bvh_build": (ctypes.c_int, [_vp, _i64, _vp, _i64, ctypes.POINTER(BuildConfig), _vp,
                                           ctypes.POINTER(_vp)]),
    "thea_point_bvh_build": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(BuildConfig), _vp, ctypes.POINTER(_vp)]),
    "thea_bvh_destroy": (ctypes.c_int, [_vp]),
    "thea_bvh_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(BvhInfo)]),
    "thea_ray_intersects": (ctypes.c_int, [_vp, _vp, _vp, _i64, ctypes.c_float, _vp, _vp]),
    "thea_sample_graph": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int32, ctypes.c_uint32, _vp, _vp, _vp, _vp, _vp,
                                         _vp]),
    "thea_sample_graph_oversampled": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _i64, ctypes.c_int32, ctypes.c_uint32,
                                                     _vp, _vp, _vp, _vp, _vp, _vp]),
    "thea_random_sphere": (ctypes.c_int, [ctypes.c_uint32, _i64, _vp, _vp]),
    "thea_shape_diameter": (ctypes.c_int, [_vp, _vp, _vp, _i64, ctypes.c_float, ctypes.c_int32, _vp, _vp]),
    "thea_best_fit_sphere": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp]),
    "thea_bvh_closest_pair": (ctypes.c_int, [_vp, _vp, ctypes.c_float, ctypes.POINTER(ctypes.c_int32),
                                             ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float), _vp, _vp,
                                             _vp]),
    "thea_bvh_k_closest_pairs": (ctypes.c_int, [_vp, _vp, ctypes.c_int32, ctypes.c_float, _vp, _vp, _vp,
                                                ctypes.POINTER(ctypes.c_int32), _vp]),
    "thea_mesh_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "thea_mesh_read_buffer": (ctypes.c_int, [_vp, _i64, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "thea_mesh_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(MeshInfo)]),
    "thea_mesh_copy": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "thea_mesh_destroy": (ctypes.c_int, [_vp]),
    "thea_triangulate_face": (ctypes.c_int, [_vp, ctypes.c_int32, _vp, ctypes.POINTER(ctypes.c_int32)]),
    "thea_visibility": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int32, ctypes.c_uint32, _vp, _vp]),
    "thea_bvh_set_transform": (ctypes.c_int, [_vp, _vp, _vp]),
    "thea_bvh_clear_transform": (ctypes.c_int, [_vp]),
    "thea_bvh_get_transform": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "thea_bvh_serialize": (ctypes.c_int, [_vp, _vp, _i64, _i64p, _vp]),
    "thea_bvh_deserialize": (ctypes.c_int, [_vp, _i64, _vp, ctypes.POINTER(_vp)]),
    "thea_closest_element": (ctypes.c_int, [_vp, _vp, _i64, _f32, _vp, _vp, _vp, _vp]),
    "thea_ray_intersection": (ctypes.c_int, [_vp, _vp, _vp, _i64, _f32, _vp, _vp, _vp, _vp]),
    "thea_k_closest": (ctypes.c_int, [_vp, _vp, _i64, _i32, _f32, _vp, _vp, _vp, _vp]),
    "thea_k_closest_self": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp]),
    "thea_sample_by_area": (ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _u32, _i32, _vp, _vp, _vp, _i64p, _vp]),
    "thea_sample_by_area_noalloc": (ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _u32, _i32, _vp, _vp, _vp, _i64p,
                                                   _vp]),
    "thea_closest_element_ex": (ctypes.c_int, [_vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "thea_ray_intersection_ex": (ctypes.c_int, [_vp, _vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "thea_mesh_forest_build": (ctypes.c_int, [_vp, _i64, _vp, _i64p, _i32, ctypes.POINTER(BuildConfig), _vp,
                                              ctypes.POINTER(_vp)]),
    "thea_point_forest_build": (ctypes.c_int, [_vp, _i64p, _i32, ctypes.POINTER(BuildConfig), _vp,
                                               ctypes.POINTER(_vp)]),
    "thea_batch_closest_element": (ctypes.c_int, [_vp, _vp, _vp, _i64, _f32, _i32, _i32, _i32, _vp, _vp, _vp, _vp,
                                                  _vp]),
    "thea_batch_ray_intersection": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, _f32, _i32, _vp, _vp, _vp]),
    "thea_batch_k_closest": (ctypes.c_int, [_vp, _vp, _vp, _i64, _i32, _f32, _i32, _vp, _vp, _vp]),
    "thea_graph_capture_begin": (ctypes.c_int, [_vp]),
    "thea_graph_capture_end": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "thea_graph_launch": (ctypes.c_int, [_vp, _vp]),
    "thea_graph_destroy": (ctypes.c_int, [_vp]),
    "thea_autotune_batch_closest": (ctypes.c_int, [_vp, _i64, _vp, _i64p, _i32, _vp, _vp, _i64, _i32, _vp,
                                                   ctypes.POINTER(Tuning)]),
    "thea_k_closest_self_ex": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "thea_radius_neighbors": (ctypes.c_int, [_vp, _vp, _i64, _f32, _vp, _vp, _vp, _vp, _vp]),
    "thea_selftest_bounded_wait": (ctypes.c_int, [_i32, _vp]),
    "thea_selftest_set_error_bits": (ctypes.c_int, [_vp, ctypes.c_uint32, _vp]),
    "thea_selftest_running_sum": (ctypes.c_int, [_vp, _i64, ctypes.c_float, _vp, _vp]),
    "thea_point_gram_tile": (ctypes.c_int, [_vp, _i32, _vp, _i32, _vp, _vp]),
    "thea_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "thea_server_destroy": (ctypes.c_int, [_vp]),
    "thea_server_add_mesh": (ctypes.c_int, [_vp, _vp, _i64, _vp, _i64, ctypes.POINTER(_i32)]),
    "thea_server_remove_mesh": (ctypes.c_int, [_vp, _i32]),
    "thea_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "thea_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, _i64, ctypes.POINTER(ctypes.c_int), _f64p]),
    "thea_server_cancel": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "thea_server_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "thea_server_reset_stats": (ctypes.c_int, [_vp]),
}

PRECISION_FP32_REFERENCE = 0
PRECISION_FP64_RECHECK = 1
RAY_FLAG_HIT_DIFFERS = 1
RAY_FLAG_ELEMENT_DIFFERS = 2

NOALLOC_MAX_FACES = 1048576

_lib = None


class TheaError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


def lib():
    """Load the native library (built by thea_gb300.build); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("thea_gb300 native library not built (%s); run thea_gb300.build.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != THEA_OK:
        msg = lib().thea_last_error_message()
        raise TheaError(status, msg.decode() if msg else "")
