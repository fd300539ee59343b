"""ctypes binding of libgbtrace.so (include/gbtrace.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for anything in this package.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbtrace.so")

GBT_OK = 0
ERRORS = {-1: "GBT_EINVAL", -2: "GBT_ECUDA", -3: "GBT_ENOMEM", -4: "GBT_ETIMEOUT", -5: "GBT_EDEVICE",
          -6: "GBT_EUNSUPPORTED"}

# every symbol include/gbtrace.h declares
EXPORTS = [
    "gbt_ctx_create", "gbt_ctx_destroy", "gbt_last_error", "gbt_ctx_stream", "gbt_ctx_sync",
    "gbt_ctx_set_profiling", "gbt_ctx_set_option", "gbt_host_alloc", "gbt_host_free",
    "gbt_scene_upload", "gbt_scene_destroy", "gbt_obj_parse",
    "gbt_lbvh_build", "gbt_lbvh_rebuild_async", "gbt_scene_update_async", "gbt_heatmap", "gbt_heatmap_async", "gbt_phr_build", "gbt_phr_build_with_cost", "gbt_phr_optimize_grid", "gbt_bvh_destroy",
    "gbt_bvh_cost", "gbt_bvh_size", "gbt_bvh_counts", "gbt_bvh_export", "gbt_lbvh_sorted",
    "gbt_trace", "gbt_trace_async", "gbt_render", "gbt_render_async", "gbt_render_last_stats",
    "gbt_device_alloc", "gbt_device_free", "gbt_copy_h2d_async", "gbt_copy_d2h_async",
    "gbt_sort_morton_pairs_noalloc", "gbt_bvh_set_layout", "gbt_bvh_set_packets",
    "gbt_bvh_get_packets",
    "gbt_render_batch_async", "gbt_render_batch_plain_async", "gbt_batch_autotune", "gbt_batch_graph_create",
    "gbt_graph_launch", "gbt_graph_destroy",
    "gbt_adjoint_forward_async", "gbt_adjoint_backward_async", "gbt_l2_loss_async",
    "gbt_buffer_create", "gbt_buffer_destroy", "gbt_render_to_buffer", "gbt_render_to_buffer_async",
    "gbt_buffer_read", "gbt_buffer_to_image", "gbt_buffer_add_async",
]


class Sphere(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float)]


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("color", C.c_float * 3), ("param", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("look_from", C.c_double * 3), ("look_at", C.c_double * 3), ("up", C.c_double * 3),
                ("aspect", C.c_double), ("fov_deg", C.c_double)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("miss_mode", C.c_int32), ("miss_color", C.c_float * 3), ("seed", C.c_uint64)]


class BatchItem(C.Structure):
    _fields_ = [("bvh", C.c_void_p), ("camera", Camera), ("params", RenderParams), ("d_rgb", C.c_void_p)]


BATCH_MEGAKERNEL, BATCH_WAVEFRONT = 0, 1


class BatchConfig(C.Structure):
    _fields_ = [("block", C.c_int32), ("fetch_min", C.c_int32), ("stack", C.c_int32), ("mode", C.c_int32),
                ("packets", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("rays_traced", C.c_uint64), ("paths", C.c_uint64), ("ms_total", C.c_double),
                ("ms_traverse", C.c_double), ("traverse_launches", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("prims_tested", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgbtrace.so is not built (run trace_gb300/build.py or __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    P, i32, u32, i64, d = C.c_void_p, C.c_int32, C.c_uint32, C.c_int64, C.c_double
    PP = C.POINTER(C.c_void_p)
    sig = {
        "gbt_ctx_create": ([C.c_int, PP], C.c_int),
        "gbt_ctx_destroy": ([P], C.c_int),
        "gbt_last_error": ([P], C.c_char_p),
        "gbt_ctx_stream": ([P], C.c_void_p),
        "gbt_ctx_sync": ([P], C.c_int),
        "gbt_ctx_set_profiling": ([P, i32], C.c_int),
        "gbt_ctx_set_option": ([P, i32, i32], C.c_int),
        "gbt_host_alloc": ([P, C.c_size_t, PP], C.c_int),
        "gbt_host_free": ([P, P], C.c_int),
        "gbt_scene_upload": ([P, P, P, u32, P, u32, P, P, u32, PP], C.c_int),
        "gbt_scene_destroy": ([P], C.c_int),
        "gbt_obj_parse": ([C.c_char_p, P, P, C.POINTER(u32), C.POINTER(i32)], C.c_int),
        "gbt_lbvh_build": ([P, P, PP], C.c_int),
        "gbt_lbvh_rebuild_async": ([P, P], C.c_int),
        "gbt_scene_update_async": ([P, P, P], C.c_int),
        "gbt_phr_build": ([P, P, d, d, i32, PP], C.c_int),
        "gbt_phr_build_with_cost": ([P, P, d, d, i32, PP, P], C.c_int),
        "gbt_heatmap": ([P, P, P, i32, i32, i32, P, P], C.c_int),
        "gbt_heatmap_async": ([P, P, P, i32, i32, i32, P, P], C.c_int),
        "gbt_phr_optimize_grid": ([P, P, i32, P, i32, P, i32, i32, i32, P, P, P], C.c_int),
        "gbt_bvh_destroy": ([P], C.c_int),
        "gbt_bvh_cost": ([P, P, C.POINTER(d)], C.c_int),
        "gbt_bvh_size": ([P, P, C.POINTER(i64)], C.c_int),
        "gbt_bvh_counts": ([P, P, P], C.c_int),
        "gbt_bvh_export": ([P, P, P, P, P, P], C.c_int),
        "gbt_lbvh_sorted": ([P, P, P, P], C.c_int),
        "gbt_trace": ([P, P, P, u32, P], C.c_int),
        "gbt_trace_async": ([P, P, P, u32, P], C.c_int),
        "gbt_render": ([P, P, P, P, P, P], C.c_int),
        "gbt_render_async": ([P, P, P, P, P], C.c_int),
        "gbt_render_last_stats": ([P, P], C.c_int),
        "gbt_device_alloc": ([P, C.c_size_t, PP], C.c_int),
        "gbt_device_free": ([P, P], C.c_int),
        "gbt_copy_h2d_async": ([P, P, P, C.c_size_t], C.c_int),
        "gbt_copy_d2h_async": ([P, P, P, C.c_size_t], C.c_int),
        "gbt_sort_morton_pairs_noalloc": ([P, P, P, P, u32], C.c_int),
        "gbt_bvh_set_layout": ([P, P, i32], C.c_int),
        "gbt_bvh_set_packets": ([P, P, i32], C.c_int),
        "gbt_bvh_get_packets": ([P, P, P], C.c_int),
        "gbt_render_batch_async": ([P, P, u32, P], C.c_int),
        "gbt_render_batch_plain_async": ([P, P, u32], C.c_int),
        "gbt_batch_autotune": ([P, P, u32, P, C.POINTER(d)], C.c_int),
        "gbt_batch_graph_create": ([P, P, u32, P, i32, PP], C.c_int),
        "gbt_graph_launch": ([P, P], C.c_int),
        "gbt_graph_destroy": ([P], C.c_int),
        "gbt_adjoint_forward_async": ([P, P, P, P, P, P, P], C.c_int),
        "gbt_adjoint_backward_async": ([P, P, P, P, P, P, P, P, P], C.c_int),
        "gbt_l2_loss_async": ([P, P, P, u32, P, P], C.c_int),
        "gbt_buffer_create": ([P, i32, i32, i32, PP], C.c_int),
        "gbt_buffer_destroy": ([P], C.c_int),
        "gbt_render_to_buffer": ([P, P, P, P, P, P], C.c_int),
        "gbt_render_to_buffer_async": ([P, P, P, P, P], C.c_int),
        "gbt_buffer_read": ([P, P, P, C.POINTER(C.c_uint64)], C.c_int),
        "gbt_buffer_to_image": ([P, P, P], C.c_int),
        "gbt_buffer_add_async": ([P, P, P, i32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


class GbtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code
