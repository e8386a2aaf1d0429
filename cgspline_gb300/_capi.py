"""ctypes binding of libcgspline_gb300.so (declarations in include/cgspline.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libcgspline_gb300.so")
# the same sources built without multiply-add contraction (parity build)
LIB_NOFMA_PATH = os.path.join(HERE, "_lib", "libcgspline_gb300_nofma.so")

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "scene not built",
    5: "perfect hash bucket overflow", 6: "perfect hash failed", 7: "empty BVH leaf", 8: "render still in flight",
    9: "device stack/iteration limit", 10: "admission refused", 11: "not found", 12: "exceeds fixed capacity",
}


class CgsError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, 'unknown')} (status {status})")


class Material(C.Structure):
    _fields_ = [("diffuse", C.c_float * 3), ("specular", C.c_float * 3), ("metalness", C.c_float),
                ("roughness", C.c_float)]


class Light(C.Structure):
    _fields_ = [("color", C.c_float * 3), ("strength", C.c_float), ("position", C.c_float * 3), ("range", C.c_float),
                ("direction", C.c_float * 3), ("angle", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("rotation", C.c_float * 4), ("position", C.c_float * 3), ("scale", C.c_float * 3),
                ("fovy", C.c_float)]


class RenderOptions(C.Structure):
    _fields_ = [("recursion_depth", C.c_int), ("eps", C.c_float), ("flip_y", C.c_int), ("method", C.c_int),
                ("precision", C.c_int), ("tol", C.c_float), ("schedule", C.c_int), ("sampling", C.c_int)]


class Rays(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("ox", "oy", "oz", "dx", "dy", "dz", "tmax", "group")]


class RenderRequest(C.Structure):
    _fields_ = [("group", C.c_uint32), ("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp", C.c_uint32), ("recursion_depth", C.c_int), ("framebuffer", C.c_void_p),
                ("linear_rgb", C.c_void_p)]


class Hits(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("t", "u", "v", "patch", "object")]


class EngineConfig(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("passes", "collect_threads", "resolve_threads", "collect_occupancy",
                                       "resolve_occupancy", "backtrack_cache", "compressed_nodes",
                                       "queue_chunk", "packet_width", "ray_order", "origin_last",
                                       "subdiv_levels")]


class ServerOptions(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("memory_budget", C.c_uint64), ("max_batch_samples", C.c_uint32),
                ("max_batch_requests", C.c_uint32), ("render", RenderOptions)]


class QueryRequest(C.Structure):
    _fields_ = [("group", C.c_uint32), ("n", C.c_uint32), ("any_hit", C.c_int), ("rays", Rays), ("hits", Hits)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("chunks", C.c_uint32), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("finish_s", C.c_double), ("samples", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "finished", "rejected", "batches", "chunks", "rays_traced",
                                          "slot_bytes", "peak_slot_bytes", "kernel_launches")] + \
        [("busy_s", C.c_double), ("max_batch_samples", C.c_uint32), ("queued", C.c_uint32)]


class Counters(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("rays", "primary_rays", "bounce_rays", "shadow_rays", "nodes",
                                          "hash_lookups", "candidates", "iterations", "device_errors",
                                          "kernel_launches", "hash_table_reads")]


_libs = {}

# (name, restype, argtypes) for every entry point declared in include/cgspline.h
P = C.c_void_p
U32 = C.c_uint32
SIGNATURES = [
    ("cgs_status_string", C.c_char_p, [C.c_int]),
    ("cgs_version", C.c_int, []),
    ("cgs_scene_create", C.c_int, [C.POINTER(P), C.c_int]),
    ("cgs_scene_destroy", C.c_int, [P]),
    ("cgs_scene_add_surface", C.c_int, [P, P, U32, P, U32, C.POINTER(U32)]),
    ("cgs_scene_add_group", C.c_int, [P, C.POINTER(U32)]),
    ("cgs_scene_add_object", C.c_int, [P, U32, P, P, C.POINTER(Material), P, P, U32, C.POINTER(U32)]),
    ("cgs_scene_set_lights", C.c_int, [P, P, U32]),
    ("cgs_scene_set_environment", C.c_int, [P, P, P]),
    ("cgs_scene_set_bvh_split", C.c_int, [P, C.c_int]),
    ("cgs_bvh_build", C.c_int, [P]),
    ("cgs_hash_build", C.c_int, [P, P]),
    ("cgs_scene_build", C.c_int, [P, P]),
    ("cgs_scene_footprint", C.c_int, [P, C.POINTER(C.c_uint64)]),
    ("cgs_scene_save", C.c_int, [P, C.c_char_p]),
    ("cgs_scene_load", C.c_int, [C.POINTER(P), C.c_char_p, C.c_int]),
    ("cgs_bvh_sizes", C.c_int, [P, C.c_int32, P]),
    ("cgs_bvh_export", C.c_int, [P, C.c_int32, P, P, P, P, P, P]),
    ("cgs_intersect", C.c_int, [P, C.POINTER(Rays), U32, C.c_int, C.c_int, C.c_float, C.c_int, C.POINTER(Hits), P]),
    ("cgs_intersect_host", C.c_int, [P, C.POINTER(Rays), U32, C.c_int, C.c_int, C.c_float, C.c_int, C.POINTER(Hits),
                                     P]),
    ("cgs_traverse", C.c_int, [P, C.POINTER(Rays), U32, C.c_int, P, P]),
    ("cgs_patch_intersect", C.c_int, [P, U32, C.POINTER(Rays), P, U32, C.c_int, C.c_float, C.POINTER(Hits), P]),
    ("cgs_patch_normal", C.c_int, [P, U32, P, P, P, U32, P, P]),
    ("cgs_render", C.c_int, [P, C.POINTER(Camera), U32, U32, C.POINTER(RenderOptions), P, U32, P, P]),
    ("cgs_render_host", C.c_int, [P, C.POINTER(Camera), U32, U32, C.POINTER(RenderOptions), P, P, P]),
    ("cgs_render_batch", C.c_int, [P, C.POINTER(RenderRequest), U32, C.POINTER(RenderOptions), P]),
    ("cgs_render_running", C.c_int, [P]),
    ("cgs_camera_rays", C.c_int, [C.POINTER(Camera), U32, U32, C.c_int, P, P]),
    ("cgs_engine_config_get", C.c_int, [C.POINTER(EngineConfig)]),
    ("cgs_engine_config_set", C.c_int, [C.POINTER(EngineConfig)]),
    ("cgs_autotune_render", C.c_int, [P, C.POINTER(RenderRequest), U32, C.POINTER(RenderOptions), C.c_int,
                                      C.POINTER(EngineConfig), C.POINTER(C.c_double), P]),
    ("cgs_scene_counters", C.c_int, [P, C.POINTER(Counters)]),
    ("cgs_debug_fail_allocation", C.c_int, [U32]),
    ("cgs_perfect_hash_build", C.c_int, [P, U32, P, U32, P, U32, P, P]),
    ("cgs_server_create", C.c_int, [C.POINTER(P), P, C.POINTER(ServerOptions)]),
    ("cgs_server_destroy", C.c_int, [P]),
    ("cgs_server_submit_render", C.c_int, [P, C.POINTER(RenderRequest), C.POINTER(C.c_uint64)]),
    ("cgs_server_submit_query", C.c_int, [P, C.POINTER(QueryRequest), C.POINTER(C.c_uint64)]),
    ("cgs_server_wait", C.c_int, [P, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
    ("cgs_server_clock", C.c_double, [P]),
    ("cgs_server_stats_get", C.c_int, [P, C.POINTER(ServerStats)]),
    ("cgs_perfect_hash_build_noalloc", C.c_int, [P, U32, P, U32, P, U32, P, P]),
]


def load(path: str = LIB_PATH):
    """Load the library at `path` (the product build by default; building it
    first if it is missing)."""
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        try:
            from . import build as _b
            _b.build(fmad=path != LIB_NOFMA_PATH)
        except Exception as e:  # no nvcc / failed build: fail loudly
            raise ImportError(f"{os.path.basename(path)} is missing and could not be built: {e}") from e
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _libs[path] = lib
    return lib


def check(status: int, where: str):
    if status != 0:
        raise CgsError(status, where)
