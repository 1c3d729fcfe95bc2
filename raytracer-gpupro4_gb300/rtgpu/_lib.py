"""ctypes binding of the C ABI declared in include/rt_api.h.

Loading fails loudly when librtgb300.so is missing: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB

RT_OK, RT_ERR_INVALID, RT_ERR_CAPACITY, RT_ERR_CUDA, RT_ERR_TIMEOUT, RT_ERR_NONFINITE = range(6)
RT_BUILD_CLEAR_UNREACHED = 1
RT_BUILD_COMPACT = 2
RT_NOALLOC_MAX_TRIS = 262144
RT_NOALLOC_MAX_DEPTH = 20
RT_NODE_SENTINEL = -2147483647

# Layouts mirrored from include/rt_api.h (LBVHNode / Intersection / Ray of the reference).
NODE_DTYPE = np.dtype([("min", "<f4", (3,)), ("max", "<f4", (3,)), ("prim_count", "<i4"), ("prim_pos", "<i4")])
HIT_DTYPE = np.dtype([("id", "<i4"), ("u", "<f4"), ("v", "<f4"), ("t", "<f4")])
RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("exclude_id", "<i4"), ("d", "<f4", (3,)), ("tmax", "<f4")])
assert NODE_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 16 and RAY_DTYPE.itemsize == 32

EXPORTED = [
    "rt_api_version", "rt_status_string", "rt_ctx_create", "rt_ctx_destroy", "rt_ctx_set_stream", "rt_ctx_sync",
    "rt_ctx_set_trace_budget", "rt_ctx_set_trace_budget_kind", "rt_ctx_set_heavy_block", "rt_ctx_set_tile_order",
    "rt_ctx_check", "rt_last_error", "rt_lbvh_create", "rt_lbvh_destroy", "rt_lbvh_build", "rt_lbvh_build_host",
    "rt_lbvh_import_host", "rt_lbvh_view_get", "rt_lbvh_compact_get", "rt_lbvh_world_bound", "rt_lbvh_download", "rt_trace_primary",
    "rt_trace_shadow_mirror", "rt_trace_rays", "rt_trace_primary_leaves", "rt_trace_shadow_mirror_from",
    "rt_trace_rays_from", "rt_trace_frame_shader_order", "rt_render_whitted", "rt_bvh_create", "rt_bvh_destroy", "rt_bvh_import_host",
    "rt_bvh_trace_primary", "rt_bvh_trace_shadow_mirror", "rt_bvh_trace_rays", "rt_render_frame_host", "rt_render_frame_host_async", "rt_pathtrace", "rt_pathtrace_counted", "rt_pathtrace_adjoint",
    "rt_lbvh_build_noalloc", "rt_radix_sort_scratch_bytes", "rt_radix_sort", "rt_radix_sort_stall_test",
    "rt_frame_capture_host", "rt_frame_capture", "rt_frame_launch", "rt_frame_node_count", "rt_frame_destroy",
    "rt_pipe_create", "rt_pipe_submit", "rt_pipe_wait", "rt_pipe_destroy",
    "rt_batch_create", "rt_batch_destroy", "rt_batch_scene_count", "rt_batch_build", "rt_batch_view_get",
    "rt_batch_download", "rt_batch_set_views", "rt_batch_trace", "rt_batch_set_tuning", "rt_batch_get_tuning", "rt_batch_frame_capture",
]
RT_BATCH_MAX_SCENES = 256
RT_BATCH_MAX_DEPTH = 23


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3), ("fwd", C.c_float * 3),
                ("tan_half_fovy", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class LbvhView(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("ids", C.c_void_p), ("keys", C.c_void_p), ("sorted_tris", C.c_void_p),
                ("n", C.c_uint32), ("depth", C.c_uint32), ("num_nodes", C.c_uint32), ("node_size", C.c_uint32)]


class BatchTuning(C.Structure):
    _fields_ = [("threads", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("grab", C.c_uint32), ("order", C.c_uint32)]


class Material(C.Structure):
    """rt_material (Structures.hlsl:69-78)."""
    _fields_ = [("ambient", C.c_float * 4), ("diffuse", C.c_float * 4), ("specular", C.c_float * 4),
                ("shininess", C.c_float), ("alpha", C.c_float)]


class ShadeParams(C.Structure):
    """rt_shade_params (cbInputOutput, ConstantBuffers.h:35-70)."""
    _fields_ = [("bounces", C.c_uint32), ("shadows", C.c_int32), ("phong", C.c_int32), ("gloss_mapping", C.c_int32),
                ("env_mapping", C.c_int32), ("env_color", C.c_float * 3), ("seed", C.c_uint32)]


assert C.sizeof(Material) == 56 and C.sizeof(ShadeParams) == 36


class PtParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("bounces", C.c_uint32), ("seed", C.c_uint64), ("sky", C.c_float * 3),
                ("first_sample", C.c_uint32)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not Path(LIB).exists():
        raise RuntimeError(f"{LIB} is missing: build it with __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(str(LIB))
    vp, u32, i32, fp = C.c_void_p, C.c_uint32, C.c_int, C.POINTER(C.c_float)
    sig = {
        "rt_api_version": (i32, []),
        "rt_status_string": (C.c_char_p, [i32]),
        "rt_ctx_create": (i32, [i32, vp, C.POINTER(vp)]),
        "rt_ctx_destroy": (i32, [vp]),
        "rt_ctx_set_stream": (i32, [vp, vp]),
        "rt_ctx_sync": (i32, [vp]),
        "rt_ctx_set_trace_budget": (i32, [vp, u32]),
        "rt_ctx_set_trace_budget_kind": (i32, [vp, u32, u32]),
        "rt_ctx_set_heavy_block": (i32, [vp, u32]),
        "rt_ctx_set_tile_order": (i32, [vp, u32]),
        "rt_ctx_check": (i32, [vp]),
        "rt_last_error": (C.c_char_p, [vp]),
        "rt_lbvh_create": (i32, [vp, u32, u32, C.POINTER(vp)]),
        "rt_lbvh_destroy": (i32, [vp]),
        "rt_lbvh_build": (i32, [vp, vp, vp, u32, u32]),
        "rt_lbvh_build_host": (i32, [vp, vp, vp, u32, u32]),
        "rt_lbvh_import_host": (i32, [vp, vp, vp, vp, vp, u32]),
        "rt_lbvh_view_get": (i32, [vp, C.POINTER(LbvhView)]),
        "rt_lbvh_compact_get": (i32, [vp, C.POINTER(vp), C.POINTER(u32)]),
        "rt_lbvh_world_bound": (i32, [vp, vp, fp]),
        "rt_lbvh_download": (i32, [vp, vp, vp, vp, vp]),
        "rt_trace_primary": (i32, [vp, vp, C.POINTER(Camera), vp, vp]),
        "rt_trace_shadow_mirror": (i32, [vp, vp, C.POINTER(Camera), fp, vp, vp, vp, vp, vp]),
        "rt_trace_rays": (i32, [vp, vp, vp, u32, i32, vp, vp]),
        "rt_trace_primary_leaves": (i32, [vp, vp, C.POINTER(Camera), vp, vp, vp]),
        "rt_trace_shadow_mirror_from": (i32, [vp, vp, C.POINTER(Camera), fp, vp, vp, vp, vp, vp, vp, vp]),
        "rt_trace_rays_from": (i32, [vp, vp, vp, u32, i32, vp, vp, vp, vp]),
        "rt_trace_frame_shader_order": (i32, [vp, vp, C.POINTER(Camera), fp, vp, vp, vp, vp, vp, vp]),
        "rt_render_whitted": (i32, [vp, vp, C.POINTER(Camera), fp, C.POINTER(ShadeParams), vp, vp, u32, vp, vp, vp]),
        "rt_bvh_create": (i32, [vp, u32, u32, C.POINTER(vp)]),
        "rt_bvh_destroy": (i32, [vp]),
        "rt_bvh_import_host": (i32, [vp, vp, vp, u32, vp, vp, u32]),
        "rt_bvh_trace_primary": (i32, [vp, vp, C.POINTER(Camera), vp, vp]),
        "rt_bvh_trace_shadow_mirror": (i32, [vp, vp, C.POINTER(Camera), fp, vp, vp, vp, vp, vp]),
        "rt_bvh_trace_rays": (i32, [vp, vp, vp, u32, i32, vp, vp]),
        "rt_render_frame_host": (i32, [vp, vp, vp, u32, C.POINTER(Camera), fp, vp, vp, vp]),
        "rt_render_frame_host_async": (i32, [vp, vp, vp, u32, C.POINTER(Camera), fp, vp, vp, vp]),
        "rt_pathtrace": (i32, [vp, vp, vp, vp, C.POINTER(Camera), C.POINTER(PtParams), vp]),
        "rt_pathtrace_counted": (i32, [vp, vp, vp, vp, C.POINTER(Camera), C.POINTER(PtParams), vp, vp]),
        "rt_pathtrace_adjoint": (i32, [vp, vp, vp, vp, C.POINTER(Camera), C.POINTER(PtParams), vp, vp, vp]),
        "rt_lbvh_build_noalloc": (i32, [vp, vp, vp, u32, u32, u32, vp, vp, vp, vp]),
        "rt_radix_sort_scratch_bytes": (C.c_size_t, [u32]),
        "rt_radix_sort": (i32, [vp, vp, vp, u32, vp, C.c_size_t]),
        "rt_radix_sort_stall_test": (i32, [vp, vp, vp, u32, vp, C.c_size_t, u32]),
        "rt_frame_capture": (i32, [vp, vp, vp, u32, u32, C.POINTER(Camera), fp, vp, vp, vp, C.POINTER(vp)]),
        "rt_frame_capture_host": (i32, [vp, vp, vp, u32, u32, C.POINTER(Camera), fp, vp, vp, vp, C.POINTER(vp)]),
        "rt_frame_launch": (i32, [vp, vp]),
        "rt_frame_node_count": (u32, [vp]),
        "rt_frame_destroy": (i32, [vp]),
        "rt_pipe_create": (i32, [vp, vp, u32, u32, C.POINTER(Camera), fp, i32, i32, C.POINTER(vp)]),
        "rt_pipe_submit": (i32, [vp, vp, vp, vp, vp, C.POINTER(C.c_uint64)]),
        "rt_pipe_wait": (i32, [vp, C.c_uint64]),
        "rt_pipe_destroy": (i32, [vp]),
        "rt_batch_create": (i32, [vp, u32, vp, u32, C.POINTER(vp)]),
        "rt_batch_destroy": (i32, [vp]),
        "rt_batch_scene_count": (u32, [vp]),
        "rt_batch_build": (i32, [vp, vp, vp, u32]),
        "rt_batch_view_get": (i32, [vp, u32, C.POINTER(LbvhView)]),
        "rt_batch_download": (i32, [vp, vp, u32, vp, vp, vp]),
        "rt_batch_set_views": (i32, [vp, vp, vp, vp]),
        "rt_batch_trace": (i32, [vp, vp, vp, vp]),
        "rt_batch_set_tuning": (i32, [vp, vp, C.POINTER(BatchTuning)]),
        "rt_batch_get_tuning": (i32, [vp, C.POINTER(BatchTuning)]),
        "rt_batch_frame_capture": (i32, [vp, vp, vp, u32, vp, vp, C.POINTER(vp)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class RtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def check(status: int, ctx=None, what: str = "") -> None:
    if status != RT_OK:
        L = lib()
        name = L.rt_status_string(status).decode()
        detail = L.rt_last_error(ctx).decode() if ctx else ""
        raise RtError(status, f"{what}: {name}: {detail}")
