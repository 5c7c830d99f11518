"""ctypes binding of the C ABI in include/cpq.h.

The shared library is built in-tree (``gpu-rt_gb300/build_ext.py``) as
``gpurt_cpq/libgpurt_cpq.so``.  There is no fallback: if it is missing or
fails to load, importing this module raises, so nothing can silently run a CPU
path in its place.
"""
from __future__ import annotations

import ctypes
from ctypes import (POINTER, Structure, c_char_p, c_double, c_float, c_int32, c_int64, c_size_t,
                    c_uint32, c_uint64, c_void_p)
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgpurt_cpq.so"

CP_SUCCESS = 0
CP_ERROR_INVALID_VALUE = 1
CP_ERROR_OUT_OF_MEMORY = 2
CP_ERROR_CUDA = 3
CP_ERROR_DEVICE_FAULT = 4
CP_ERROR_NOT_SUPPORTED = 5
CP_ERROR_SCRATCH_TOO_SMALL = 6

CP_DEVICE_STACK_OVERFLOW = 0x1
CP_DEVICE_BAD_INDEX = 0x2
CP_DEVICE_NONFINITE = 0x4

CP_TIMING_EVENTS = 1
CP_TIMING_COUNTERS = 2

CP_COLLAPSE_COUNT = 0
CP_COLLAPSE_SAH = 1


class BuildOpts(Structure):
    _fields_ = [("branching", c_int32), ("leaf_size", c_int32), ("collapse", c_int32),
                ("sah_node_cost", c_float), ("sah_tri_cost", c_float)]


class QueryOpts(Structure):
    _fields_ = [("block_size", c_int32), ("sort_queries", c_int32), ("blocks_per_sm", c_int32),
                ("short_stack", c_int32), ("traversal", c_int32), ("seed_chunk", c_int32)]


class RayOpts(Structure):
    _fields_ = [("tmin", c_float), ("tmax", c_float), ("det_epsilon", c_float), ("any_hit", c_int32),
                ("sort_rays", c_int32), ("block_size", c_int32)]


class ShadeCamera(Structure):
    _fields_ = [("eye", c_float * 3), ("right", c_float * 3), ("up", c_float * 3), ("fwd", c_float * 3),
                ("tan_half_y", c_float), ("aspect", c_float), ("width", c_int32), ("height", c_int32)]


class ShadeParams(Structure):
    _fields_ = [("clear", c_float * 3), ("env", c_float * 3), ("samples", c_int32), ("max_depth", c_int32),
                ("qmc", c_int32), ("integrator", c_int32), ("brdf", c_int32), ("use_rr", c_int32),
                ("use_metalness", c_int32), ("frame", c_int32), ("max_frame", c_int32),
                ("new_samples", c_int32), ("temporal_multiplier", c_int32), ("use_temporal", c_int32),
                ("debug_view", c_int32), ("seed", c_uint32), ("use_normal_map", c_int32)]


CP_TRAVERSAL_AUTO = 0
CP_TRAVERSAL_THREAD = 1
CP_TRAVERSAL_PACKET = 2


class MeshInfo(Structure):
    _fields_ = [("num_vertices", c_int64), ("num_triangles", c_int64),
                ("num_binary_nodes", c_int64), ("num_wide_nodes", c_int64),
                ("num_leaves", c_int64), ("branching", c_int32), ("leaf_size", c_int32),
                ("max_wide_depth", c_int32), ("stack_bound", c_int32),
                ("device_bytes", c_int64), ("build_ms", c_float)]


# name -> (restype, argtypes); every symbol include/cpq.h declares
SIGNATURES = {
    "cp_build_opts_default": (None, [POINTER(BuildOpts)]),
    "cp_query_opts_default": (None, [POINTER(QueryOpts)]),
    "cp_last_error_string": (c_char_p, []),
    "cp_status_string": (c_char_p, [c_int32]),
    "cp_version": (c_int32, []),
    "cp_kernel_launches": (c_uint64, []),
    "cp_timing_enable": (c_int32, [c_int32]),
    "cp_timing_read": (c_int32, [POINTER(c_double), POINTER(c_int64), c_int32]),
    "cp_probe_read_bandwidth": (c_int32, [c_int64, c_int32, POINTER(c_double), c_void_p]),
    "cp_traversal_stats": (c_int32, [POINTER(c_uint64), c_int32]),
    "cp_mesh_create": (c_int32, [c_void_p, c_int64, c_int64, c_void_p, c_int64, POINTER(BuildOpts),
                                 c_void_p, POINTER(c_void_p)]),
    "cp_mesh_refit": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p]),
    "cp_mesh_destroy": (c_int32, [c_void_p]),
    "cp_mesh_save": (c_int32, [c_void_p, c_char_p]),
    "cp_mesh_load": (c_int32, [c_char_p, c_void_p, POINTER(c_void_p)]),
    "cp_mesh_info": (c_int32, [c_void_p, POINTER(MeshInfo)]),
    "cp_mesh_device_status": (c_int32, [c_void_p, c_void_p, POINTER(c_uint32)]),
    "cp_query_workspace_size": (c_int32, [c_void_p, c_int64, POINTER(QueryOpts), POINTER(c_size_t)]),
    "cp_query": (c_int32, [c_void_p, c_void_p, c_int64, POINTER(QueryOpts), c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "cp_query_host_async": (c_int32, [c_void_p, c_void_p, c_int64, POINTER(QueryOpts), c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "cp_query_host": (c_int32, [c_void_p, c_void_p, c_int64, POINTER(QueryOpts), c_void_p, c_void_p,
                                c_void_p, c_void_p, c_void_p]),
    "cp_query_noalloc": (c_int32, [c_void_p, c_void_p, c_int64, POINTER(QueryOpts), c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p]),
    "cp_query_noalloc_scratch_bytes": (c_size_t, []),
    "cp_backward": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                              c_void_p, c_void_p]),
    "cp_gltf_load": (c_int32, [c_char_p, POINTER(c_void_p)]),
    "cp_gltf_free": (None, [c_void_p]),
    "cp_gltf_primitives": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_void_p), POINTER(c_void_p),
                                     POINTER(c_void_p), POINTER(c_void_p)]),
    "cp_gltf_instances": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_void_p), POINTER(c_void_p)]),
    "cp_gltf_shading": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_void_p), POINTER(c_void_p)]),
    "cp_gltf_textures": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_void_p), POINTER(c_void_p),
                                   POINTER(c_void_p), POINTER(c_int32), POINTER(c_void_p), POINTER(c_int32),
                                   POINTER(c_void_p), POINTER(c_void_p)]),
    "cp_ray_opts_default": (None, [POINTER(RayOpts)]),
    "cp_ray_workspace_size": (c_int32, [c_void_p, c_int64, POINTER(RayOpts), POINTER(c_size_t)]),
    "cp_ray_query": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, POINTER(RayOpts),
                               c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "cp_batch_create": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, POINTER(BuildOpts),
                                  c_void_p, POINTER(c_void_p)]),
    "cp_batch_destroy": (c_int32, [c_void_p]),
    "cp_batch_info": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_int64), POINTER(c_int64),
                                POINTER(c_int32)]),
    "cp_batch_query_workspace_size": (c_int32, [c_void_p, c_int64, POINTER(QueryOpts),
                                                POINTER(c_size_t)]),
    "cp_batch_query": (c_int32, [c_void_p, c_void_p, c_void_p, POINTER(QueryOpts), c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int32,
                                 c_void_p]),
    "cp_batch_save": (c_int32, [c_void_p, c_char_p]),
    "cp_batch_load": (c_int32, [c_char_p, c_void_p, POINTER(c_void_p)]),
    "cp_debug_fail_allocation": (None, [c_int64]),
    "cp_debug_order_sort": (c_int32, [c_void_p, c_int32, c_int64, c_int32, c_int32, c_void_p, c_void_p]),
    "cp_query_order": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "cp_scene_create": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, POINTER(c_void_p)]),
    "cp_scene_update": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "cp_scene_refit": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "cp_scene_destroy": (c_int32, [c_void_p]),
    "cp_scene_ray_workspace_size": (c_int32, [c_void_p, c_int64, POINTER(RayOpts), POINTER(c_size_t)]),
    "cp_scene_ray_query": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, POINTER(RayOpts),
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "cp_scene_query_workspace_size": (c_int32, [c_void_p, c_int64, POINTER(QueryOpts), POINTER(c_size_t)]),
    "cp_scene_query": (c_int32, [c_void_p, c_void_p, c_int64, POINTER(QueryOpts), c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "cp_autotune": (c_int32, [c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64, c_char_p,
                              POINTER(BuildOpts), POINTER(QueryOpts)]),
    "cp_size_class": (c_int32, [c_int64]),
    "cp_batch_autotune": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_int32,
                                    c_char_p, c_void_p, POINTER(QueryOpts)]),
    "cp_batch_create_leaves": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_void_p,
                                         POINTER(BuildOpts), c_void_p, POINTER(c_void_p)]),
    "cp_mesh_export_build": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p]),
    "cp_mesh_export_wide": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "cp_batch_export_build": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
    "cp_batch_export_wide": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "cp_shade_scene_create": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p,
                                        c_int32, c_void_p, POINTER(c_void_p)]),
    "cp_shade_scene_destroy": (c_int32, [c_void_p]),
    "cp_shade_scene_textures": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                                          c_void_p]),
    "cp_shade_scene_lights": (c_int32, [c_void_p, POINTER(c_int32)]),
    "cp_shade_render": (c_int32, [c_void_p, POINTER(ShadeCamera), POINTER(ShadeParams), c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "cp_shade_tonemap": (c_int32, [c_int32, c_float, c_float, c_int64, c_void_p, c_void_p, c_void_p]),
}


class CpError(RuntimeError):
    """A cp_* call returned a status other than CP_SUCCESS."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python gpu-rt_gb300/build_ext.py` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status: int, what: str = "") -> None:
    if status != CP_SUCCESS:
        msg = lib.cp_last_error_string().decode(errors="replace")
        raise CpError(status, f"{what}: {msg}" if what else msg)


__all__ = ["lib", "check", "CpError", "BuildOpts", "QueryOpts", "MeshInfo", "ShadeCamera", "ShadeParams",
           "SIGNATURES", "LIB_PATH"]
