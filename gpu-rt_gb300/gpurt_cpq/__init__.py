"""GB300 closest-point engine (Python binding of include/cpq.h).

Mesh in, BVH built on the GPU, a batch of points in; closest point, unsigned
distance and triangle index out.  See :class:`Mesh`, :class:`Batch` and
:class:`Scene` (instances) and :func:`closest_distance`; the reference's path
tracer on the GPU in :mod:`gpurt_cpq.shading`.
"""
from ._lib import CpError, LIB_PATH, lib  # noqa: F401  (raises if the library is missing)
from . import shading  # noqa: F401
from .gltf import GltfScene, load_gltf  # noqa: F401
from .mesh import (Batch, Mesh, QueryResult, RayResult, Scene, SceneRayResult, SceneResult,  # noqa: F401
                   autotune, autotune_batch, build_opts, closest_distance, query_opts, ray_opts)

__all__ = ["Mesh", "Batch", "Scene", "SceneResult", "SceneRayResult", "QueryResult", "RayResult", "closest_distance", "autotune", "autotune_batch",
           "build_opts",
           "query_opts", "ray_opts", "load_gltf", "GltfScene", "CpError", "lib", "LIB_PATH", "shading"]
