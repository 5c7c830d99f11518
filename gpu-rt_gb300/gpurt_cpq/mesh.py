"""Host-side mirror of the closest-point query surface.

A :class:`Mesh` plays the role of the reference's ``VK::Mesh`` + ``VK::Accel``
pair (src/vk/mesh.h:14-58, src/vk/vulkan.h:256-284): it is built once from
vertices and triangles and then queried; :meth:`Mesh.query` takes the place of
``trace_ray`` (src/shaders/rt/rt.rgen:257-270) with a closest-point query, and
:class:`Batch` the place of the TLAS over many BLASes
(src/vk/vulkan.cpp:777-856).  Every method is a thin call into the C ABI
(include/cpq.h); device tensors are passed as raw pointers on torch's current
CUDA stream.
"""
from __future__ import annotations

from ctypes import byref, c_int32, c_int64, c_size_t, c_uint32, c_void_p
from dataclasses import dataclass

import numpy as np
import torch

from ._lib import (CP_COLLAPSE_COUNT, CP_COLLAPSE_SAH, BuildOpts, MeshInfo, QueryOpts, RayOpts, check,
                   lib)


def _stream(stream=None) -> c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return c_void_p(stream.cuda_stream)


def _ptr(t: torch.Tensor | None) -> c_void_p:
    return c_void_p(t.data_ptr()) if t is not None else c_void_p(None)


def _check_dev(t: torch.Tensor, name: str, dtype, cols: int | None) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if cols is not None and (t.dim() != 2 or t.shape[1] != cols):
        raise ValueError(f"{name} must have shape (N, {cols})")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def build_opts(branching: int = 2, leaf_size: int = 4, collapse: str = "count",
               sah_node_cost: float = 1.0, sah_tri_cost: float = 1.0) -> BuildOpts:
    o = BuildOpts()
    lib.cp_build_opts_default(byref(o))
    o.branching = branching
    o.leaf_size = leaf_size
    modes = {"count": CP_COLLAPSE_COUNT, "sah": CP_COLLAPSE_SAH}
    if collapse not in modes:
        raise ValueError(f"collapse must be one of {sorted(modes)}, not {collapse!r}")
    o.collapse = modes[collapse]
    o.sah_node_cost = sah_node_cost
    o.sah_tri_cost = sah_tri_cost
    return o


def query_opts(block_size: int = 0, sort_queries: bool = True, blocks_per_sm: int = 0,
               short_stack: int = 0, traversal: str = "auto", seed_chunk: int = 0) -> QueryOpts:
    """seed_chunk: packets a warp claims at once, each after the first seeded
    from the previous packet's closest points (1 or 0: no seeding)."""
    o = QueryOpts()
    lib.cp_query_opts_default(byref(o))
    if block_size:
        o.block_size = block_size
    o.sort_queries = 1 if sort_queries else 0
    o.blocks_per_sm = blocks_per_sm
    if short_stack:
        o.short_stack = short_stack
    if seed_chunk:
        o.seed_chunk = seed_chunk
    kinds = {"auto": 0, "thread": 1, "packet": 2}
    if traversal not in kinds:
        raise ValueError(f"traversal must be one of {sorted(kinds)}, not {traversal!r}")
    o.traversal = kinds[traversal]
    return o


def ray_opts(tmin: float = 0.0, tmax: float = float("inf"), det_epsilon: float = 0.0,
             any_hit: bool = False, sort_rays: bool = True, block_size: int = 0) -> RayOpts:
    """cp_ray_opts: hits count for t in [tmin, tmax]; det_epsilon as the reference's
    triangle_hit (1e-5 there); any_hit stops at the first hit (its visibility())."""
    o = RayOpts()
    lib.cp_ray_opts_default(byref(o))
    o.tmin, o.tmax, o.det_epsilon = tmin, tmax, det_epsilon
    o.any_hit = 1 if any_hit else 0
    o.sort_rays = 1 if sort_rays else 0
    if block_size:
        o.block_size = block_size
    return o


@dataclass
class RayResult:
    t: torch.Tensor     # (N,) float32, +inf on a miss
    tri: torch.Tensor   # (N,) int32, -1 on a miss
    uv: torch.Tensor | None  # (N, 2) float32: weights of vertices 1 and 2 at the hit


@dataclass
class QueryResult:
    point: torch.Tensor | None   # (N, 3) float32
    dist: torch.Tensor           # (N,) float32
    tri: torch.Tensor            # (N,) int32
    bary: torch.Tensor | None    # (N, 2) float32, weights of vertices 1 and 2


class Mesh:
    """A triangle mesh with a GPU-built BVH (see include/cpq.h, cp_mesh_create)."""

    def __init__(self, verts: torch.Tensor, tris: torch.Tensor, *, branching: int = 2,
                 leaf_size: int = 4, collapse: str = "count", sah_node_cost: float = 1.0,
                 sah_tri_cost: float = 1.0, stream=None):
        if verts.dim() != 2 or verts.shape[1] < 3:
            raise ValueError("verts must have shape (V, >=3)")
        if not verts.is_cuda or verts.dtype != torch.float32 or verts.stride(1) != 1:
            raise ValueError("verts must be a CUDA float32 tensor with unit column stride")
        _check_dev(tris, "tris", torch.int32, 3)
        self.num_vertices = int(verts.shape[0])
        self.num_triangles = int(tris.shape[0])
        self.opts = build_opts(branching, leaf_size, collapse, sah_node_cost, sah_tri_cost)
        h = c_void_p()
        check(lib.cp_mesh_create(_ptr(verts), self.num_vertices, verts.stride(0) * 4, _ptr(tris),
                                 self.num_triangles, byref(self.opts), _stream(stream), byref(h)),
              "cp_mesh_create")
        self._h = h
        self.device = verts.device

    # -- saved BVHs -------------------------------------------------------------
    def save(self, path) -> None:
        """Write the built BVH to `path` (cp_mesh_save)."""
        check(lib.cp_mesh_save(self._h, str(path).encode()), "cp_mesh_save")

    @classmethod
    def load(cls, path, *, device=None, stream=None) -> "Mesh":
        """A mesh read from a file cp_mesh_save wrote, without a build (cp_mesh_load)."""
        h = c_void_p()
        check(lib.cp_mesh_load(str(path).encode(), _stream(stream), byref(h)), "cp_mesh_load")
        m = cls.__new__(cls)
        m._h = h
        info = m.info()
        m.num_vertices = int(info.num_vertices)
        m.num_triangles = int(info.num_triangles)
        m.opts = build_opts(info.branching, info.leaf_size)
        m.device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        return m

    # -- lifetime ------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib.cp_mesh_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> c_void_p:
        return self._h

    def info(self) -> MeshInfo:
        out = MeshInfo()
        check(lib.cp_mesh_info(self._h, byref(out)), "cp_mesh_info")
        return out

    def device_status(self, stream=None) -> int:
        bits = c_uint32(0)
        check(lib.cp_mesh_device_status(self._h, _stream(stream), byref(bits)), "cp_mesh_device_status")
        return bits.value

    def query_order(self, points: torch.Tensor, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        """(perm, keys): the order cp_query with sort_queries walks these
        queries in (perm[i] = the input index of the i-th) and each query's
        Hilbert key in input order (int64, values below 2^30)."""
        _check_dev(points, "points", torch.float32, 3)
        n = points.shape[0]
        perm = torch.empty(n, dtype=torch.int32, device=points.device)
        keys = torch.empty(n, dtype=torch.int32, device=points.device)
        check(lib.cp_query_order(self._h, _ptr(points), n, _ptr(perm), _ptr(keys), _stream(stream)),
              "cp_query_order")
        return perm, keys.to(torch.int64) & 0xFFFFFFFF

    # -- queries -------------------------------------------------------------
    def workspace_size(self, nq: int, opts: QueryOpts | None = None) -> int:
        b = c_size_t(0)
        o = opts or query_opts()
        check(lib.cp_query_workspace_size(self._h, nq, byref(o), byref(b)), "cp_query_workspace_size")
        return b.value

    def query(self, points: torch.Tensor, *, want_point: bool = True, want_bary: bool = False,
              opts: QueryOpts | None = None, workspace: torch.Tensor | None = None,
              out: QueryResult | None = None, stream=None) -> QueryResult:
        _check_dev(points, "points", torch.float32, 3)
        n = int(points.shape[0])
        o = opts or query_opts()
        if out is None:
            dev = points.device
            out = QueryResult(
                point=torch.empty((n, 3), dtype=torch.float32, device=dev) if want_point else None,
                dist=torch.empty((n,), dtype=torch.float32, device=dev),
                tri=torch.empty((n,), dtype=torch.int32, device=dev),
                bary=torch.empty((n, 2), dtype=torch.float32, device=dev) if want_bary else None)
        ws_ptr, ws_bytes = c_void_p(None), 0
        if workspace is not None:
            ws_ptr, ws_bytes = c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
        check(lib.cp_query(self._h, _ptr(points), n, byref(o), _ptr(out.point), _ptr(out.dist),
                           _ptr(out.tri), _ptr(out.bary), ws_ptr, ws_bytes, _stream(stream)),
              "cp_query")
        return out

    def ray_query(self, origins: torch.Tensor, directions: torch.Tensor, *,
                  tmax_per_ray: torch.Tensor | None = None, opts: RayOpts | None = None,
                  want_uv: bool = True, stream=None) -> RayResult:
        """Closest (or, with opts.any_hit, some) hit of each ray (cp_ray_query)."""
        _check_dev(origins, "origins", torch.float32, 3)
        _check_dev(directions, "directions", torch.float32, 3)
        n = int(origins.shape[0])
        if directions.shape[0] != n:
            raise ValueError("origins and directions must have the same length")
        if tmax_per_ray is not None and (not tmax_per_ray.is_cuda or tmax_per_ray.dtype != torch.float32
                                         or tmax_per_ray.numel() != n):
            raise ValueError("tmax_per_ray must be a CUDA float32 tensor of one value per ray")
        o = opts or ray_opts()
        dev = origins.device
        out = RayResult(t=torch.empty((n,), dtype=torch.float32, device=dev),
                        tri=torch.empty((n,), dtype=torch.int32, device=dev),
                        uv=torch.empty((n, 2), dtype=torch.float32, device=dev) if want_uv else None)
        tm = tmax_per_ray.contiguous() if tmax_per_ray is not None else None
        check(lib.cp_ray_query(self._h, _ptr(origins), _ptr(directions), _ptr(tm), n, byref(o),
                               _ptr(out.t), _ptr(out.tri), _ptr(out.uv), c_void_p(None), 0, _stream(stream)),
              "cp_ray_query")
        return out

    def query_host(self, points: np.ndarray | torch.Tensor, *, want_point: bool = True,
                   want_bary: bool = False, opts: QueryOpts | None = None,
                   out: dict | None = None) -> dict:
        """Host arrays in and out (pinned torch CPU tensors give full copy speed)."""
        if isinstance(points, np.ndarray):
            points = torch.from_numpy(np.ascontiguousarray(points, dtype=np.float32))
        if points.is_cuda or points.dtype != torch.float32 or not points.is_contiguous():
            raise ValueError("points must be a contiguous float32 CPU tensor")
        n = int(points.shape[0])
        pin = points.is_pinned()
        if out is None:
            out = {"dist": torch.empty((n,), dtype=torch.float32, pin_memory=pin),
                   "tri": torch.empty((n,), dtype=torch.int32, pin_memory=pin)}
            if want_point:
                out["point"] = torch.empty((n, 3), dtype=torch.float32, pin_memory=pin)
            if want_bary:
                out["bary"] = torch.empty((n, 2), dtype=torch.float32, pin_memory=pin)
        o = opts or query_opts()
        check(lib.cp_query_host(self._h, _ptr(points), n, byref(o), _ptr(out.get("point")),
                                _ptr(out["dist"]), _ptr(out["tri"]), _ptr(out.get("bary")),
                                _stream()), "cp_query_host")
        return out

    def query_host_async(self, points: torch.Tensor, out: dict, *, opts: QueryOpts | None = None,
                         stream=None) -> dict:
        """cp_query_host_async: pinned host tensors in and out, enqueued on
        `stream` (default: the current stream); the outputs are ready when the
        stream has reached this call.  `out` holds "dist", "tri" and
        optionally "point" and "bary"."""
        if points.is_cuda or points.dtype != torch.float32 or not points.is_contiguous():
            raise ValueError("points must be a contiguous float32 CPU tensor")
        o = opts or query_opts()
        check(lib.cp_query_host_async(self._h, _ptr(points), int(points.shape[0]), byref(o),
                                      _ptr(out.get("point")), _ptr(out["dist"]), _ptr(out["tri"]),
                                      _ptr(out.get("bary")), _stream(stream)), "cp_query_host_async")
        return out

    def refit(self, verts: torch.Tensor, stream=None) -> None:
        if not verts.is_cuda or verts.dtype != torch.float32 or verts.shape[0] != self.num_vertices:
            raise ValueError("verts must be a CUDA float32 tensor with the mesh's vertex count")
        check(lib.cp_mesh_refit(self._h, _ptr(verts), verts.stride(0) * 4, _stream(stream)),
              "cp_mesh_refit")

    def backward(self, points: torch.Tensor, tri: torch.Tensor, bary: torch.Tensor | None,
                 grad_dist: torch.Tensor, *, need_points: bool = True, need_verts: bool = True,
                 grad_verts: torch.Tensor | None = None, stream=None):
        """Adjoint (cp_backward).  bary=None recomputes the exact barycentrics."""
        _check_dev(points, "points", torch.float32, 3)
        n = int(points.shape[0])
        grad_dist = grad_dist.contiguous().to(torch.float32)
        gq = torch.empty((n, 3), dtype=torch.float32, device=points.device) if need_points else None
        if need_verts and grad_verts is None:
            grad_verts = torch.zeros((self.num_vertices, 3), dtype=torch.float32, device=points.device)
        bary = bary.contiguous() if bary is not None else None
        check(lib.cp_backward(self._h, _ptr(points), _ptr(tri.contiguous()), _ptr(bary),
                              _ptr(grad_dist), n, _ptr(gq), _ptr(grad_verts if need_verts else None),
                              _stream(stream)), "cp_backward")
        return gq, (grad_verts if need_verts else None)

    # -- inspection ----------------------------------------------------------
    def export_build(self) -> dict:
        return _export_build(lib.cp_mesh_export_build, self._h, self.num_triangles,
                             self.info().num_wide_nodes)

    def export_wide(self) -> dict:
        info = self.info()
        return _export_wide(lib.cp_mesh_export_wide, self._h, info.branching, info.num_wide_nodes)


def _export_build(fn, handle, n: int, num_wide: int) -> dict:
    """The build's intermediate arrays (cp_mesh_export_build / cp_batch_export_build)."""
    out = {"keys": np.empty(n, np.uint64), "order": np.empty(n, np.int32),
           "left": np.empty(max(n - 1, 1), np.int32), "right": np.empty(max(n - 1, 1), np.int32),
           "parent": np.empty(2 * n - 1, np.int32), "cluster": np.empty(2 * n - 1, np.uint8),
           "wide_src": np.empty(num_wide, np.int32)}
    check(fn(handle, *(c_void_p(out[k].ctypes.data) for k in
                       ("keys", "order", "left", "right", "parent", "cluster", "wide_src"))), "export")
    if n == 1:
        out["left"] = out["left"][:0]
        out["right"] = out["right"][:0]
    return out


def _export_wide(fn, handle, K: int, w: int) -> dict:
    """Wide-node boxes, child refs and counts (cp_mesh_export_wide / cp_batch_export_wide)."""
    out = {"boxes": np.empty(w * 6 * K, np.float32), "refs": np.empty(w * K, np.int32),
           "counts": np.empty(w * K, np.int32)}
    check(fn(handle, c_void_p(out["boxes"].ctypes.data), c_void_p(out["refs"].ctypes.data),
             c_void_p(out["counts"].ctypes.data)), "export")
    return out


class Batch:
    """Many meshes with one batched build and one persistent query launch."""

    def __init__(self, verts: torch.Tensor, vert_offsets, tris: torch.Tensor, tri_offsets, *,
                 branching: int = 2, leaf_size: int = 4, collapse: str = "count", leaf_sizes=None,
                 stream=None):
        """leaf_sizes (one per mesh, e.g. from autotune_batch) replaces leaf_size
        mesh by mesh (cp_batch_create_leaves)."""
        _check_dev(verts, "verts", torch.float32, 3)
        _check_dev(tris, "tris", torch.int32, 3)
        self.vert_offsets = np.ascontiguousarray(vert_offsets, dtype=np.int64)
        self.tri_offsets = np.ascontiguousarray(tri_offsets, dtype=np.int64)
        self.nmeshes = len(self.tri_offsets) - 1
        self.opts = build_opts(branching, leaf_size, collapse)
        h = c_void_p()
        if leaf_sizes is None:
            self.leaf_sizes = None
            check(lib.cp_batch_create(_ptr(verts), c_void_p(self.vert_offsets.ctypes.data), _ptr(tris),
                                      c_void_p(self.tri_offsets.ctypes.data), self.nmeshes,
                                      byref(self.opts), _stream(stream), byref(h)), "cp_batch_create")
        else:
            self.leaf_sizes = np.ascontiguousarray(leaf_sizes, dtype=np.int32)
            if self.leaf_sizes.shape != (self.nmeshes,):
                raise ValueError("leaf_sizes needs one value per mesh")
            check(lib.cp_batch_create_leaves(_ptr(verts), c_void_p(self.vert_offsets.ctypes.data), _ptr(tris),
                                             c_void_p(self.tri_offsets.ctypes.data), self.nmeshes,
                                             c_void_p(self.leaf_sizes.ctypes.data), byref(self.opts),
                                             _stream(stream), byref(h)), "cp_batch_create_leaves")
        self._h = h

    def save(self, path) -> None:
        """Write the built batch to a file (cp_batch_save)."""
        check(lib.cp_batch_save(self._h, str(path).encode()), "cp_batch_save")

    @classmethod
    def load(cls, path, *, stream=None) -> "Batch":
        """A batch read from a file cp_batch_save (or cp_mesh_save, as a batch
        of one) wrote, without a build (cp_batch_load)."""
        h = c_void_p()
        check(lib.cp_batch_load(str(path).encode(), _stream(stream), byref(h)), "cp_batch_load")
        b = cls.__new__(cls)
        b._h = h
        b.nmeshes = int(b.info()["nmeshes"])
        # the build's branching, leaf size and collapse from the file's header
        k, leaf, collapse = np.fromfile(str(path), dtype=np.int32, count=5)[2:5]
        b.opts = build_opts(int(k), int(leaf), "sah" if collapse == CP_COLLAPSE_SAH else "count")
        b.vert_offsets = b.tri_offsets = b.leaf_sizes = None
        return b

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib.cp_batch_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        nm, nw, ntri, sb = c_int32(), c_int64(), c_int64(), c_int32()
        check(lib.cp_batch_info(self._h, byref(nm), byref(nw), byref(ntri), byref(sb)), "cp_batch_info")
        return {"nmeshes": nm.value, "num_wide_nodes": nw.value, "num_triangles": ntri.value,
                "stack_bound": sb.value}

    def workspace_size(self, nq: int, opts: QueryOpts | None = None) -> int:
        b = c_size_t(0)
        o = opts or query_opts()
        check(lib.cp_batch_query_workspace_size(self._h, nq, byref(o), byref(b)), "workspace")
        return b.value

    def export_build(self) -> dict:
        info = self.info()
        return _export_build(lib.cp_batch_export_build, self._h, info["num_triangles"],
                             info["num_wide_nodes"])

    def export_wide(self) -> dict:
        return _export_wide(lib.cp_batch_export_wide, self._h, self.opts.branching,
                            self.info()["num_wide_nodes"])

    def query(self, points: torch.Tensor, q_offsets, *, want_point: bool = True,
              want_bary: bool = False, opts: QueryOpts | None = None,
              workspace: torch.Tensor | None = None, use_graph: bool = False,
              out: QueryResult | None = None, stream=None) -> QueryResult:
        _check_dev(points, "points", torch.float32, 3)
        qoff = np.ascontiguousarray(q_offsets, dtype=np.int64)
        n = int(points.shape[0])
        if int(qoff[-1]) != n:
            raise ValueError("q_offsets[-1] must equal the number of points")
        o = opts or query_opts()
        if out is None:
            dev = points.device
            out = QueryResult(
                point=torch.empty((n, 3), dtype=torch.float32, device=dev) if want_point else None,
                dist=torch.empty((n,), dtype=torch.float32, device=dev),
                tri=torch.empty((n,), dtype=torch.int32, device=dev),
                bary=torch.empty((n, 2), dtype=torch.float32, device=dev) if want_bary else None)
        ws_ptr, ws_bytes = c_void_p(None), 0
        if workspace is not None:
            ws_ptr, ws_bytes = c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
        check(lib.cp_batch_query(self._h, _ptr(points), c_void_p(qoff.ctypes.data), byref(o),
                                 _ptr(out.point), _ptr(out.dist), _ptr(out.tri), _ptr(out.bary),
                                 ws_ptr, ws_bytes, 1 if use_graph else 0, _stream(stream)),
              "cp_batch_query")
        return out


@dataclass
class SceneResult:
    point: torch.Tensor | None   # (N, 3) float32, world space
    dist: torch.Tensor           # (N,) float32, world units
    instance: torch.Tensor       # (N,) int32
    tri: torch.Tensor            # (N,) int32, local to the instance's mesh
    bary: torch.Tensor | None    # (N, 2) float32


@dataclass
class SceneRayResult:
    t: torch.Tensor          # (N,) float32, +inf on a miss
    instance: torch.Tensor   # (N,) int32, -1 on a miss
    tri: torch.Tensor        # (N,) int32, local to the instance's mesh
    uv: torch.Tensor | None  # (N, 2) float32


def _transforms(transforms) -> np.ndarray:
    """(n, 3, 4) or (n, 4, 4) object-to-world matrices -> (n, 12) float32 row-major 3 x 4."""
    t = np.asarray(transforms.cpu() if isinstance(transforms, torch.Tensor) else transforms)
    if t.ndim != 3 or t.shape[1:] not in ((3, 4), (4, 4)):
        raise ValueError("transforms must be (n, 3, 4) or (n, 4, 4)")
    return np.ascontiguousarray(t[:, :3, :4].reshape(-1, 12), dtype=np.float32)


class Scene:
    """Instances of a batch's meshes placed by affine transforms
    (cp_scene_create); queries are in world space.  Keeps the batch alive."""

    def __init__(self, batch: Batch, instance_mesh, transforms, *, stream=None):
        self.batch = batch
        self.instance_mesh = np.ascontiguousarray(instance_mesh, dtype=np.int32)
        t = _transforms(transforms)
        if len(t) != len(self.instance_mesh):
            raise ValueError("one transform per instance")
        self.n = len(t)
        h = c_void_p()
        check(lib.cp_scene_create(batch._h, c_void_p(self.instance_mesh.ctypes.data), c_void_p(t.ctypes.data),
                                  self.n, _stream(stream), byref(h)), "cp_scene_create")
        self._h = h

    def update(self, transforms, *, stream=None) -> None:
        t = _transforms(transforms)
        if len(t) != self.n:
            raise ValueError("one transform per instance")
        check(lib.cp_scene_update(self._h, c_void_p(t.ctypes.data), _stream(stream)), "cp_scene_update")

    def refit(self, transforms, *, stream=None) -> None:
        """New transforms keeping the trees' topology (cp_scene_refit): the
        TLAS update of the reference, where update() is its rebuild."""
        t = _transforms(transforms)
        if len(t) != self.n:
            raise ValueError("one transform per instance")
        check(lib.cp_scene_refit(self._h, c_void_p(t.ctypes.data), _stream(stream)), "cp_scene_refit")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib.cp_scene_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def workspace_size(self, nq: int, opts: QueryOpts | None = None) -> int:
        b = c_size_t(0)
        o = opts or query_opts()
        check(lib.cp_scene_query_workspace_size(self._h, nq, byref(o), byref(b)), "workspace")
        return b.value

    def ray_query(self, origins: torch.Tensor, directions: torch.Tensor, *,
                  tmax_per_ray: torch.Tensor | None = None, opts: RayOpts | None = None,
                  want_uv: bool = True, stream=None) -> SceneRayResult:
        """Closest (or any) hit of each world-space ray (cp_scene_ray_query)."""
        _check_dev(origins, "origins", torch.float32, 3)
        _check_dev(directions, "directions", torch.float32, 3)
        n = int(origins.shape[0])
        if directions.shape[0] != n:
            raise ValueError("origins and directions must have the same length")
        if tmax_per_ray is not None and (not tmax_per_ray.is_cuda or tmax_per_ray.dtype != torch.float32
                                         or tmax_per_ray.numel() != n or not tmax_per_ray.is_contiguous()):
            raise ValueError("tmax_per_ray must be a contiguous CUDA float32 tensor of one value per ray")
        dev = origins.device
        out = SceneRayResult(t=torch.empty((n,), dtype=torch.float32, device=dev),
                             instance=torch.empty((n,), dtype=torch.int32, device=dev),
                             tri=torch.empty((n,), dtype=torch.int32, device=dev),
                             uv=torch.empty((n, 2), dtype=torch.float32, device=dev) if want_uv else None)
        o = opts or ray_opts()
        check(lib.cp_scene_ray_query(self._h, _ptr(origins), _ptr(directions), _ptr(tmax_per_ray), n, byref(o),
                                     _ptr(out.t), _ptr(out.instance), _ptr(out.tri), _ptr(out.uv),
                                     c_void_p(None), 0, _stream(stream)), "cp_scene_ray_query")
        return out

    def query(self, points: torch.Tensor, *, want_point: bool = True, want_bary: bool = False,
              opts: QueryOpts | None = None, workspace: torch.Tensor | None = None,
              stream=None) -> SceneResult:
        _check_dev(points, "points", torch.float32, 3)
        n = int(points.shape[0])
        dev = points.device
        out = SceneResult(
            point=torch.empty((n, 3), dtype=torch.float32, device=dev) if want_point else None,
            dist=torch.empty((n,), dtype=torch.float32, device=dev),
            instance=torch.empty((n,), dtype=torch.int32, device=dev),
            tri=torch.empty((n,), dtype=torch.int32, device=dev),
            bary=torch.empty((n, 2), dtype=torch.float32, device=dev) if want_bary else None)
        o = opts or query_opts()
        ws_ptr, ws_bytes = c_void_p(None), 0
        if workspace is not None:
            ws_ptr, ws_bytes = c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
        check(lib.cp_scene_query(self._h, _ptr(points), n, byref(o), _ptr(out.point), _ptr(out.dist),
                                 _ptr(out.instance), _ptr(out.tri), _ptr(out.bary), ws_ptr, ws_bytes,
                                 _stream(stream)), "cp_scene_query")
        return out


def autotune_batch(verts: torch.Tensor, vert_offsets, tris: torch.Tensor, tri_offsets, queries: torch.Tensor,
                   q_offsets, branching: int = 4, cache_path: str | None = None):
    """Run cp_batch_autotune: a leaf size per mesh, chosen per size class
    (floor(log2(triangles))) by timing each class's own meshes and queries.
    Returns (leaf_sizes, QueryOpts)."""
    _check_dev(verts, "verts", torch.float32, 3)
    _check_dev(tris, "tris", torch.int32, 3)
    _check_dev(queries, "queries", torch.float32, 3)
    voff = np.ascontiguousarray(vert_offsets, dtype=np.int64)
    toff = np.ascontiguousarray(tri_offsets, dtype=np.int64)
    qoff = np.ascontiguousarray(q_offsets, dtype=np.int64)
    leaves = np.zeros(len(toff) - 1, np.int32)
    qo = QueryOpts()
    torch.cuda.synchronize()
    check(lib.cp_batch_autotune(_ptr(verts), c_void_p(voff.ctypes.data), _ptr(tris), c_void_p(toff.ctypes.data),
                                len(toff) - 1, _ptr(queries), c_void_p(qoff.ctypes.data), branching,
                                cache_path.encode() if cache_path else None, c_void_p(leaves.ctypes.data),
                                byref(qo)), "cp_batch_autotune")
    return leaves, qo


def autotune(verts: torch.Tensor, tris: torch.Tensor, sample: torch.Tensor,
             cache_path: str | None = None, branching: int = 0):
    """Run cp_autotune; returns (BuildOpts, QueryOpts).  branching=2/4/8 fixes the width."""
    _check_dev(verts, "verts", torch.float32, 3)
    _check_dev(tris, "tris", torch.int32, 3)
    _check_dev(sample, "sample", torch.float32, 3)
    bo, qo = BuildOpts(), QueryOpts()
    bo.branching = branching
    torch.cuda.synchronize()
    check(lib.cp_autotune(_ptr(verts), verts.shape[0], _ptr(tris), tris.shape[0], _ptr(sample),
                          sample.shape[0], cache_path.encode() if cache_path else None, byref(bo),
                          byref(qo)), "cp_autotune")
    return bo, qo


class _ClosestDistance(torch.autograd.Function):
    """Unsigned distance with a hand-written adjoint (cp_backward).

    The forward keeps only the winning triangle index and its barycentrics;
    the backward recomputes the closest point from them instead of storing
    traversal state.
    """

    @staticmethod
    def forward(ctx, points, verts, mesh: Mesh):
        res = mesh.query(points.detach().contiguous(), want_point=False, want_bary=True)
        ctx.mesh = mesh
        ctx.save_for_backward(points.detach().contiguous(), res.tri, res.bary)
        ctx.mark_non_differentiable(res.tri)
        return res.dist, res.tri

    @staticmethod
    def backward(ctx, grad_dist, _grad_tri):
        points, tri, bary = ctx.saved_tensors
        need_q, need_v = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if grad_dist is None or not (need_q or need_v):
            return None, None, None
        gq, gv = ctx.mesh.backward(points, tri, bary, grad_dist, need_points=need_q,
                                   need_verts=need_v)
        return gq, gv, None


def closest_distance(points: torch.Tensor, mesh: Mesh, verts: torch.Tensor | None = None):
    """Differentiable unsigned distance from each point to the mesh.

    ``verts`` is the (V, 3) tensor the mesh was built from (or refitted to);
    pass it with ``requires_grad`` to receive d(distance)/d(vertices).
    Returns (dist, tri).
    """
    if verts is None:
        verts = torch.empty((mesh.num_vertices, 3), device=points.device)
    return _ClosestDistance.apply(points, verts, mesh)
