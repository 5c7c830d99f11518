"""ORACLE — test infrastructure only.

ctypes wrapper of oracle/liboracle.so (cpq_oracle.c): the FP64 closest-point
checker and the FP32 CPU restatement of the LBVH build and traversal.  The
same library holds the shading restatement (shade_oracle.c), whose
signatures are registered here and wrapped in oracle/shade.py.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module; the product never does.

Parity unpinned: the reference's closest-point code is absent (its FCPW-GPU
branch, README.md:6-8, is not in the mounted tree); what this restates is
named in cpq_oracle.h.  Hand-computed known answers in tests/golden pin the
FP64 routine.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, Structure, c_double, c_float, c_int, c_int32, c_int64, c_uint8, c_uint64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build() -> Path:
    """Compile liboracle.so with the committed Makefile (gcc, no fast-math)."""
    src = [HERE / n for n in ("cpq_oracle.c", "cpq_oracle.h", "shade_oracle.c", "shade_oracle.h", "Makefile")]
    if LIB.exists() and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB


class OrcTree(Structure):
    _fields_ = [("nt", c_int64), ("nmeshes", c_int32), ("branching", c_int32),
                ("leaf_size", c_int32), ("collapse", c_int32), ("max_wide_depth", c_int32),
                ("stack_bound", c_int32), ("num_wide", c_int64), ("num_leaves", c_int64),
                ("keys", POINTER(c_uint64)), ("order", POINTER(c_int32)),
                ("left", POINTER(c_int32)), ("right", POINTER(c_int32)),
                ("parent", POINTER(c_int32)), ("first", POINTER(c_int32)),
                ("last", POINTER(c_int32)), ("box", POINTER(c_float)), ("cost", POINTER(c_float)),
                ("cluster", POINTER(c_uint8)), ("mesh_root", POINTER(c_int32)),
                ("wide_root", POINTER(c_int32)), ("wide_src", POINTER(c_int32)),
                ("wide_box", POINTER(c_float)), ("wide_ref", POINTER(c_int32)),
                ("wide_count", POINTER(c_int32)), ("tri_verts", POINTER(c_float)),
                ("mesh_of_tri", POINTER(c_int32)), ("tri_local", POINTER(c_int32))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        L.orc_point_tri_f64.restype = c_double
        L.orc_point_tri_f64.argtypes = [c_void_p] * 6
        L.orc_brute_f64.restype = None
        L.orc_brute_f64.argtypes = [c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_exact_f64.restype = c_int
        L.orc_exact_f64.argtypes = [c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_exact_f64_dq.restype = c_int
        L.orc_exact_f64_dq.argtypes = [c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                       c_void_p, c_void_p, c_int]
        L.orc_point_tri_batch_f64.restype = None
        L.orc_point_tri_batch_f64.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                              c_void_p]
        L.orc_build.restype = c_int
        L.orc_build.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int64, c_int64,
                                c_int32, c_int32, c_int32, c_float, c_float, POINTER(POINTER(OrcTree))]
        L.orc_build_leaves.restype = c_int
        L.orc_build_leaves.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int64, c_int64,
                                       c_int32, c_void_p, c_int32, c_float, c_float, POINTER(POINTER(OrcTree))]
        L.orc_tree_free.restype = None
        L.orc_tree_free.argtypes = [POINTER(OrcTree)]
        L.orc_query_f32.restype = c_double
        L.orc_query_f32.argtypes = [POINTER(OrcTree), c_void_p, c_void_p, c_int64, c_void_p,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_backward_f64.restype = None
        L.orc_backward_f64.argtypes = [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_int64, c_void_p, c_void_p]
        L.orc_brute_f64_dv.restype = None
        L.orc_brute_f64_dv.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_void_p,
                                       c_void_p, c_int]
        L.orc_ray_brute_f32.restype = c_double
        L.orc_ray_brute_f32.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int64,
                                        c_float, c_float, c_float, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_ray_brute_f64.restype = c_double
        L.orc_ray_brute_f64.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int64,
                                        c_double, c_double, c_double, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_ray_brute_f64_dv.restype = None
        L.orc_ray_brute_f64_dv.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_double,
                                           c_double, c_void_p, c_void_p, c_void_p, c_int]
        _shade_signatures(L)
        _lib = L
    return _lib


def _shade_signatures(L) -> None:
    """Argument types of the shading restatement (shade_oracle.h)."""
    P = c_void_p
    for name, args, res in [
        ("orc_sh_tea", [c_int64, P, P, P], None),
        ("orc_sh_lcg_stream", [ctypes.c_uint32, c_int64, P, P], None),
        ("orc_sh_radical_inverse", [c_int64, P, P], None),
        ("orc_sh_math", [c_int32, c_int64, P, P, P], None),
        ("orc_sh_sample", [c_int32, c_int64, ctypes.c_uint32, P, c_float, P, P, P], None),
        ("orc_sh_material", [c_int32, c_int64, P, c_float, P, P, P, P, P], None),
        ("orc_sh_triangle_pdf", [c_int64, P, P, P, P], None),
        ("orc_sh_hit_bbox", [c_int64, P, P, P, P, P], None),
        ("orc_sh_make_tanspace", [c_int64, P, P, P], None),
        ("orc_sh_light_pdf", [P, c_int64, P, P, P], None),
        ("orc_sh_render", [P, P, P, P, P, P], c_int),
        ("orc_sh_tonemap", [c_int32, c_float, c_float, c_int64, P, P], c_int),
        ("orc_sh_reservoir_stream", [ctypes.c_uint32, c_int64, P, P, P], None),
    ]:
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def nthreads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def _p(a: np.ndarray | None) -> c_void_p:
    return c_void_p(a.ctypes.data) if a is not None else c_void_p(None)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def point_tri_f64(p, a, b, c):
    """(d2, closest point, barycentrics) of point p and triangle abc in FP64."""
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (p, a, b, c)]
    cp = np.zeros(3)
    w = np.zeros(3)
    d2 = lib().orc_point_tri_f64(*(_p(x) for x in arr), _p(cp), _p(w))
    return d2, cp, w


def brute_f64(verts, tris, q, threads: int | None = None):
    verts, tris, q = _f32(verts), _i32(tris), _f32(q)
    n = q.shape[0]
    d2 = np.empty(n)
    tri = np.empty(n, np.int32)
    p = np.empty((n, 3))
    w = np.empty((n, 3))
    lib().orc_brute_f64(_p(verts), verts.shape[0], _p(tris), tris.shape[0], _p(q), n, _p(d2),
                        _p(tri), _p(p), _p(w), threads or nthreads())
    return {"d2": d2, "dist": np.sqrt(d2), "tri": tri, "point": p, "bary": w}


def exact_f64(verts, tris, q, threads: int | None = None):
    verts, tris, q = _f32(verts), _i32(tris), _f32(q)
    n = q.shape[0]
    d2 = np.empty(n)
    tri = np.empty(n, np.int32)
    p = np.empty((n, 3))
    w = np.empty((n, 3))
    rc = lib().orc_exact_f64(_p(verts), verts.shape[0], _p(tris), tris.shape[0], _p(q), n, _p(d2),
                             _p(tri), _p(p), _p(w), threads or nthreads())
    if rc != 0:
        raise RuntimeError(f"orc_exact_f64 failed ({rc})")
    return {"d2": d2, "dist": np.sqrt(d2), "tri": tri, "point": p, "bary": w}


def exact_f64_dq(verts, tris, q64, threads: int | None = None):
    """FP64 distances for FP64 query points (finite differences)."""
    verts, tris = _f32(verts), _i32(tris)
    q64 = np.ascontiguousarray(q64, dtype=np.float64)
    n = q64.shape[0]
    d2 = np.empty(n)
    tri = np.empty(n, np.int32)
    rc = lib().orc_exact_f64_dq(_p(verts), verts.shape[0], _p(tris), tris.shape[0], _p(q64), n,
                                _p(d2), _p(tri), threads or nthreads())
    if rc != 0:
        raise RuntimeError(f"orc_exact_f64_dq failed ({rc})")
    return np.sqrt(d2), tri


def dist_to_tri_f64(verts, tris, q, tri_idx, want_bary: bool = False):
    """FP64 distance from each query to the given triangle (and its barycentrics)."""
    verts, tris, q, tri_idx = _f32(verts), _i32(tris), _f32(q), _i32(tri_idx)
    out = np.empty(q.shape[0])
    bary = np.empty((q.shape[0], 3)) if want_bary else None
    lib().orc_point_tri_batch_f64(_p(verts), _p(tris), _p(q), _p(tri_idx), q.shape[0], _p(out),
                                  _p(bary))
    return (np.sqrt(out), bary) if want_bary else np.sqrt(out)


class Tree:
    """FP32 CPU restatement of the GPU build (owns the C tree)."""

    def __init__(self, verts, tris, branching=2, leaf_size=4, collapse=0, c_node=1.0, c_tri=1.0,
                 vert_offsets=None, tri_offsets=None, mesh_leaf=None):
        self.verts, self.tris = _f32(verts), _i32(tris)
        self.voff = None if vert_offsets is None else np.ascontiguousarray(vert_offsets, np.int64)
        self.toff = None if tri_offsets is None else np.ascontiguousarray(tri_offsets, np.int64)
        nm = 1 if self.toff is None else len(self.toff) - 1
        ptr = POINTER(OrcTree)()
        if mesh_leaf is None:
            rc = lib().orc_build(_p(self.verts), _p(self.voff), _p(self.tris), _p(self.toff), nm,
                                 self.verts.shape[0], self.tris.shape[0], branching, leaf_size,
                                 collapse, c_node, c_tri, ctypes.byref(ptr))
        else:
            self.mesh_leaf = np.ascontiguousarray(mesh_leaf, np.int32)
            rc = lib().orc_build_leaves(_p(self.verts), _p(self.voff), _p(self.tris), _p(self.toff), nm,
                                        self.verts.shape[0], self.tris.shape[0], branching, _p(self.mesh_leaf),
                                        collapse, c_node, c_tri, ctypes.byref(ptr))
        if rc != 0:
            raise RuntimeError(f"orc_build failed ({rc})")
        self._ptr = ptr
        t = ptr.contents
        n, nn, K, W = t.nt, 2 * t.nt - 1, t.branching, t.num_wide

        def arr(p, count, dtype):
            return np.ctypeslib.as_array(p, shape=(count,)).astype(dtype, copy=True)

        self.nt, self.K, self.num_wide = n, K, W
        self.max_wide_depth, self.stack_bound = t.max_wide_depth, t.stack_bound
        self.num_leaves = t.num_leaves
        self.keys = arr(t.keys, n, np.uint64)
        self.order = arr(t.order, n, np.int32)
        self.left = arr(t.left, max(n - 1, 0), np.int32) if n > 1 else np.empty(0, np.int32)
        self.right = arr(t.right, max(n - 1, 0), np.int32) if n > 1 else np.empty(0, np.int32)
        self.parent = arr(t.parent, nn, np.int32)
        self.first = arr(t.first, nn, np.int32)
        self.last = arr(t.last, nn, np.int32)
        self.box = arr(t.box, 6 * nn, np.float32).reshape(nn, 6)
        self.cost = arr(t.cost, nn, np.float32)
        self.first = arr(t.first, nn, np.int32)
        self.last = arr(t.last, nn, np.int32)
        self.cluster = arr(t.cluster, nn, np.uint8)
        self.mesh_root = arr(t.mesh_root, t.nmeshes, np.int32)
        self.wide_root = arr(t.wide_root, t.nmeshes, np.int32)
        self.wide_src = arr(t.wide_src, W, np.int32)
        self.wide_box = arr(t.wide_box, W * 6 * K, np.float32)
        self.wide_ref = arr(t.wide_ref, W * K, np.int32)
        self.wide_count = arr(t.wide_count, W * K, np.int32)

    def query(self, q, q_mesh=None, threads: int | None = None, stats: bool = False):
        q = _f32(q)
        n = q.shape[0]
        d = np.empty(n, np.float32)
        tri = np.empty(n, np.int32)
        p = np.empty((n, 3), np.float32)
        w = np.empty((n, 2), np.float32)
        nv = np.empty(n, np.int32) if stats else None
        tt = np.empty(n, np.int32) if stats else None
        qm = None if q_mesh is None else _i32(q_mesh)
        secs = lib().orc_query_f32(self._ptr, _p(q), _p(qm), n, _p(d), _p(tri), _p(p), _p(w),
                                   _p(nv), _p(tt), threads or nthreads())
        out = {"dist": d, "tri": tri, "point": p, "bary": w, "seconds": secs}
        if stats:
            out["node_visits"], out["tri_tests"] = nv, tt
        return out

    def close(self):
        if getattr(self, "_ptr", None):
            lib().orc_tree_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def backward_f64(verts, tris, q, tri, bary3, grad):
    verts, tris, q, tri = _f32(verts), _i32(tris), _f32(q), _i32(tri)
    bary3 = np.ascontiguousarray(bary3, np.float64)
    grad = np.ascontiguousarray(grad, np.float64)
    n = q.shape[0]
    gq = np.zeros((n, 3))
    gv = np.zeros((verts.shape[0], 3))
    lib().orc_backward_f64(_p(verts), verts.shape[0], _p(tris), _p(q), _p(tri), _p(bary3), _p(grad),
                           n, _p(gq), _p(gv))
    return gq, gv


def ray_brute(verts, tris, orig, dirs, tmin=0.0, tmax=float("inf"), det_eps=0.0, tmax_per_ray=None,
              fp64=False, threads: int | None = None):
    """Closest hit of every ray over every triangle (Möller–Trumbore of the
    reference's triangle_hit): FP32 as the GPU evaluates it, or FP64."""
    v, t = _f32(verts), _i32(tris)
    o, d = _f32(orig), _f32(dirs)
    n = o.shape[0]
    tm = None if tmax_per_ray is None else _f32(tmax_per_ray)
    dt = np.float64 if fp64 else np.float32
    out_t = np.empty(n, dt)
    out_tri = np.empty(n, np.int32)
    out_uv = np.empty((n, 2), dt)
    fn = lib().orc_ray_brute_f64 if fp64 else lib().orc_ray_brute_f32
    secs = fn(_p(v), _p(t), t.shape[0], _p(o), _p(d), _p(tm), n, tmin, tmax, det_eps, _p(out_t),
              _p(out_tri), _p(out_uv), threads or nthreads())
    return {"t": out_t, "tri": out_tri, "uv": out_uv, "seconds": secs}


def brute_f64_dv(verts64, tris, q, threads: int | None = None):
    """FP64 brute force over FP64 vertices (e.g. instances placed by an FP64 transform)."""
    v = np.ascontiguousarray(verts64, dtype=np.float64)
    t, qq = _i32(tris), _f32(q)
    n = qq.shape[0]
    d2 = np.empty(n)
    tri = np.empty(n, np.int32)
    p = np.empty((n, 3))
    lib().orc_brute_f64_dv(_p(v), _p(t), t.shape[0], _p(qq), n, _p(d2), _p(tri), _p(p), threads or nthreads())
    return {"dist": np.sqrt(d2), "tri": tri, "point": p}


def ray_brute_f64_dv(verts64, tris, orig, dirs, tmin=0.0, tmax=float("inf"), threads: int | None = None):
    """FP64 closest hit of every ray over FP64 vertices (instanced scenes)."""
    v = np.ascontiguousarray(verts64, dtype=np.float64)
    t, o, d = _i32(tris), _f32(orig), _f32(dirs)
    n = o.shape[0]
    out_t = np.empty(n)
    out_tri = np.empty(n, np.int32)
    out_uv = np.empty((n, 2))
    lib().orc_ray_brute_f64_dv(_p(v), _p(t), t.shape[0], _p(o), _p(d), n, tmin, tmax, _p(out_t), _p(out_tri),
                               _p(out_uv), threads or nthreads())
    return {"t": out_t, "tri": out_tri, "uv": out_uv}
