"""CPU tests of the C-ABI library: it loads, exports every entry point that
include/cpq.h declares, and its pure host calls behave.  No compute calls."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "cpq.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"CP_API\s+[\w\s\*]+?\b(cp_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("cp_mesh_create", "cp_query", "cp_backward", "cp_batch_query", "cp_mesh_refit",
                 "cp_autotune", "cp_query_host"):
        assert must in names


def test_library_exports_every_declared_symbol(cpq):
    from gpurt_cpq._lib import SIGNATURES

    lib = ctypes.CDLL(str(cpq.LIB_PATH))
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert name in SIGNATURES, f"{name} has no ctypes signature"


def test_host_only_calls(cpq):
    from ctypes import byref

    from gpurt_cpq._lib import BuildOpts, QueryOpts, lib

    b = BuildOpts()
    lib.cp_build_opts_default(byref(b))
    assert (b.branching, b.leaf_size, b.collapse) == (2, 4, 0)
    q = QueryOpts()
    lib.cp_query_opts_default(byref(q))
    assert q.block_size == 256 and q.sort_queries == 1 and q.short_stack == 8
    assert lib.cp_version() == 100
    assert lib.cp_size_class(2093058) == 20
    assert lib.cp_size_class(1) == 0
    assert lib.cp_status_string(0) == b"success"
    assert lib.cp_status_string(5) == b"not supported"


def test_null_arguments_rejected_without_gpu(cpq):
    from ctypes import byref, c_void_p

    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE, lib

    out = c_void_p()
    st = lib.cp_mesh_create(None, 3, 12, None, 1, None, None, byref(out))
    assert st == CP_ERROR_INVALID_VALUE
    assert b"NULL" in lib.cp_last_error_string()
    assert lib.cp_query(None, None, 0, None, None, None, None, None, None, 0, None) == CP_ERROR_INVALID_VALUE
    assert lib.cp_mesh_destroy(None) == 0


def test_no_gpu_reports_not_supported(cpq):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ctypes import byref, c_void_p

    from gpurt_cpq._lib import CP_ERROR_NOT_SUPPORTED, lib

    out = c_void_p()
    dummy = ctypes.c_float(0)
    st = lib.cp_mesh_create(ctypes.cast(ctypes.pointer(dummy), c_void_p), 3, 12,
                            ctypes.cast(ctypes.pointer(dummy), c_void_p), 1, None, None, byref(out))
    assert st == CP_ERROR_NOT_SUPPORTED


def test_workload_shapes():
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(4)
    assert v.shape == (2562, 3) and t.shape == (5120, 3)
    v, t = W.torus(500, 200)
    assert v.shape == (100000, 3) and t.shape == (200000, 3)
    v, t = W.heightfield(64, seed=1)
    assert t.shape == (2 * 63 * 63, 3)
    assert 2 * 1023 * 1023 == 2093058
    q = W.heightfield_queries(v, t, 1000, seed=2)
    assert q.shape == (1000, 3) and q.dtype.name == "float32"
    a = W.heightfield_queries(v, t, 1000, seed=2)
    assert (a == q).all()
    meshes, queries = W.batched(nmeshes=6, tri_range=(1000, 20000), q_range=(100, 1000))
    assert len(meshes) == 6 and all(1 <= len(x) for x in queries)


def test_argument_checks_of_every_handle_kind(cpq):
    """NULL handles, NULL arrays, empty or inconsistent sizes and unknown flags
    are refused with CP_ERROR_INVALID_VALUE and a message, before any device
    work — for meshes, batches, scenes, rays, glTF files and diagnostics."""
    import numpy as np
    from ctypes import byref, c_size_t, c_uint64, c_void_p

    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE, lib

    def refused(st, text):
        assert st == CP_ERROR_INVALID_VALUE, st
        assert text.encode() in lib.cp_last_error_string(), lib.cp_last_error_string()

    out = c_void_p()
    size = c_size_t()
    some = np.zeros(64, np.float32)
    p = c_void_p(some.ctypes.data)
    # scenes: the batch and both host arrays are required, and instances
    refused(lib.cp_scene_create(None, p, p, 1, None, byref(out)), "NULL")
    refused(lib.cp_scene_create(p, p, p, 0, None, byref(out)), "at least one instance")
    refused(lib.cp_scene_query(None, p, 1, None, None, None, None, None, None, None, 0, None), "scene is NULL")
    refused(lib.cp_scene_ray_query(None, p, p, None, 1, None, None, None, None, None, None, 0, None),
            "scene is NULL")
    refused(lib.cp_scene_update(None, p, None), "NULL")
    refused(lib.cp_scene_query_workspace_size(None, 1, None, byref(size)), "NULL")
    refused(lib.cp_scene_ray_workspace_size(None, 1, None, byref(size)), "NULL")
    assert lib.cp_scene_destroy(None) == 0
    # rays and the no-allocation query on a NULL mesh
    refused(lib.cp_ray_query(None, p, p, None, 1, None, None, None, None, None, 0, None), "mesh")
    refused(lib.cp_query_noalloc(None, p, 1, None, None, None, None, None, None), "mesh is NULL")
    # batches: arrays, mesh count, offsets starting at zero, no empty mesh
    off = np.array([0, 3], np.int64)
    bad_off = np.array([1, 3], np.int64)
    empty = np.array([0, 0], np.int64)
    po, pb, pe = (c_void_p(a.ctypes.data) for a in (off, bad_off, empty))
    refused(lib.cp_batch_create(None, po, p, po, 1, None, None, byref(out)), "NULL")
    refused(lib.cp_batch_create(p, po, p, po, 0, None, None, byref(out)), "nmeshes")
    refused(lib.cp_batch_create(p, pb, p, po, 1, None, None, byref(out)), "start at 0")
    refused(lib.cp_batch_create(p, po, p, pe, 1, None, None, byref(out)), "at least one triangle")
    # glTF and diagnostics
    refused(lib.cp_gltf_load(None, byref(out)), "NULL")
    lib.cp_gltf_free(None)
    refused(lib.cp_timing_enable(4), "unknown flag")
    refused(lib.cp_traversal_stats(None, 0), "NULL")
    counts = (c_uint64 * 7)()
    assert lib.cp_traversal_stats(counts, 0) == 0


def test_python_option_helpers(cpq):
    """The binding's option structs carry what they are given and the
    library's defaults otherwise; unknown names are refused."""
    from gpurt_cpq import mesh as M

    b = cpq.build_opts(branching=8, leaf_size=2, collapse="sah", sah_node_cost=1.5, sah_tri_cost=0.25)
    assert (b.branching, b.leaf_size, b.collapse) == (8, 2, M.CP_COLLAPSE_SAH)
    assert (b.sah_node_cost, b.sah_tri_cost) == (1.5, 0.25)
    assert cpq.build_opts().collapse == M.CP_COLLAPSE_COUNT
    d = cpq.query_opts()
    q = cpq.query_opts(block_size=128, sort_queries=False, short_stack=24, traversal="packet")
    assert (q.block_size, q.sort_queries, q.short_stack, q.traversal) == (128, 0, 24, 2)
    assert (cpq.query_opts(traversal="thread").traversal, d.traversal, d.sort_queries) == (1, 0, 1)
    r = cpq.ray_opts(tmin=1e-5, tmax=1e7, det_epsilon=1e-5, any_hit=True, sort_rays=False)
    assert abs(r.tmin - 1e-5) < 1e-12 and r.tmax == 1e7 and r.any_hit == 1 and r.sort_rays == 0
    with pytest.raises(ValueError, match="collapse"):
        cpq.build_opts(collapse="median")
    with pytest.raises(ValueError, match="traversal"):
        cpq.query_opts(traversal="warp")


def test_scene_transform_shapes():
    """Scene transforms: (n, 3, 4) and (n, 4, 4) give row-major 3 x 4 rows;
    other shapes are refused."""
    import torch
    from gpurt_cpq.mesh import _transforms

    m = np.arange(2 * 16, dtype=np.float64).reshape(2, 4, 4)
    want = m[:, :3, :].reshape(2, 12).astype(np.float32)
    np.testing.assert_array_equal(_transforms(m), want)
    np.testing.assert_array_equal(_transforms(m[:, :3, :]), want)
    np.testing.assert_array_equal(_transforms(torch.from_numpy(m)), want)
    for bad in (m.reshape(2, 16), m[:, :2, :], m[0]):
        with pytest.raises(ValueError):
            _transforms(bad)
