"""CPU tests of the C-ABI library: it loads, exports every entry point that
include/cpq.h declares, and its pure host calls behave.  No compute calls."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

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
