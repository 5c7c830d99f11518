"""cp_query_noalloc: the query for callers that may not allocate device memory.

Render or simulation loops that forbid allocation after start-up, plugins
whose host owns all device memory, and code running under a lock of its own
allocator cannot let a query call cudaMalloc.  cp_query_noalloc takes its
scratch from a fixed array inside the library instead.  These tests call it
through the C ABI: a zero-count call first, which loads the array on the
device as a caller does at start-up; then results against cp_query, the
regular entry point, on two calls in a row (the second call must not see the
first call's leftovers in the shared array); then the same call while the
library's allocator is set to fail, which cp_query cannot survive; and the
refusals: more than 1,048,576 ordered queries (before anything launches) and
more than 2^31 - 1 queries.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

from ctypes import byref, c_void_p

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6  # the distance tolerance the other GPU tests use


def _ptr(t):
    return c_void_p(t.data_ptr()) if t is not None else c_void_p(None)


def _run(lib, fn, mesh, q, opts, torch):
    n = q.shape[0]
    point = torch.empty((n, 3), dtype=torch.float32, device=q.device)
    dist = torch.empty(n, dtype=torch.float32, device=q.device)
    tri = torch.empty(n, dtype=torch.int32, device=q.device)
    bary = torch.empty((n, 2), dtype=torch.float32, device=q.device)
    stream = c_void_p(torch.cuda.current_stream().cuda_stream)
    if fn == "cp_query":
        st = lib.cp_query(mesh.handle, _ptr(q), n, byref(opts), _ptr(point), _ptr(dist), _ptr(tri),
                          _ptr(bary), None, 0, stream)
    else:
        st = lib.cp_query_noalloc(mesh.handle, _ptr(q), n, byref(opts), _ptr(point), _ptr(dist),
                                  _ptr(tri), _ptr(bary), stream)
    torch.cuda.synchronize()
    return st, point, dist, tri, bary


def _same(torch, a, b):
    _, pa, da, ta, ba = a
    _, pb, db, tb, bb = b
    rel = ((da.double() - db.double()).abs() / db.double().clamp_min(1e-30)).max()
    assert float(rel) <= REL_TOL
    assert torch.equal(ta, tb)
    assert float((pa - pb).abs().max()) <= 1e-6
    assert float((ba - bb).abs().max()) <= 1e-6


def _load_array(lib, mesh, torch):
    """The start-up call: a zero count loads the fixed array and runs nothing."""
    st = lib.cp_query_noalloc(mesh.handle, None, 0, None, None, None, None, None,
                              c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.cp_last_error_string()


def test_noalloc_matches_cp_query_on_two_calls(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import lib

    v, t = W.heightfield(256, seed=5)
    mesh = cpq.Mesh(torch.from_numpy(v).to(cuda), torch.from_numpy(t).to(cuda), branching=4)
    q1 = torch.from_numpy(W.heightfield_queries(v, t, 300_000, seed=6)).to(cuda)
    q2 = torch.from_numpy(W.uniform_queries(200_000, -0.2, 1.2, 7)).to(cuda)
    _load_array(lib, mesh, torch)
    for sort in (True, False):
        opts = cpq.query_opts(sort_queries=sort)
        for q in (q1, q2):  # two calls in a row through the shared scratch array
            ref = _run(lib, "cp_query", mesh, q, opts, torch)
            got = _run(lib, "cp_query_noalloc", mesh, q, opts, torch)
            assert ref[0] == 0 and got[0] == 0, lib.cp_last_error_string()
            _same(torch, got, ref)
    assert mesh.device_status() == 0


def test_noalloc_allocates_nothing(cpq, cuda):
    """With the library's next device allocation set to fail, cp_query without
    a workspace fails for lack of memory, and cp_query_noalloc still answers,
    equal to cp_query's answers from before."""
    import torch

    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_ERROR_OUT_OF_MEMORY, lib

    v, t = W.heightfield(128, seed=9)
    mesh = cpq.Mesh(torch.from_numpy(v).to(cuda), torch.from_numpy(t).to(cuda), branching=4)
    q = torch.from_numpy(W.heightfield_queries(v, t, 100_000, seed=10)).to(cuda)
    opts = cpq.query_opts()
    ref = _run(lib, "cp_query", mesh, q, opts, torch)
    assert ref[0] == 0
    _load_array(lib, mesh, torch)
    try:
        for _ in range(2):
            lib.cp_debug_fail_allocation(0)  # the library's next device allocation fails
            got = _run(lib, "cp_query_noalloc", mesh, q, opts, torch)
            assert got[0] == 0, lib.cp_last_error_string()
            _same(torch, got, ref)
            failed = _run(lib, "cp_query", mesh, q, opts, torch)  # allocates its workspace
            assert failed[0] == CP_ERROR_OUT_OF_MEMORY
    finally:
        lib.cp_debug_fail_allocation(-1)
    assert _run(lib, "cp_query", mesh, q, opts, torch)[0] == 0  # the library is still usable
    assert mesh.device_status() == 0


def test_noalloc_refuses_more_than_its_scratch(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_ERROR_NOT_SUPPORTED, CP_ERROR_SCRATCH_TOO_SMALL, lib

    v, t = W.icosphere(3)
    mesh = cpq.Mesh(torch.from_numpy(v).to(cuda), torch.from_numpy(t).to(cuda))
    assert lib.cp_query_noalloc_scratch_bytes() == 32 << 20
    n = 3 << 20  # three times the 1,048,576 queries the fixed array is sized for
    q = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    dist = torch.full((n,), -1.0, device=cuda)
    st = lib.cp_query_noalloc(mesh.handle, _ptr(q), n, byref(cpq.query_opts()), None, _ptr(dist),
                              None, None, c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == CP_ERROR_SCRATCH_TOO_SMALL
    assert b"fixed area" in lib.cp_last_error_string()
    assert bool((dist == -1.0).all())  # refused before anything ran
    # the same count without Morton ordering needs no per-query scratch
    st = lib.cp_query_noalloc(mesh.handle, _ptr(q), n, byref(cpq.query_opts(sort_queries=False)),
                              None, _ptr(dist), None, None,
                              c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == 0
    np.testing.assert_allclose(dist[:8].cpu().numpy(), 1.0, rtol=1e-2)
    # the ordered limit is exact: 1,048,576 queries run, one more is refused
    stream = c_void_p(torch.cuda.current_stream().cuda_stream)
    lim = 1 << 20
    dist.fill_(-1.0)
    assert lib.cp_query_noalloc(mesh.handle, _ptr(q), lim, byref(cpq.query_opts()), None, _ptr(dist),
                                None, None, stream) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(dist[:lim].cpu().numpy(), 1.0, rtol=1e-2)
    assert bool((dist[lim:] == -1.0).all())
    st = lib.cp_query_noalloc(mesh.handle, _ptr(q), lim + 1, byref(cpq.query_opts()), None, _ptr(dist),
                              None, None, stream)
    assert st == CP_ERROR_SCRATCH_TOO_SMALL
    # more than 2^31 - 1 queries: refused on the host, as cp_query refuses them
    st = lib.cp_query_noalloc(mesh.handle, _ptr(q), 1 << 31, byref(cpq.query_opts(sort_queries=False)),
                              None, _ptr(dist), None, None, stream)
    assert st == CP_ERROR_NOT_SUPPORTED
    torch.cuda.synchronize()
    assert bool((dist[lim:] == -1.0).all())
