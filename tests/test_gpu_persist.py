"""Saved BVHs (cp_mesh_save / cp_mesh_load).

A mesh read back from its file must answer queries, refit and export exactly
as the mesh that wrote it, without a build.  A damaged file must be refused
with a message before anything reaches the GPU: the tests damage a saved file
in each way a kernel would otherwise follow out of bounds or around a loop
(a child outside the nodes, a cycle, a leaf past the triangles, a broken
order, a vertex index outside its mesh, unsorted keys, a depth bound below
the tree's depth) and in the ways a file breaks (truncated, extended, a
foreign header).
"""
from __future__ import annotations

import struct

import numpy as np
import pytest

from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE

HEADER = 88


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def layout(n, w, K, nm=1):
    """Byte offset of each stored array in a file of n triangles, w wide nodes."""
    nn, inner = 2 * n - 1, max(n - 1, 1)
    sizes = [("tris", 12 * n), ("keys", 8 * n), ("order", 4 * n), ("inv_order", 4 * n), ("left", 4 * inner),
             ("right", 4 * inner), ("parent", 4 * nn), ("first", 4 * nn), ("last", 4 * nn), ("box", 24 * nn),
             ("cost", 4 * nn), ("leaf_flag", nn), ("cluster", nn), ("mesh_root", 4 * nm), ("wide_root", 4 * nm),
             ("frame", 24 * nm), ("recs", 48 * n), ("fast", 80 * n), ("nodes", 32 * K * w), ("wide_src", 4 * w),
             ("slot_src", 4 * w * K)]
    off, out = HEADER + 16 * (nm + 1), {}
    for name, size in sizes:
        out[name] = (off, size)
        off += size
    return out, off


@pytest.mark.gpu
@pytest.mark.parametrize("K,leaf,collapse", [(4, 8, "count"), (2, 4, "sah"), (8, 2, "count")])
def test_saved_mesh_answers_as_built(cpq, cuda, tmp_path, K, leaf, collapse):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.heightfield(128, seed=12)
    vd, td = dev(v, cuda), dev(t, cuda)
    m = cpq.Mesh(vd, td, branching=K, leaf_size=leaf, collapse=collapse)
    path = tmp_path / "mesh.bvh"
    m.save(path)
    info = m.info()
    _, total = layout(info.num_triangles, info.num_wide_nodes, K)
    assert path.stat().st_size == total
    loaded = cpq.Mesh.load(path)
    li = loaded.info()
    for f in ("num_triangles", "num_wide_nodes", "num_leaves", "branching", "leaf_size", "max_wide_depth",
              "stack_bound"):
        assert getattr(li, f) == getattr(info, f), f
    q = dev(np.concatenate([W.heightfield_queries(v, t, 40_000, seed=13), W.uniform_queries(20_000, -0.2, 1.2, 14)]),
            cuda)
    for opts in (cpq.query_opts(), cpq.query_opts(traversal="thread"), cpq.query_opts(seed_chunk=4)):
        a, b = m.query(q, want_bary=True, opts=opts), loaded.query(q, want_bary=True, opts=opts)
        for k in ("dist", "tri", "point", "bary"):
            assert torch.equal(getattr(a, k), getattr(b, k)), k
    eb, lb = m.export_build(), loaded.export_build()
    for k in eb:
        np.testing.assert_array_equal(eb[k], lb[k], err_msg=k)
    ew, lw = m.export_wide(), loaded.export_wide()
    np.testing.assert_array_equal(ew["boxes"].view(np.uint32), lw["boxes"].view(np.uint32))
    np.testing.assert_array_equal(ew["refs"], lw["refs"])
    # refit after moving the vertices: the same boxes and answers
    moved = vd + 1e-3 * torch.randn(vd.shape, generator=torch.Generator(device=cuda).manual_seed(3), device=cuda)
    m.refit(moved)
    loaded.refit(moved)
    a, b = m.query(q), loaded.query(q)
    assert torch.equal(a.dist, b.dist) and torch.equal(a.tri, b.tri)
    np.testing.assert_array_equal(m.export_wide()["boxes"].view(np.uint32),
                                  loaded.export_wide()["boxes"].view(np.uint32))
    assert loaded.device_status() == 0


@pytest.mark.gpu
def test_saved_batch_answers_as_built(cpq, cuda, tmp_path):
    """A batch with a leaf size per mesh, saved and read back: the same
    answers, trees and boxes; a batch file is refused by cp_mesh_load, a
    mesh file reads as a batch of one, and a truncated batch file is
    refused."""
    import torch

    from gpurt_cpq import CpError
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched(seed=3, nmeshes=9, tri_range=(200, 20000), q_range=(100, 8000))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    leaves = np.int32([1, 2, 4, 8, 2, 2, 4, 1, 8])
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=4, leaf_sizes=leaves)
    path = tmp_path / "batch.bvh"
    b.save(path)
    loaded = cpq.Batch.load(path)
    assert loaded.nmeshes == 9 and loaded.opts.branching == 4
    assert loaded.info() == b.info()
    qd = dev(Q, cuda)
    for opts in (cpq.query_opts(), cpq.query_opts(seed_chunk=4), cpq.query_opts(traversal="thread")):
        a, c = b.query(qd, qoff, want_bary=True, opts=opts), loaded.query(qd, qoff, want_bary=True, opts=opts)
        for k in ("dist", "tri", "point", "bary"):
            assert torch.equal(getattr(a, k), getattr(c, k)), k
    eb, lb = b.export_build(), loaded.export_build()
    for k in eb:
        np.testing.assert_array_equal(eb[k], lb[k], err_msg=k)
    np.testing.assert_array_equal(b.export_wide()["boxes"].view(np.uint32),
                                  loaded.export_wide()["boxes"].view(np.uint32))
    with pytest.raises(CpError, match="batch of 9 meshes"):
        cpq.Mesh.load(path)
    data = path.read_bytes()
    (tmp_path / "short.bvh").write_bytes(data[:-7])
    with pytest.raises(CpError, match="cp_batch_load"):
        cpq.Batch.load(tmp_path / "short.bvh")
    # a mesh file as a batch of one
    v, t = meshes[2][0], meshes[2][1]
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    m.save(tmp_path / "mesh.bvh")
    one = cpq.Batch.load(tmp_path / "mesh.bvh")
    q = dev(queries[2], cuda)
    r1, r2 = m.query(q), one.query(q, [0, q.shape[0]])
    assert torch.equal(r1.dist, r2.dist) and torch.equal(r1.tri, r2.tri)


def _refused(lib, path):
    from ctypes import byref, c_void_p

    h = c_void_p()
    st = lib.cp_mesh_load(str(path).encode(), None, byref(h))
    return st == CP_ERROR_INVALID_VALUE and not h.value, lib.cp_last_error_string().decode()


@pytest.mark.gpu
def test_damaged_files_are_refused(cpq, cuda, tmp_path):
    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import lib

    v, t = W.icosphere(3)
    K = 4
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=4)
    good = tmp_path / "good.bvh"
    m.save(good)
    data = bytearray(good.read_bytes())
    info = m.info()
    n, w = info.num_triangles, info.num_wide_nodes
    lay, total = layout(n, w, K)
    assert len(data) == total

    def i32(name, k):
        off, _ = lay[name]
        return off + 4 * k

    nodes_off = lay["nodes"][0]
    root = struct.unpack_from("<i", data, lay["wide_root"][0])[0]
    assert root >= 0

    def child_pos(node, slot):
        return nodes_off + node * 32 * K + 4 * (6 * K + slot)

    # the first inner child slot of the root (a node, not a leaf)
    slot = next(s for s in range(K) if struct.unpack_from("<i", data, child_pos(root, s))[0] >= 0)
    damage = {
        "truncated": lambda d: d[:-1],
        "extended": lambda d: d + b"\0",
        "magic": lambda d: b"XPQBVH\0\1" + d[8:],
        "branching": lambda d: d[:8] + struct.pack("<i", 3) + d[12:],
        "child outside the nodes": lambda d: _put(d, child_pos(root, slot), w + 5),
        "cycle to the root": lambda d: _put(d, child_pos(struct.unpack_from("<i", d, child_pos(root, slot))[0], 0),
                                            root),
        "leaf past the triangles": lambda d: _put(d, child_pos(root, slot), ~(((n - 2) << 4) | 7)),
        "broken order": lambda d: _put(d, i32("inv_order", 0), 1),
        "vertex outside the mesh": lambda d: _put(d, i32("tris", 5), len(v)),
        "unsorted keys": lambda d: d[:lay["keys"][0]] + struct.pack("<Q", 2 ** 62) + d[lay["keys"][0] + 8:],
        "depth bound below the tree": lambda d: _put(_put(d, 40, info.max_wide_depth - 1), 44,
                                                     (K - 1) * info.max_wide_depth),
    }
    for what, f in damage.items():
        path = tmp_path / "bad.bvh"
        path.write_bytes(bytes(f(bytearray(data))))
        ok, msg = _refused(lib, path)
        assert ok, what
        assert msg.startswith("cp_mesh_load"), (what, msg)
    # the good file still loads
    assert cpq.Mesh.load(good).info().num_wide_nodes == w


def _put(d, pos, value):
    d = bytearray(d)
    struct.pack_into("<i", d, pos, value)
    return d


def test_foreign_files_are_refused_without_a_gpu(tmp_path):
    """Files that are not a saved BVH are refused by the header checks, which
    run before any device work (so this runs without a GPU)."""
    from ctypes import byref, c_void_p

    from gpurt_cpq._lib import lib

    cases = {"missing": None, "empty": b"", "text": b"not a bvh at all, just some text\n" * 10,
             "random": np.random.default_rng(1).integers(0, 256, 4096, dtype=np.uint8).tobytes()}
    for name, content in cases.items():
        path = tmp_path / f"{name}.bvh"
        if content is not None:
            path.write_bytes(content)
        h = c_void_p()
        st = lib.cp_mesh_load(str(path).encode(), None, byref(h))
        assert st == CP_ERROR_INVALID_VALUE and not h.value, name
        assert b"cp_mesh_load" in lib.cp_last_error_string()
