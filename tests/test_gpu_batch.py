"""GPU batched form: many meshes in one build and one persistent launch,
checked per mesh against FP64, against separate per-mesh launches, and in
CUDA-graph mode against the plain launch."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def check_mesh(orc, v, t, q, dist, tri, ref=None):
    if ref is None:
        ref = orc.exact_f64(v, t, q)
    rel = np.abs(dist.astype(np.float64) - ref["dist"])
    nz = ref["dist"] > 0
    rel[nz] /= ref["dist"][nz]
    assert rel[nz].max(initial=0) <= 1e-6
    assert np.all(rel[~nz] <= 1e-7)
    mm = np.nonzero(tri != ref["tri"])[0]
    if len(mm):
        dt = orc.dist_to_tri_f64(v, t, q[mm], tri[mm])
        assert np.all((dt - ref["dist"][mm]) / np.maximum(ref["dist"][mm], 1e-30) <= 1e-6)


def test_batch_reference_meshes(orc, cpq, cuda):
    """The reference's demo meshes (cube and mis_test, 8 meshes, 2..960 tris)."""
    g = np.load(GOLDEN / "ref_meshes.npz")
    b = cpq.Batch(dev(g["verts"], cuda), g["vert_offsets"], dev(g["tris"], cuda), g["tri_offsets"],
                  branching=4)
    r = b.query(dev(g["queries"], cuda), g["q_offsets"])
    d, tri = r.dist.cpu().numpy(), r.tri.cpu().numpy()
    vo, to, qo = g["vert_offsets"], g["tri_offsets"], g["q_offsets"]
    for m in range(len(to) - 1):
        s = slice(qo[m], qo[m + 1])
        v, t = g["verts"][vo[m]:vo[m + 1]], g["tris"][to[m]:to[m + 1]]
        check_mesh(orc, v, t, g["queries"][s], d[s], tri[s],
                   ref={"dist": g["dist"][s], "tri": g["tri"][s]})


def test_batch_bit_exact_tree(orc, cpq, cuda):
    """A batch's per-mesh subtrees and its wide nodes equal the restatement's."""
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched(seed=9, nmeshes=12, tri_range=(20, 3000), q_range=(10, 200))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    for K in (2, 4, 8):
        ref = orc.Tree(V, T, K, 4, 0, vert_offsets=voff, tri_offsets=toff)
        b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=K)
        info = b.info()
        assert info["num_wide_nodes"] == ref.num_wide
        assert info["stack_bound"] == ref.stack_bound
        r = b.query(dev(Q, cuda), qoff)
        q_mesh = np.repeat(np.arange(len(qoff) - 1), np.diff(qoff)).astype(np.int32)
        cpu = ref.query(Q, q_mesh=q_mesh)
        # same tree, same per-query arithmetic order up to FMA contraction:
        # distances agree to FP32 rounding, indices up to ties
        np.testing.assert_allclose(r.dist.cpu().numpy(), cpu["dist"], rtol=1e-6, atol=1e-7)


def test_batch_synthetic_vs_fp64_and_per_mesh(orc, cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    meshes, queries = W.batched(seed=4, nmeshes=24, tri_range=(1000, 60000), q_range=(1000, 20000))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=4)
    r = b.query(dev(Q, cuda), qoff, want_bary=True)
    d, tri = r.dist.cpu().numpy(), r.tri.cpu().numpy()
    for m, ((v, t, _), q) in enumerate(zip(meshes, queries)):
        s = slice(qoff[m], qoff[m + 1])
        check_mesh(orc, v, t, q, d[s], tri[s])
        # plain per-mesh launch: same distances (different trees, same answers)
        pm = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
        rp = pm.query(dev(q, cuda))
        np.testing.assert_allclose(rp.dist.cpu().numpy(), d[s], rtol=1e-6, atol=1e-7)
    # graph mode: capture once, replay, identical results
    ws = torch.empty(b.workspace_size(Q.shape[0]), dtype=torch.uint8, device=cuda)
    qd = dev(Q, cuda)
    out = cpq.QueryResult(point=torch.empty((Q.shape[0], 3), device=cuda),
                          dist=torch.empty(Q.shape[0], device=cuda),
                          tri=torch.empty(Q.shape[0], dtype=torch.int32, device=cuda), bary=None)
    for _ in range(3):
        out.dist.fill_(-1)
        b.query(qd, qoff, workspace=ws, use_graph=True, out=out)
        torch.cuda.synchronize()
        assert torch.equal(out.dist, r.dist)
        assert torch.equal(out.tri, r.tri)
    # a replay launches nothing through the library; a changed option
    # (here the seed chunk) captures a new graph, whose kernels it counts
    from gpurt_cpq._lib import lib
    n0 = lib.cp_kernel_launches()
    b.query(qd, qoff, workspace=ws, use_graph=True, out=out)
    assert lib.cp_kernel_launches() == n0
    b.query(qd, qoff, workspace=ws, use_graph=True, out=out, opts=cpq.query_opts(seed_chunk=4))
    torch.cuda.synchronize()
    assert lib.cp_kernel_launches() > n0
    assert torch.equal(out.dist, r.dist)


def test_batch_rejects_bad_offsets(cpq, cuda):
    from gpurt_cpq._lib import CpError

    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.int32)
    with pytest.raises(CpError):
        cpq.Batch(dev(v, cuda), [0, 3, 3], dev(t, cuda), [0, 1, 1])  # empty mesh
    b = cpq.Batch(dev(v, cuda), [0, 3], dev(t, cuda), [0, 1])
    with pytest.raises((CpError, ValueError)):
        b.query(dev(np.zeros((4, 3), np.float32), cuda), [0, 5])


def test_batch_per_mesh_leaf_sizes_bit_exact(orc, cpq, cuda):
    """A leaf size per mesh in one build (cp_batch_create_leaves): keys,
    topology and wide nodes equal the restatement built with the same sizes,
    and the answers are FP64's."""
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched(seed=9, nmeshes=12, tri_range=(20, 3000), q_range=(10, 200))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    leaves = np.array([1, 2, 4, 8, 3, 15, 2, 1, 8, 4, 6, 2], np.int32)
    ref = orc.Tree(V, T, 4, 0, 0, vert_offsets=voff, tri_offsets=toff, mesh_leaf=leaves)
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=4, leaf_sizes=leaves)
    bld, wide = b.export_build(), b.export_wide()
    for k in ("keys", "order", "left", "right", "parent", "cluster", "wide_src"):
        np.testing.assert_array_equal(bld[k], getattr(ref, k), err_msg=k)
    np.testing.assert_array_equal(wide["boxes"].view(np.uint32), ref.wide_box.view(np.uint32))
    np.testing.assert_array_equal(wide["refs"], ref.wide_ref)
    np.testing.assert_array_equal(wide["counts"], ref.wide_count)
    # every mesh's leaves hold at most its own count
    counts, refs = wide["counts"], wide["refs"]
    tri_mesh = np.searchsorted(toff, np.arange(toff[-1]), side="right") - 1
    for c, r in zip(counts, refs):
        if c > 0:
            assert c <= leaves[tri_mesh[ref.order[r]]]
    r = b.query(dev(Q, cuda), qoff)
    d, tri = r.dist.cpu().numpy(), r.tri.cpu().numpy()
    for m in range(len(toff) - 1):
        s = slice(qoff[m], qoff[m + 1])
        check_mesh(orc, V[voff[m]:voff[m + 1]], T[toff[m]:toff[m + 1]], Q[s], d[s], tri[s])


def test_batch_autotune_per_size_class(orc, cpq, cuda, tmp_path):
    """cp_batch_autotune: one leaf size per triangle-count class, written to
    and read back from the cache file; the tuned batch answers as FP64."""
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched(seed=5, nmeshes=24, tri_range=(1000, 40000), q_range=(500, 5000))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    Vd, Td, Qd = dev(V, cuda), dev(T, cuda), dev(Q, cuda)
    cache = tmp_path / "tune.txt"
    leaves, qo = cpq.autotune_batch(Vd, voff, Td, toff, Qd, qoff, branching=4, cache_path=str(cache))
    cls = np.floor(np.log2(np.diff(toff))).astype(int)
    assert set(np.unique(leaves)) <= {1, 2, 4, 8}
    for c in np.unique(cls):
        assert len(set(leaves[cls == c])) == 1  # one choice per class
    lines = [ln.split() for ln in cache.read_text().splitlines() if ln.startswith("B ")]
    assert sorted(int(x[1]) for x in lines) == sorted(np.unique(cls).tolist())
    again, _ = cpq.autotune_batch(Vd, voff, Td, toff, Qd, qoff, branching=4, cache_path=str(cache))
    np.testing.assert_array_equal(again, leaves)  # from the cache
    b = cpq.Batch(Vd, voff, Td, toff, branching=4, leaf_sizes=leaves)
    r = b.query(Qd, qoff, opts=qo)
    d, tri = r.dist.cpu().numpy(), r.tri.cpu().numpy()
    for m in range(len(toff) - 1):
        s = slice(qoff[m], qoff[m + 1])
        check_mesh(orc, V[voff[m]:voff[m + 1]], T[toff[m]:toff[m + 1]], Q[s], d[s], tri[s])
