"""Bit-exact builds at the workloads' full sizes.

Morton codes and the BVH topology must equal the CPU restatement bit for bit.
The small-mesh parity tests cover every build option; these cover the builds
the measured workloads actually use, at their sizes:

* the large heightfield (1024 x 1024 vertices, 2,093,058 triangles), 4-wide,
  leaf 8, with count and SAH leaf collapse;
* the dynamic workload's 8,388,608-triangle Gaussian-cluster soup (4-wide,
  leaf 2), whose keys need more than 32 bits and whose clusters make long
  runs of near-equal keys;
* the batched workload's 256 meshes (22,243,304 triangles) in one build
  (4-wide, leaf 2), keys carrying the mesh id in their high bits.

Compared: sorted keys, triangle order, left / right / parent, leaf-cluster
flags, the binary node behind each wide node, the wide nodes' child boxes as
bit patterns, child refs and counts, and the node counts and depth bounds.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _equal(name, got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, f"{name}: shape {got.shape} vs {want.shape}"
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, (f"{name}: {len(bad)} of {len(want)} differ, first at {bad[0]}: "
                           f"{got[bad[0]]} vs {want[bad[0]]}")


def _compare(ref, build, wide, num_wide):
    assert num_wide == ref.num_wide
    for k in ("keys", "order", "left", "right", "parent", "cluster", "wide_src"):
        _equal(k, build[k], getattr(ref, k))
    _equal("wide boxes (bits)", wide["boxes"].view(np.uint32), ref.wide_box.view(np.uint32))
    _equal("wide refs", wide["refs"], ref.wide_ref)
    _equal("wide counts", wide["counts"], ref.wide_count)


@pytest.mark.parametrize("collapse", ["count", "sah"])
def test_large_heightfield_build_bit_exact(orc, cpq, cuda, collapse):
    from gpurt_cpq import workloads as W

    v, t = W.heightfield(1024)
    assert t.shape[0] == 2_093_058
    ref = orc.Tree(v, t, 4, 8, 1 if collapse == "sah" else 0, 1.0, 1.0)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=8, collapse=collapse)
    info = m.info()
    assert info.max_wide_depth == ref.max_wide_depth
    assert info.stack_bound == ref.stack_bound
    assert info.num_leaves == ref.num_leaves
    _compare(ref, m.export_build(), m.export_wide(), info.num_wide_nodes)


def test_soup_build_bit_exact(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t = W.soup()
    assert t.shape[0] == 8 * (1 << 20)
    ref = orc.Tree(v, t, 4, 2, 0)
    assert int(ref.keys.max()) >= 1 << 32  # the keys use more than 32 bits
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=2)
    info = m.info()
    assert info.max_wide_depth == ref.max_wide_depth
    assert info.stack_bound == ref.stack_bound
    _compare(ref, m.export_build(), m.export_wide(), info.num_wide_nodes)


def test_batched_build_bit_exact(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched()
    V, voff, T, toff, _, _ = W.concat_batch(meshes, queries)
    assert len(toff) == 257
    ref = orc.Tree(V, T, 4, 2, 0, vert_offsets=voff, tri_offsets=toff)
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=4, leaf_size=2)
    info = b.info()
    assert info["num_triangles"] == T.shape[0]
    assert info["stack_bound"] == ref.stack_bound
    _compare(ref, b.export_build(), b.export_wide(), info["num_wide_nodes"])
