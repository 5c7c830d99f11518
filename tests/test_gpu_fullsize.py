"""Every answer of the large and torus workloads against FP64, at full size.

The benched configuration (2,093,058-triangle heightfield, 16,777,216
queries, 4-wide BVH with leaf 8, packets seeded in chunks of 4): each
distance within 1e-6 relative of the FP64 oracle's, every triangle index
that differs from the oracle's an FP64-confirmed tie within 1e-6, and each
closest point on the same triangle within 1e-6 of the oracle's (relative to
max(1, |p|)).  The oracle's search runs on all host cores (about 35 s on 16).
The torus workload (200,000 triangles, 4,194,304 queries, 4-wide BVH with
leaf 2, unseeded: the differentiable form's forward) the same way.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_every_answer(orc, v, t, q, d, tri, p, name):
    ref = orc.exact_f64(v, t, q)
    nz = ref["dist"] > 0
    assert np.all(np.abs(d[~nz]) <= 1e-7), "queries on the surface"
    rel = np.abs(d[nz] - ref["dist"][nz]) / ref["dist"][nz]
    print(f"{name}, all {len(q):,} queries: max {rel.max():.3e} p99 {np.percentile(rel, 99):.3e}")
    assert rel.max() <= 1e-6, f"max relative error {rel.max():.3e}"
    mm = np.nonzero(tri != ref["tri"])[0]
    assert np.all(tri[mm] >= 0)
    gap = (orc.dist_to_tri_f64(v, t, q[mm], tri[mm]) - ref["dist"][mm]) / np.maximum(ref["dist"][mm], 1e-30)
    print(f"index mismatches: {len(mm):,}, worst FP64 gap {gap.max(initial=0):.3e}")
    assert np.all(gap <= 1e-6), f"worst FP64 gap {gap.max():.3e}"
    same = tri == ref["tri"]
    scale = np.maximum(1.0, np.abs(ref["point"]).max(axis=1))
    perr = np.linalg.norm(p - ref["point"], axis=1) / scale
    assert perr[same].max() <= 1e-6, f"point error {perr[same].max():.3e}"


def _query(cpq, cuda, v, t, q, K, leaf, opts):
    import torch

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)

    m = cpq.Mesh(dev(v), dev(t), branching=K, leaf_size=leaf)
    r = m.query(dev(q), opts=opts)
    out = (r.dist.cpu().numpy().astype(np.float64), r.tri.cpu().numpy(), r.point.cpu().numpy().astype(np.float64))
    assert m.device_status() == 0
    del r, m
    torch.cuda.empty_cache()
    return out


def test_large_workload_every_answer(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t, q = W.large()
    assert q.shape[0] == 16 * (1 << 20)
    d, tri, p = _query(cpq, cuda, v, t, q, 4, 8, cpq.query_opts(seed_chunk=4))
    _check_every_answer(orc, v, t, q, d, tri, p, "large")


def test_torus_workload_every_answer(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t, q, _ = W.torus_workload()
    assert q.shape[0] == 4 * (1 << 20)
    d, tri, p = _query(cpq, cuda, v, t, q, 4, 2, cpq.query_opts())
    _check_every_answer(orc, v, t, q, d, tri, p, "torus")
