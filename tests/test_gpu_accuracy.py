"""Distance accuracy against FP64 for every workload configuration, with the
maximum and 99th-percentile relative error printed (run with -s to see them).

Samples follow the oracle definition: every query of the small
configuration; seeded 65,536-query samples of the large, torus and dynamic
configurations (the dynamic one at iteration 0 and after 50 perturb + refit
iterations); 256 queries of each of the 256 batched meshes, queried in one
batched launch.  The bound is 1e-6 relative for every query.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SAMPLE = 65536


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def report(name, d, ref):
    d = np.asarray(d, np.float64)
    nz = ref > 0
    rel = np.zeros_like(ref)
    rel[nz] = np.abs(d[nz] - ref[nz]) / ref[nz]
    print(f"ACCURACY {name}: n={len(ref)} max={rel.max():.3e} p99={np.percentile(rel, 99):.3e} "
          f"zero-distance queries={int((~nz).sum())}")
    assert rel.max() <= 1e-6, f"{name}: max relative error {rel.max():.3e}"
    assert np.all(np.abs(d[~nz]) <= 1e-7), f"{name}: queries on the surface"


def test_accuracy_small(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t, q = W.small()
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=2, leaf_size=4)
    report("small (all 65,536 queries, binary leaf 4)", m.query(dev(q, cuda)).dist.cpu().numpy(),
           orc.brute_f64(v, t, q)["dist"])


def test_accuracy_large_sample(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t, q = W.large()
    s = np.random.default_rng(101).choice(len(q), SAMPLE, replace=False)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=8)
    d = m.query(dev(q, cuda)).dist.cpu().numpy()[s]
    report("large (65,536 of 16,777,216 queries, K4 leaf 8)", d, orc.exact_f64(v, t, q[s])["dist"])


def test_accuracy_torus_sample(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t, q, _ = W.torus_workload()
    s = np.random.default_rng(102).choice(len(q), SAMPLE, replace=False)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=2)
    d = m.query(dev(q, cuda)).dist.cpu().numpy()[s]
    report("torus (65,536 of 4,194,304 queries, K4 leaf 2)", d, orc.exact_f64(v, t, q[s])["dist"])


def test_accuracy_batched(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    meshes, queries = W.batched()
    per = 256
    V, voff, T, toff, _, _ = W.concat_batch(meshes, [q[:per] for q in queries])
    Q = np.concatenate([q[:per] for q in queries])
    qoff = np.arange(len(meshes) + 1, dtype=np.int64) * per
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=4, leaf_size=2)
    d = b.query(dev(Q, cuda), qoff).dist.cpu().numpy()
    ref = np.concatenate([orc.exact_f64(v, t, q[:per])["dist"] for (v, t, _), q in zip(meshes, queries)])
    report(f"batched (256 queries x {len(meshes)} meshes, {len(T):,} tris, one launch)", d, ref)


def test_accuracy_dynamic(orc, cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.soup()
    q = W.uniform_queries(SAMPLE, 0.0, 1.0, 103)
    vd = dev(v, cuda)
    m = cpq.Mesh(vd, dev(t, cuda), branching=4, leaf_size=2)
    qd = dev(q, cuda)
    report("dynamic soup, iteration 0 (65,536 queries, 8,388,608 tris)", m.query(qd).dist.cpu().numpy(),
           orc.exact_f64(v, t, q)["dist"])
    gen = torch.Generator(device=cuda).manual_seed(104)
    for _ in range(50):
        vd.add_(torch.randn(vd.shape, device=cuda, generator=gen) * 1e-4)
        m.refit(vd)
    d = m.query(qd).dist.cpu().numpy()
    report("dynamic soup, after 50 perturb + refit iterations", d, orc.exact_f64(vd.cpu().numpy(), t, q)["dist"])
