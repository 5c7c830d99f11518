"""GPU adjoint: d(distance)/d(query) against FP64 central finite differences
(h = 1e-4) and the FP64 analytic gradient; d(distance)/d(vertices) against the
FP64 analytic gradient; the torch.autograd.Function wrapper end to end."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_ATOL = 2e-5   # |grad_gpu - grad_fp64| per component, gradients are O(|g|) ~ 1
FD_H = 1e-4


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def bary3(b2):
    b2 = np.asarray(b2, np.float64)
    return np.stack([1.0 - b2[:, 0] - b2[:, 1], b2[:, 0], b2[:, 1]], 1)


def test_backward_torus(orc, cpq, cuda):
    """The differentiable workload at its full size: torus of 200,000
    triangles, 4,194,304 queries uniform in [-1.5, 1.5]^3, upstream gradient
    N(0, 1)."""
    from gpurt_cpq import workloads as W

    v, t, q, g = W.torus_workload()
    assert q.shape[0] == 4 * (1 << 20) and t.shape[0] == 200_000
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=2)
    qd, gd = dev(q, cuda), dev(g, cuda)
    r = m.query(qd, want_point=True, want_bary=True)
    gq, gv = m.backward(qd, r.tri, r.bary, gd)
    gq, gv = gq.cpu().numpy(), gv.cpu().numpy()
    tri, b2 = r.tri.cpu().numpy(), r.bary.cpu().numpy()
    g64 = g.astype(np.float64)
    # 1. the FP64 analytic gradient at the GPU's own (tri, bary)
    rq, rv = orc.backward_f64(v, t, q, tri, bary3(b2), g64)
    assert np.abs(gq - rq).max() <= GRAD_ATOL
    scale = np.maximum(1.0, np.abs(rv))
    assert (np.abs(gv - rv) / scale).max() <= 1e-4
    # 2. with bary = NULL the adjoint recomputes the exact closest point on the
    #    forward's triangle: it matches the FP64 analytic gradient at the FP64
    #    closest point of that triangle.  (Where the forward's triangle differs
    #    from the FP64 optimum, FP64 confirms a distance tie within 1e-6, but
    #    far from a finely tessellated surface the tied closest points can sit
    #    ~1e-4 apart, so the gradient is compared per selected triangle.)
    gq_x, _ = m.backward(qd, r.tri, None, gd, need_verts=False)
    gq_x = gq_x.cpu().numpy()
    idx = np.random.default_rng(1).choice(q.shape[0], 10000, replace=False)
    d_sel, b_sel = orc.dist_to_tri_f64(v, t, q[idx], tri[idx], want_bary=True)
    rq2, _ = orc.backward_f64(v, t, q[idx], tri[idx], b_sel, g64[idx])
    err2 = np.abs(gq_x[idx] - rq2).max(axis=1)
    assert err2.max() <= GRAD_ATOL, np.sort(err2)[-10:]
    e_all = orc.exact_f64(v, t, q)  # the FP64 optimum of every query
    e = {k: e_all[k][idx] for k in ("dist", "tri", "point")}
    assert np.all((d_sel - e["dist"]) / e["dist"] <= 1e-6)
    # 3. central finite differences in FP64 on the same 10k queries, at the
    #    configured step h = 1e-4 and at h / 2.  A central difference measures
    #    the gradient only where the distance is smooth across the stencil:
    #    the FP64 closest triangle is the same at q and at every q +- h and
    #    q +- h/2 (a stencil across a medial sheet of the polyhedral surface
    #    straddles a jump in the gradient).  Where the stencil stays in one
    #    triangle's face region the distance is linear across it and the
    #    difference is exact up to FP64 rounding, so there the configured step
    #    measures the FP32 error of the adjoint itself.  Near an edge or vertex
    #    its truncation error grows like |g| h^2 / d^2, and a stencil that
    #    crosses from a face's region into an edge's (the same triangle) meets a
    #    jump in the second derivative; the Richardson combination
    #    (4 D(h/2) - D(h)) / 3 cancels the h^2 term.
    q64 = q[idx].astype(np.float64)
    fd = {FD_H: np.zeros((len(idx), 3)), FD_H / 2: np.zeros((len(idx), 3))}
    smooth = np.ones(len(idx), bool)
    for h in fd:
        for k in range(3):
            qp, qm = q64.copy(), q64.copy()
            qp[:, k] += h
            qm[:, k] -= h
            dp, tp = orc.exact_f64_dq(v, t, qp)
            dm, tm = orc.exact_f64_dq(v, t, qm)
            fd[h][:, k] = g64[idx] * (dp - dm) / (2 * h)
            smooth &= (tp == e["tri"]) & (tm == e["tri"])
    # compare at queries whose forward closest point is the FP64 optimum's
    # (tied closest points elsewhere, see 2.) and at least 0.01 from the surface
    same = np.linalg.norm(r.point.cpu().numpy()[idx] - e["point"], axis=1) <= 1e-6
    assert same.mean() >= 0.95
    use = same & smooth & (e["dist"] >= 0.01)
    assert use.mean() >= 0.8
    # face-region queries: the FP64 closest point lies more than 2h inside
    # every edge of its triangle (the projection moves it by at most h)
    tv = v[t[e["tri"]]].astype(np.float64)
    area2 = np.linalg.norm(np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]), axis=1)
    b3 = e_all["bary"][idx]
    inside = np.ones(len(idx), bool)
    for k in range(3):
        opp = np.linalg.norm(tv[:, (k + 2) % 3] - tv[:, (k + 1) % 3], axis=1)
        inside &= b3[:, k] * area2 / opp > 2 * FD_H
    face = use & inside
    assert face.sum() >= 0.25 * use.sum()
    err_h = np.abs(gq[idx] - fd[FD_H]).max(axis=1)
    rich = (4.0 * fd[FD_H / 2] - fd[FD_H]) / 3.0
    err_r = np.abs(gq[idx] - rich).max(axis=1)
    print(f"FD check, h = 1e-4: {face.sum()} face-region queries max {err_h[face].max():.2e}, "
          f"p99 {np.percentile(err_h[face], 99):.2e}; all {use.sum()} smooth queries p99 "
          f"{np.percentile(err_h[use], 99):.2e}, max {err_h[use].max():.2e}; Richardson (h, h/2) p99 "
          f"{np.percentile(err_r[use], 99):.2e}, max {err_r[use].max():.2e}")
    assert err_h[face].max() <= 1e-5
    assert np.median(err_r[use]) <= 1e-6
    assert np.percentile(err_r[use], 99) <= 1e-5
    assert np.percentile(err_h[use], 99) <= 1e-4
    assert err_h[use].max() <= 1e-3
    # 4. d/dvertices independent of the forward's choice: the FP64 analytic
    #    gradient at each query's FP64 optimum (its own triangle and weights)
    #    over every query whose GPU closest point is that optimum's point,
    #    against the GPU adjoint of the forward's (tri, bary) with the upstream
    #    gradient of the other queries zeroed.  Equal closest points at a
    #    shared edge or vertex put equal weights on the same vertices,
    #    whichever triangle holds them.
    agree = np.linalg.norm(r.point.cpu().numpy() - e_all["point"], axis=1) <= 1e-6
    assert agree.mean() >= 0.95
    g_m = np.where(agree, g, 0.0).astype(np.float32)
    _, gv_m = m.backward(qd, r.tri, r.bary, dev(g_m, cuda))
    _, rv_opt = orc.backward_f64(v, t, q, e_all["tri"], e_all["bary"], g_m.astype(np.float64))
    dv_err = np.abs(gv_m.cpu().numpy() - rv_opt) / np.maximum(1.0, np.abs(rv_opt))
    print(f"d/dvertices vs the FP64 optimum's gradient over {agree.sum()} queries: "
          f"max {dv_err.max():.2e}, p99 {np.percentile(dv_err, 99):.2e}")
    assert np.percentile(dv_err, 99) <= 1e-5
    assert dv_err.max() <= 1e-3


def test_backward_zero_distance_and_invalid(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.icosphere(2)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda))
    q = dev(v[:10], cuda)  # on the surface: d = 0 -> zero gradient
    r = m.query(q, want_bary=True)
    g = torch.ones(10, device=cuda)
    gq, gv = m.backward(q, r.tri, r.bary, g)
    assert float(gq.abs().max()) == 0.0 and float(gv.abs().max()) == 0.0
    # tri = -1 (a query that found nothing) contributes nothing
    tri = r.tri.clone()
    tri[0] = -1
    gq, gv = m.backward(q, tri, r.bary, g)
    assert float(gq[0].abs().max()) == 0.0


def test_warp_aggregated_atomics_many_shared_vertices(orc, cpq, cuda):
    """All queries hit one small mesh: lanes share vertices, the warp sums them first."""
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(1)  # 80 triangles, 42 vertices
    q = W.uniform_queries(100000, -2, 2, 5)
    g = np.random.default_rng(2).normal(size=q.shape[0]).astype(np.float32)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    qd = dev(q, cuda)
    r = m.query(qd, want_point=False, want_bary=True)
    _, gv = m.backward(qd, r.tri, r.bary, dev(g, cuda))
    _, rv = orc.backward_f64(v, t, q, r.tri.cpu().numpy(), bary3(r.bary.cpu().numpy()),
                             g.astype(np.float64))
    np.testing.assert_allclose(gv.cpu().numpy(), rv, rtol=1e-4, atol=1e-3)


def test_autograd_function(orc, cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.torus(100, 40)
    vd = dev(v, cuda).requires_grad_(True)
    m = cpq.Mesh(vd.detach(), dev(t, cuda), branching=4)
    q = dev(W.uniform_queries(20000, -1.5, 1.5, 6), cuda).requires_grad_(True)
    d, tri = cpq.closest_distance(q, m, vd)
    w = torch.randn_like(d)
    (d * w).sum().backward()
    r = m.query(q.detach(), want_point=False, want_bary=True)
    gq, gv = m.backward(q.detach(), r.tri, r.bary, w)
    assert torch.allclose(q.grad, gq, atol=1e-6)
    assert torch.allclose(vd.grad, gv, atol=1e-5)
    assert torch.equal(tri, r.tri)
    # forward+backward of the autograd path matches the FP64 analytic gradient
    rq, _ = orc.backward_f64(v, t, q.detach().cpu().numpy(), tri.cpu().numpy(),
                             bary3(r.bary.cpu().numpy()), w.cpu().numpy().astype(np.float64))
    assert np.abs(q.grad.cpu().numpy() - rq).max() <= GRAD_ATOL
