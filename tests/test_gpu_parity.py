"""GPU parity: the CUDA build must equal the CPU restatement bit for bit, and
queries must match the FP64 oracle (distances within 1e-6 relative; indices
equal except at FP64-confirmed ties within 1e-6).  Queries closer than 1e-2
of a triangle's size to a shared edge or vertex are held to the bound of
_check_near_surface instead (the FP32 choice among near-tied triangles).
All calls go through the C ABI (gpurt_cpq is a ctypes binding of
include/cpq.h)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
REL_TOL = 1e-6      # distance tolerance against FP64 (relative)
ABS_TOL = 1e-7      # for exact zero distances (query on the surface)


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def rel_err(d, ref):
    d = np.asarray(d, np.float64)
    out = np.abs(d - ref)
    nz = ref > 0
    out[nz] /= ref[nz]
    return out


def check_against_fp64(orc, v, t, q, res, ref=None, rel=REL_TOL):
    """Distances, indices (ties confirmed in FP64), points; returns stats."""
    if ref is None:
        ref = orc.brute_f64(v, t, q) if t.shape[0] * q.shape[0] <= 4e8 else orc.exact_f64(v, t, q)
    d = res.dist.cpu().numpy()
    tri = res.tri.cpu().numpy()
    err = rel_err(d, ref["dist"])
    zero = ref["dist"] == 0
    assert np.all(np.abs(d[zero]) <= ABS_TOL), "zero distances"
    assert err[~zero].max(initial=0) <= rel, f"max rel err {err[~zero].max()}"
    mm = np.nonzero(tri != ref["tri"])[0]
    if len(mm):
        assert np.all(tri[mm] >= 0)
        dt = orc.dist_to_tri_f64(v, t, q[mm], tri[mm])
        gap = (dt - ref["dist"][mm]) / np.maximum(ref["dist"][mm], 1e-30)
        assert np.all(gap <= 1e-6), f"{len(mm)} index mismatches, worst FP64 gap {gap.max()}"
    if res.point is not None:
        p = res.point.cpu().numpy().astype(np.float64)
        scale = np.maximum(1.0, np.abs(ref["point"]).max(axis=1))
        perr = np.linalg.norm(p - ref["point"], axis=1) / scale
        # a tie may legitimately move the closest point along the shared feature
        ok = (perr <= 1e-6) | (tri != ref["tri"])
        assert ok.all(), f"point error {perr[~ok].max()}"
    return {"max_rel": float(err[~zero].max(initial=0)),
            "p99_rel": float(np.percentile(err[~zero], 99)) if (~zero).any() else 0.0,
            "mismatch": int(len(mm))}


# ---------------------------------------------------------------- known answers

def test_kat_gpu(cpq, cuda):
    cases = json.loads((GOLDEN / "kat_point_triangle.json").read_text())
    for c in cases["cases"]:
        v = np.array([c["a"], c["b"], c["c"]], np.float32)
        t = np.array([[0, 1, 2]], np.int32)
        q = np.array([c["q"]], np.float32)
        m = cpq.Mesh(dev(v, cuda), dev(t, cuda))
        r = m.query(dev(q, cuda), want_bary=True)
        d = float(r.dist.cpu()[0])
        if c["dist"] == 0:
            assert abs(d) <= ABS_TOL, c
        else:
            assert abs(d - c["dist"]) <= REL_TOL * c["dist"], (c, d)
        np.testing.assert_allclose(r.point.cpu().numpy()[0], c["point"], atol=1e-5, rtol=1e-6)
        if c["bary"] is not None:
            b = r.bary.cpu().numpy()[0]
            np.testing.assert_allclose([1 - b[0] - b[1], b[0], b[1]], c["bary"], atol=1e-6)
        assert int(r.tri.cpu()[0]) == 0
    tm = cases["tie_mesh"]
    m = cpq.Mesh(dev(np.array(tm["verts"], np.float32), cuda), dev(np.array(tm["tris"], np.int32), cuda))
    r = m.query(dev(np.array(tm["queries"], np.float32), cuda))
    np.testing.assert_array_equal(r.tri.cpu().numpy(), tm["tri"])


# ---------------------------------------------------------------- bit-exact build

def meshes_for_build():
    from gpurt_cpq import workloads as W

    rng = np.random.default_rng(5)
    ico = W.icosphere(4)
    hf = W.heightfield(64, seed=9)
    rv = rng.normal(size=(500, 3)).astype(np.float32)
    rt = rng.integers(0, 500, (2000, 3)).astype(np.int32)
    rt[:50] = rt[0]  # duplicated triangles: equal keys
    tiny = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32),
            np.array([[0, 1, 2], [1, 3, 2]], np.int32))
    one = (tiny[0], tiny[1][:1])
    return {"icosphere4": ico, "heightfield64": hf, "random_dup": (rv, rt), "two": tiny, "one": one}


BUILDS = [(2, 4, 0), (4, 4, 0), (8, 4, 0), (4, 1, 0), (4, 8, 1), (8, 15, 0), (2, 2, 1)]


@pytest.mark.parametrize("name", ["icosphere4", "heightfield64", "random_dup", "two", "one"])
@pytest.mark.parametrize("K,leaf,collapse", BUILDS)
def test_build_bit_exact(orc, cpq, cuda, name, K, leaf, collapse):
    v, t = meshes_for_build()[name]
    ref = orc.Tree(v, t, K, leaf, collapse, 1.0, 1.0)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=leaf,
                 collapse="sah" if collapse else "count")
    info = m.info()
    assert info.num_wide_nodes == ref.num_wide
    assert info.max_wide_depth == ref.max_wide_depth
    assert info.stack_bound == ref.stack_bound
    assert info.num_leaves == ref.num_leaves
    b = m.export_build()
    np.testing.assert_array_equal(b["keys"], ref.keys)
    np.testing.assert_array_equal(b["order"], ref.order)
    np.testing.assert_array_equal(b["left"], ref.left)
    np.testing.assert_array_equal(b["right"], ref.right)
    np.testing.assert_array_equal(b["parent"], ref.parent)
    np.testing.assert_array_equal(b["cluster"], ref.cluster)
    np.testing.assert_array_equal(b["wide_src"], ref.wide_src)
    w = m.export_wide()
    np.testing.assert_array_equal(w["boxes"].view(np.uint32), ref.wide_box.view(np.uint32))
    np.testing.assert_array_equal(w["refs"], ref.wide_ref)
    np.testing.assert_array_equal(w["counts"], ref.wide_count)


def test_vertex_stride_48(orc, cpq, cuda):
    """The reference's VK::Mesh::Vertex layout (pos, norm, tang as Vec4) builds the same tree."""
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.icosphere(3)
    fat = np.zeros((v.shape[0], 12), np.float32)
    fat[:, :3] = v
    fat[:, 4:7] = v  # normal slot
    m12 = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    m48 = cpq.Mesh(dev(fat, cuda), dev(t, cuda), branching=4)
    a, b = m12.export_wide(), m48.export_wide()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    q = dev(W.uniform_queries(4096, -2, 2, 1), cuda)
    r1, r2 = m12.query(q), m48.query(q)
    assert torch.equal(r1.dist, r2.dist) and torch.equal(r1.tri, r2.tri)


# ---------------------------------------------------------------- queries

@pytest.mark.parametrize("K", [2, 4, 8])
def test_query_small_config(orc, cpq, cuda, K):
    from gpurt_cpq import workloads as W

    v, t, q = W.small()
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=4)
    r = m.query(dev(q, cuda), want_bary=True)
    stats = check_against_fp64(orc, v, t, q, r)
    print(f"small K={K}: {stats}")
    b = r.bary.cpu().numpy()
    assert np.all(b >= -1e-6) and np.all(b.sum(1) <= 1 + 1e-6)
    assert m.device_status() == 0


@pytest.mark.parametrize("K", [2, 4, 8])
@pytest.mark.parametrize("leaf", [3, 8, 15])
def test_query_leaf_compaction(orc, cpq, cuda, K, leaf):
    """Leaves of 3 or more triangles: the packet kernel spreads a leaf's
    (query, triangle) pairs over the warp when few lanes need it, in one or
    several rounds.  Queries near the surface and far from it give both few
    and many active lanes per leaf; every answer is checked in FP64."""
    from gpurt_cpq import workloads as W

    v, t = W.torus(120, 48)
    near = W.surface_points(v, t, 20000, np.random.default_rng(11))
    near += np.random.default_rng(12).normal(0.0, 0.02, near.shape)
    q = np.concatenate([near.astype(np.float32), W.uniform_queries(20000, -1.6, 1.6, 13)])
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=leaf)
    r = m.query(dev(q, cuda), opts=cpq.query_opts(traversal="packet"))
    stats = check_against_fp64(orc, v, t, q, r)
    print(f"leaf compaction K={K} leaf={leaf}: {stats}")
    assert m.device_status() == 0


def test_query_options_do_not_change_results(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.heightfield(128, seed=3)
    q = W.heightfield_queries(v, t, 50000, seed=4)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    qd = dev(q, cuda)
    base = m.query(qd, want_bary=True, opts=cpq.query_opts(traversal="thread"))
    for kw in [dict(sort_queries=False, traversal="thread"), dict(block_size=128, traversal="thread"),
               dict(block_size=64, short_stack=4, traversal="thread"),
               dict(short_stack=16, traversal="thread"), dict(blocks_per_sm=1, traversal="thread")]:
        r = m.query(qd, want_bary=True, opts=cpq.query_opts(**kw))
        assert torch.equal(r.dist, base.dist), kw
        assert torch.equal(r.tri, base.tri), kw
        assert torch.equal(r.point, base.point), kw
    # the warp-packet kernel visits nodes in another order: every triangle
    # closer than the answer is still tested, so results agree up to exact
    # FP32 ties of the traversal distance
    for kw in [dict(traversal="packet"), dict(traversal="packet", sort_queries=False),
               dict(traversal="packet", block_size=64), dict(traversal="auto")]:
        r = m.query(qd, want_bary=True, opts=cpq.query_opts(**kw))
        same = r.tri == base.tri
        # exact ties (a closest point on a grid vertex or edge shared by
        # several triangles, whose box bound equals the tied distance) resolve
        # by visit order; the distances must agree everywhere
        assert float(same.float().mean()) > 0.9, kw
        assert torch.equal(r.dist[same], base.dist[same]), kw
        rel = ((r.dist - base.dist).abs() / base.dist.clamp_min(1e-30)).max()
        assert float(rel) <= 1e-6, kw


def test_query_heightfield_sampled(orc, cpq, cuda):
    """The large workload's mesh at full size; FP64 checked on a seeded sample."""
    from gpurt_cpq import workloads as W

    v, t = W.heightfield(1024, seed=1)
    q = W.heightfield_queries(v, t, 1 << 20, seed=2)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    r = m.query(dev(q, cuda))
    idx = np.random.default_rng(0).choice(q.shape[0], 65536, replace=False)
    ref = orc.exact_f64(v, t, q[idx])

    class Sub:
        pass

    s = Sub()
    s.dist, s.tri, s.point = r.dist[idx], r.tri[idx], r.point[idx]
    stats = check_against_fp64(orc, v, t, q[idx], s, ref=ref)
    print(f"heightfield 1024^2 sample: {stats}")


def test_full_size_properties(cpq, cuda):
    """Size-independent checks on every query of the 16M-query large workload:
    p lies on the reported triangle at the reported barycentrics, |q - p| is
    the reported distance, and the answer is no farther than a probe triangle."""
    import torch

    from gpurt_cpq import workloads as W

    v, t, q = W.large()
    vd, td, qd = dev(v, cuda), dev(t, cuda), dev(q, cuda)
    m = cpq.Mesh(vd, td, branching=4, leaf_size=4)
    r = m.query(qd, want_bary=True)
    assert int((r.tri < 0).sum()) == 0
    tri = td[r.tri.long()].long()
    a, b, c = vd[tri[:, 0]].double(), vd[tri[:, 1]].double(), vd[tri[:, 2]].double()
    bv, bw = r.bary[:, 0:1].double(), r.bary[:, 1:2].double()
    p = a + bv * (b - a) + bw * (c - a)
    assert float((p - r.point.double()).norm(dim=1).max()) < 1e-5
    d = (qd.double() - r.point.double()).norm(dim=1)
    # the FP32 rounding of the reported point bounds the difference
    assert float(((d - r.dist.double()).abs() - 1e-6 * d).max()) < 5e-7
    # the distance to triangle 0 bounds every answer from above
    probe = (qd.double() - vd[td[0, 0].long()].double()).norm(dim=1)
    assert bool((r.dist.double() <= probe + 1e-6).all())
    assert m.device_status() == 0
    del tri, a, b, c, p, d, probe
    torch.cuda.empty_cache()


def test_reference_meshes(orc, cpq, cuda):
    g = np.load(GOLDEN / "ref_meshes.npz")
    vo, to, qo = g["vert_offsets"], g["tri_offsets"], g["q_offsets"]
    for mi in range(len(to) - 1):
        v = g["verts"][vo[mi]:vo[mi + 1]]
        t = g["tris"][to[mi]:to[mi + 1]]
        q = g["queries"][qo[mi]:qo[mi + 1]]
        ref = {"dist": g["dist"][qo[mi]:qo[mi + 1]], "tri": g["tri"][qo[mi]:qo[mi + 1]]}
        ref.update({k: orc.brute_f64(v, t, q)[k] for k in ("point",)})
        m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
        check_against_fp64(orc, v, t, q, m.query(dev(q, cuda)), ref=ref)


def test_degenerate_triangles(orc, cpq, cuda):
    rng = np.random.default_rng(2)
    v = rng.normal(size=(300, 3)).astype(np.float32)
    t = rng.integers(0, 300, (1000, 3)).astype(np.int32)
    v[:3] = [[0, 0, 0], [1, 0, 0], [2, 0, 0]]
    t[:20] = [0, 1, 2]           # collinear
    t[20:40] = [[5, 5, 6]]       # repeated vertex
    t[40:60] = [[7, 7, 7]]       # a point
    q = (rng.normal(size=(20000, 3)) * 1.5).astype(np.float32)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    check_against_fp64(orc, v, t, q, m.query(dev(q, cuda)))


def _check_near_surface(orc, v, t, q, res, strict_from):
    """Queries at distances down to 1e-9 of the triangle size.

    The winner is re-evaluated in float-float, so its distance is right to
    ~1e-7 however close the query is.  The winner is CHOSEN by the FP32 test,
    whose error is a few ulps of the triangle's size L: where several
    triangles lie within that of the closest one (a query almost on a shared
    edge or vertex), a neighbour can be chosen.  For a sliver the FP32 face
    test is ill-conditioned and its edges bound it instead, within half its
    width h.  So every answer is at least the true distance (to 1e-6 relative)
    and exceeds it by at most 1e-6 relative + 4e-7 L + h / 2; from
    `strict_from` * L on (and for triangles wider than 2e-2 L), within 1e-6
    relative.
    """
    ref = orc.exact_f64(v, t, q)
    d = res.dist.cpu().numpy().astype(np.float64)
    rd = ref["dist"]
    tv = v[t[ref["tri"]]].astype(np.float64)
    edges = np.linalg.norm(tv - np.roll(tv, 1, axis=1), axis=2)
    size = edges.max(axis=1)
    width = np.linalg.norm(np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]), axis=1) / size
    assert np.all(d >= rd * (1 - 1e-6) - 1e-12 * size), "below the true distance"
    excess = d - rd * (1 + 1e-6)
    allowed = 4e-7 * size + 0.5 * width
    assert np.all(excess <= allowed), f"excess {np.max(excess / allowed):.2f} of the allowed bound"
    far = (rd >= strict_from * size) & (width >= 2e-2 * size)
    rel = np.abs(d - rd) / np.maximum(rd, 1e-300)
    assert rel[far].max(initial=0) <= 1e-6, f"max rel err {rel[far].max()} beyond {strict_from} L"
    return {"max_rel_strict": float(rel[far].max(initial=0)), "strict": int(far.sum()),
            "max_excess_over_L": float(np.max(excess / size)), "n": int(len(d))}


def test_queries_very_close_to_faces_edges_vertices(orc, cpq, cuda):
    """Distances from 1e-9 to 1e-1 of the triangle size, above face interiors,
    edges and vertices, where an FP32 residual would lose all its digits."""
    from gpurt_cpq import workloads as W

    v, t = W.heightfield(64, seed=9)
    rng = np.random.default_rng(21)
    n = 24000
    tri = rng.integers(0, t.shape[0], n)
    a, b, c = (v[t[tri, k]].astype(np.float64) for k in range(3))
    kind = rng.integers(0, 3, n)                  # 0 face, 1 edge ab, 2 vertex a
    u1, u2 = rng.random(n), rng.random(n)
    s = np.sqrt(u1)
    bw = np.where((kind == 0)[:, None],
                  (1 - s)[:, None] * a + (s * (1 - u2))[:, None] * b + (s * u2)[:, None] * c,
                  np.where((kind == 1)[:, None], (1 - u1)[:, None] * a + u1[:, None] * b, a))
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    size = np.linalg.norm(b - a, axis=1)
    d = size * 10.0 ** rng.uniform(-9, -1, n) * np.where(rng.random(n) < 0.5, -1, 1)
    q = (bw + d[:, None] * nrm).astype(np.float32)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    stats = _check_near_surface(orc, v, t, q, m.query(dev(q, cuda)), strict_from=1e-2)
    print(f"very close: {stats}")


def test_queries_near_thin_triangles(orc, cpq, cuda):
    """Slivers (angles of 0.05 to 1 degree), queries 1e-7 to 1e-1 away:
    ill-conditioned barycentrics in the float-float re-evaluation."""
    rng = np.random.default_rng(22)
    k = 400
    base = rng.normal(size=(k, 3))
    e1 = rng.normal(size=(k, 3))
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = rng.normal(size=(k, 3))
    e2 -= (e2 * e1).sum(1, keepdims=True) * e1
    e2 /= np.linalg.norm(e2, axis=1, keepdims=True)
    ang = np.radians(rng.uniform(0.05, 1.0, k))
    vs = np.concatenate([base, base + e1, base + np.cos(ang)[:, None] * e1 + np.sin(ang)[:, None] * e2])
    ts = np.stack([np.arange(k), k + np.arange(k), 2 * k + np.arange(k)], 1).astype(np.int32)
    vs = vs.astype(np.float32)
    pick = rng.integers(0, k, 8000)
    w = rng.dirichlet([1, 1, 1], 8000)
    p = w[:, :1] * vs[ts[pick, 0]] + w[:, 1:2] * vs[ts[pick, 1]] + w[:, 2:] * vs[ts[pick, 2]]
    qs = (p + rng.normal(size=p.shape) * 10.0 ** rng.uniform(-7, -1, (8000, 1))).astype(np.float32)
    ms = cpq.Mesh(dev(vs, cuda), dev(ts, cuda), branching=4, leaf_size=4)
    stats = _check_near_surface(orc, vs, ts, qs, ms.query(dev(qs, cuda)), strict_from=1e-2)
    print(f"thin triangles: {stats}")


def test_queries_on_surface_and_far(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(4)
    far = np.array([[1e4, 0, 0], [0, -3e4, 1e4], [123.5, 77.25, -1000]], np.float32)
    q = np.concatenate([v[:500], far]).astype(np.float32)   # exactly on vertices, then far away
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=8)
    check_against_fp64(orc, v, t, q, m.query(dev(q, cuda)))


def test_edge_cases(cpq, cuda):
    import torch

    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE, CP_ERROR_SCRATCH_TOO_SMALL, CpError
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(2)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda))
    empty = torch.empty((0, 3), dtype=torch.float32, device=cuda)
    r = m.query(empty)
    assert r.dist.numel() == 0
    one = m.query(dev(np.array([[0, 0, 2]], np.float32), cuda))
    assert abs(float(one.dist.cpu()[0]) - 1.0) < 1e-3
    # a NaN query finds nothing: tri -1, NaN distance, and the status bit
    nan = m.query(dev(np.array([[np.nan, 0, 0], [0, 0, 3]], np.float32), cuda))
    assert int(nan.tri.cpu()[0]) == -1 and np.isnan(float(nan.dist.cpu()[0]))
    assert int(nan.tri.cpu()[1]) >= 0
    assert m.device_status() & 0x4
    assert m.device_status() == 0
    # too small a workspace is refused before any launch
    q = dev(W.uniform_queries(1000, -1, 1, 0), cuda)
    ws = torch.empty(16, dtype=torch.uint8, device=cuda)
    with pytest.raises(CpError) as e:
        m.query(q, workspace=ws)
    assert e.value.status == CP_ERROR_SCRATCH_TOO_SMALL
    # caller-provided workspace of the reported size works
    ws = torch.empty(m.workspace_size(1000), dtype=torch.uint8, device=cuda)
    assert torch.equal(m.query(q, workspace=ws).dist, m.query(q).dist)
    # invalid meshes are refused with a status, not a fault
    bad = t.copy()
    bad[3, 1] = v.shape[0] + 5
    with pytest.raises(CpError) as e:
        cpq.Mesh(dev(v, cuda), dev(bad, cuda))
    assert e.value.status == CP_ERROR_INVALID_VALUE
    bad[3, 1] = -1
    with pytest.raises(CpError):
        cpq.Mesh(dev(v, cuda), dev(bad, cuda))
    vn = v.copy()
    vn[7, 2] = np.inf
    with pytest.raises(CpError) as e:
        cpq.Mesh(dev(vn, cuda), dev(t, cuda))
    assert e.value.status == CP_ERROR_INVALID_VALUE
    with pytest.raises(CpError):
        cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=3)
    with pytest.raises(CpError):
        cpq.Mesh(dev(v, cuda), dev(t, cuda), leaf_size=16)


def test_host_buffers_match_device(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.torus(100, 40)
    q = W.uniform_queries(200000, -1.5, 1.5, 8)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    d = m.query(dev(q, cuda), want_bary=True)
    h = m.query_host(torch.from_numpy(q).pin_memory(), want_bary=True)
    assert torch.equal(h["dist"], d.dist.cpu())
    assert torch.equal(h["tri"], d.tri.cpu())
    assert torch.equal(h["point"], d.point.cpu())
    assert torch.equal(h["bary"], d.bary.cpu())


def test_host_buffers_two_chunks(cpq, cuda):
    """Past 64M queries the host path pipelines chunks on two streams; the
    answers are those of one device call (each query's answer does not depend
    on the ordering, only ties between equal distances may pick another
    triangle)."""
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.torus(100, 40)
    nq = (1 << 26) + 4097
    q = torch.from_numpy(W.uniform_queries(nq, -1.5, 1.5, 9)).pin_memory()
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    h = m.query_host(q)
    d = m.query(q.to(cuda))
    torch.testing.assert_close(h["dist"], d.dist.cpu(), rtol=1e-6, atol=0)
    assert (h["tri"] == d.tri.cpu()).float().mean() > 0.9999
    del d, h


def test_host_buffers_async_two_streams(cpq, cuda):
    """cp_query_host_async: batches alternating over two streams (one batch's
    copies under the other's kernels) give the device call's answers bit for
    bit; every output set is written by its own batch; unpinned host arrays
    are refused before anything is enqueued."""
    import torch

    from gpurt_cpq import CpError
    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE

    v, t = W.torus(100, 40)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    batches = [torch.from_numpy(W.uniform_queries(150_000 + 1000 * k, -1.5, 1.5, 20 + k)).pin_memory()
               for k in range(5)]
    want = [m.query(b.to(cuda), want_bary=True) for b in batches]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]

    def outs(n):
        return {"dist": torch.full((n,), -1.0).pin_memory(), "tri": torch.full((n,), -7, dtype=torch.int32).pin_memory(),
                "point": torch.empty((n, 3)).pin_memory(), "bary": torch.empty((n, 2)).pin_memory()}

    got = [outs(b.shape[0]) for b in batches]
    for k, b in enumerate(batches):
        m.query_host_async(b, got[k], stream=streams[k % 2])
    for s in streams:
        s.synchronize()
    for g, w in zip(got, want):
        assert torch.equal(g["dist"], w.dist.cpu())
        assert torch.equal(g["tri"], w.tri.cpu())
        assert torch.equal(g["point"], w.point.cpu())
        assert torch.equal(g["bary"], w.bary.cpu())
    # pageable input or output: refused
    with pytest.raises(CpError) as e:
        m.query_host_async(batches[0].clone(), outs(batches[0].shape[0]))
    assert e.value.status == CP_ERROR_INVALID_VALUE
    page = {"dist": torch.empty(batches[0].shape[0]), "tri": torch.empty(batches[0].shape[0], dtype=torch.int32)}
    with pytest.raises(CpError):
        m.query_host_async(batches[0], page)
    # each of the call's device allocations failing in turn: out of memory,
    # what it held released, and the next call answers
    from gpurt_cpq._lib import CP_ERROR_OUT_OF_MEMORY, lib
    for k in range(6):
        lib.cp_debug_fail_allocation(k)
        try:
            with pytest.raises(CpError) as e:
                m.query_host_async(batches[0], got[0])
            assert e.value.status == CP_ERROR_OUT_OF_MEMORY, k
        finally:
            lib.cp_debug_fail_allocation(-1)
    torch.cuda.synchronize()
    m.query_host_async(batches[1], got[1])
    torch.cuda.synchronize()
    assert torch.equal(got[1]["dist"], want[1].dist.cpu())
    assert m.device_status() == 0


def test_refit_moves_vertices(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(4)
    rng = np.random.default_rng(1)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    before = m.export_build()
    v2 = (v * 1.3 + rng.normal(0, 0.02, v.shape)).astype(np.float32)
    m.refit(dev(v2, cuda))
    q = W.uniform_queries(30000, -2.5, 2.5, 3)
    check_against_fp64(orc, v2, t, q, m.query(dev(q, cuda)))
    after = m.export_build()
    np.testing.assert_array_equal(before["order"], after["order"])
    # every wide box still contains the triangles below it
    w = m.export_wide()
    K = 4
    boxes = w["boxes"].reshape(-1, 6, K)
    order = after["order"]
    for node in range(0, boxes.shape[0], 7):
        for s in range(K):
            c = w["counts"][node * K + s]
            if c > 0:
                f = w["refs"][node * K + s]
                pts = v2[t[order[f:f + c]]].reshape(-1, 3)
                lo, hi = boxes[node, 0::2, s], boxes[node, 1::2, s]
                assert np.all(pts >= lo) and np.all(pts <= hi)


def test_autotuner_picks_valid_options_and_caches(orc, cpq, cuda, tmp_path):
    """cp_autotune times candidates on the given mesh and queries, returns
    options the library accepts, writes one line per size class and
    branching to its cache, and answers a second call from the cache with the
    same choice; the tuned mesh answers within the FP64 bound."""
    import time

    from gpurt_cpq import workloads as W

    v, t = W.torus(120, 48)
    q = W.uniform_queries(200000, -1.5, 1.5, 31)
    vd, td, qd = dev(v, cuda), dev(t, cuda), dev(q, cuda)
    cache = tmp_path / "tune.txt"
    t0 = time.perf_counter()
    bo, qo = cpq.autotune(vd, td, qd, cache_path=str(cache), branching=4)
    first = time.perf_counter() - t0
    assert bo.branching == 4 and 1 <= bo.leaf_size <= 15
    assert 32 <= qo.block_size <= 256 and qo.block_size % 32 == 0
    assert qo.traversal in (1, 2)
    lines = [ln.split() for ln in cache.read_text().splitlines() if ln.strip() and not ln.startswith("#")]
    assert len(lines) == 1 and int(lines[0][2]) == 4
    assert (int(lines[0][0]), int(lines[0][1])) == (cpq.lib.cp_size_class(len(t)), cpq.lib.cp_size_class(len(q)))
    t0 = time.perf_counter()
    bo2, qo2 = cpq.autotune(vd, td, qd, cache_path=str(cache), branching=4)
    assert time.perf_counter() - t0 < first
    assert (bo2.leaf_size, qo2.block_size, qo2.traversal, qo2.short_stack) == \
        (bo.leaf_size, qo.block_size, qo.traversal, qo.short_stack)
    m = cpq.Mesh(vd, td, branching=bo.branching, leaf_size=bo.leaf_size)
    d = m.query(qd[:8192], opts=qo).dist.cpu().numpy()
    ref = orc.exact_f64(v, t, q[:8192])["dist"]
    assert (np.abs(d - ref) / ref).max() <= 1e-6


def test_timing_and_counters(cpq, cuda):
    """cp_timing_enable(EVENTS) brackets each traversal launch with events
    (cp_timing_read: device ms and launch count, reset on read);
    cp_timing_enable(COUNTERS) runs the counting build, whose per-warp counts
    are consistent with the query; both off leave nothing recorded."""
    from ctypes import byref, c_double, c_int64, c_uint64

    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_TIMING_COUNTERS, CP_TIMING_EVENTS, lib

    v, t = W.torus(100, 40)
    q = dev(W.uniform_queries(65536, -1.5, 1.5, 41), cuda)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=8)
    o = cpq.query_opts(traversal="packet")
    ms, n = c_double(), c_int64()
    counts = (c_uint64 * 7)()
    try:
        assert lib.cp_timing_enable(CP_TIMING_EVENTS) == 0
        lib.cp_timing_read(byref(ms), byref(n), 1)
        for _ in range(3):
            m.query(q, opts=o)
        assert lib.cp_timing_read(byref(ms), byref(n), 1) == 0
        assert n.value == 3 and ms.value > 0.0
        assert lib.cp_timing_enable(CP_TIMING_COUNTERS) == 0
        lib.cp_traversal_stats(counts, 1)
        r = m.query(q, opts=o)
        assert lib.cp_traversal_stats(counts, 1) == 0
        nodes, leaf_tris, pops, skips, lane_tris, rounds, lane_nodes = list(counts)
        packets = 65536 // 32
        assert nodes >= packets and pops >= skips and leaf_tris >= rounds > 0
        assert lane_tris <= 32 * rounds and lane_nodes <= 32 * nodes
        assert r.dist.isfinite().all()
        lib.cp_timing_enable(0)
        lib.cp_timing_read(byref(ms), byref(n), 1)
        m.query(q, opts=o)
        lib.cp_timing_read(byref(ms), byref(n), 1)
        assert n.value == 0
    finally:
        lib.cp_timing_enable(0)


def test_allocation_failures_are_reported_and_release_memory(cpq, cuda):
    """Host-side fault injection (cp_debug_fail_allocation): a device
    allocation failing at any point of a build, or in a query's workspace,
    returns CP_ERROR_OUT_OF_MEMORY through the C ABI and releases what the
    call held; the hook disarms itself after firing.  The whole sweep runs
    twice: one-time growth (modules loaded on first use, memory pools) lands
    in the first pass, a leak would show again in the second."""
    import torch

    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_ERROR_OUT_OF_MEMORY, CpError, lib

    v, t = W.icosphere(3)
    vd, td = dev(v, cuda), dev(t, cuda)
    q = dev(W.uniform_queries(4096, -2, 2, 51), cuda)
    ref = cpq.Mesh(vd, td, branching=4).query(q).dist

    def sweep():
        failed_at = []
        for k in range(500):
            lib.cp_debug_fail_allocation(k)
            try:
                m = cpq.Mesh(vd, td, branching=4)
            except CpError as e:
                assert e.status == CP_ERROR_OUT_OF_MEMORY, e
                failed_at.append(k)
                # the hook fired and disarmed: the next build succeeds untouched
                cpq.Mesh(vd, td, branching=4).close()
                continue
            lib.cp_debug_fail_allocation(-1)
            break
        assert len(failed_at) >= 10 and failed_at == list(range(len(failed_at)))
        lib.cp_debug_fail_allocation(0)
        with pytest.raises(CpError) as e:
            m.query(q)  # its workspace comes from the pool: that allocation fails
        assert e.value.status == CP_ERROR_OUT_OF_MEMORY
        assert torch.equal(m.query(q).dist, ref)
        m.close()
        torch.cuda.synchronize()
        return torch.cuda.mem_get_info()[0]

    try:
        first = sweep()
        second = sweep()
    finally:
        lib.cp_debug_fail_allocation(-1)
    assert abs(second - first) < (16 << 20), (first, second)


@pytest.mark.parametrize("K,leaf", [(2, 2), (4, 8), (8, 4)])
def test_seeded_packets_change_no_answer(orc, cpq, cuda, K, leaf):
    """Packets claimed in chunks and seeded from the packet before them give
    the unseeded answers bit for bit (a seed is an upper bound with a margin
    far above the tests' errors), on a mesh and on a batch whose packets
    cross mesh boundaries; and they are FP64's."""
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.heightfield(256, seed=4)
    q = np.concatenate([W.heightfield_queries(v, t, 60_000, seed=5), W.uniform_queries(40_000, -0.2, 1.2, 6)])
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=leaf)
    qd = dev(q, cuda)
    base = m.query(qd, want_bary=True, opts=cpq.query_opts(seed_chunk=1))
    for chunk in (2, 4, 16):
        r = m.query(qd, want_bary=True, opts=cpq.query_opts(seed_chunk=chunk))
        for k in ("dist", "tri", "point", "bary"):
            assert torch.equal(getattr(r, k), getattr(base, k)), (chunk, k)
    check_against_fp64(orc, v, t, q[:20000], type(base)(point=base.point[:20000], dist=base.dist[:20000],
                                                         tri=base.tri[:20000], bary=None))
    meshes, queries = W.batched(seed=3, nmeshes=10, tri_range=(200, 20000), q_range=(100, 8000))
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    b = cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=K, leaf_size=leaf)
    b1 = b.query(dev(Q, cuda), qoff, opts=cpq.query_opts(seed_chunk=1))
    b4 = b.query(dev(Q, cuda), qoff, opts=cpq.query_opts(seed_chunk=4))
    assert torch.equal(b1.dist, b4.dist) and torch.equal(b1.tri, b4.tri)
    assert m.device_status() == 0
