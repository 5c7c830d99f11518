"""CPU tests: pin the oracle against hand-computed answers and check the FP32
restatement of the build for structural invariants.  No GPU needed."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def kats():
    return json.loads((GOLDEN / "kat_point_triangle.json").read_text())


@pytest.mark.parametrize("case", kats()["cases"], ids=lambda c: str(c["q"]))
def test_kat_point_triangle_f64(orc, case):
    d2, cp, w = orc.point_tri_f64(case["q"], case["a"], case["b"], case["c"])
    assert np.sqrt(d2) == pytest.approx(case["dist"], rel=1e-12, abs=1e-12)
    np.testing.assert_allclose(cp, case["point"], rtol=0, atol=1e-12)
    if case["bary"] is not None:
        np.testing.assert_allclose(w, case["bary"], rtol=0, atol=1e-12)
    assert abs(w.sum() - 1.0) < 1e-12


def test_kat_tie_smallest_index(orc):
    tm = kats()["tie_mesh"]
    v = np.array(tm["verts"], np.float32)
    t = np.array(tm["tris"], np.int32)
    q = np.array(tm["queries"], np.float32)
    for fn in (orc.brute_f64, orc.exact_f64):
        r = fn(v, t, q)
        np.testing.assert_array_equal(r["tri"], tm["tri"])
        np.testing.assert_allclose(r["dist"], tm["dist"], rtol=1e-12)


def random_mesh(rng, nt, nv, degenerate=0):
    v = rng.normal(size=(nv, 3)).astype(np.float32)
    t = rng.integers(0, nv, (nt, 3)).astype(np.int32)
    if degenerate:
        # collinear and repeated-vertex triangles
        v[:3] = [[0, 0, 0], [1, 0, 0], [2, 0, 0]]
        t[:degenerate] = [0, 1, 2]
        t[degenerate:2 * degenerate] = [[3, 3, 4]]
    return v, t


def test_exact_search_equals_brute_force(orc):
    rng = np.random.default_rng(11)
    v, t = random_mesh(rng, 3000, 1200, degenerate=5)
    q = (rng.normal(size=(4000, 3)) * 1.5).astype(np.float32)
    a, b = orc.brute_f64(v, t, q), orc.exact_f64(v, t, q)
    np.testing.assert_array_equal(a["d2"], b["d2"])
    np.testing.assert_array_equal(a["tri"], b["tri"])


def test_golden_small_sample(orc):
    """The small workload regenerated here equals the committed fixture bit for bit."""
    from gpurt_cpq import workloads as W

    g = np.load(GOLDEN / "small_sample.npz")
    v, t, q = W.small()
    np.testing.assert_array_equal(v, g["verts"])
    np.testing.assert_array_equal(t, g["tris"])
    np.testing.assert_array_equal(q[:4096], g["queries"])
    r = orc.brute_f64(v, t, g["queries"])
    np.testing.assert_array_equal(r["tri"], g["tri"])
    np.testing.assert_allclose(r["dist"], g["dist"], rtol=1e-15)


def test_golden_reference_meshes(orc):
    g = np.load(GOLDEN / "ref_meshes.npz")
    vo, to, qo = g["vert_offsets"], g["tri_offsets"], g["q_offsets"]
    for m in range(len(to) - 1):
        v = g["verts"][vo[m]:vo[m + 1]]
        t = g["tris"][to[m]:to[m + 1]]
        q = g["queries"][qo[m]:qo[m + 1]]
        r = orc.exact_f64(v, t, q)
        np.testing.assert_array_equal(r["tri"], g["tri"][qo[m]:qo[m + 1]])
        np.testing.assert_allclose(r["dist"], g["dist"][qo[m]:qo[m + 1]], rtol=1e-15)


def check_tree_invariants(tree, nmeshes=1, toff=None):
    n = tree.nt
    nn = 2 * n - 1
    # the sorted keys ascend and the order is a permutation
    assert np.all(np.diff(tree.keys.astype(np.float64)) >= 0) or np.all(tree.keys[1:] >= tree.keys[:-1])
    assert np.array_equal(np.sort(tree.order), np.arange(n))
    if n > 1:
        # every internal node's range is the union of its children's ranges
        for i in range(n - 1):
            l, r = tree.left[i], tree.right[i]
            assert tree.first[i] == tree.first[l] and tree.last[i] == tree.last[r]
            assert tree.last[l] + 1 == tree.first[r]
            assert tree.parent[l] == i and tree.parent[r] == i
    assert (tree.parent == -1).sum() == 1
    # boxes: parents contain children
    if n > 1:
        b = tree.box
        for i in range(n - 1):
            for c in (tree.left[i], tree.right[i]):
                assert np.all(b[i, :3] <= b[c, :3]) and np.all(b[i, 3:] >= b[c, 3:])
    # clusters partition the sorted triangles of each mesh
    covered = np.zeros(n, np.int32)
    for v in np.nonzero(tree.cluster)[0]:
        covered[tree.first[v]:tree.last[v] + 1] += 1
        assert tree.last[v] - tree.first[v] + 1 <= max(tree.wide_count.max(), 1)
    assert np.all(covered == 1)
    # the wide tree reaches every triangle exactly once
    K = tree.K
    hit = np.zeros(n, np.int32)
    inner_refs = []
    for w in range(tree.num_wide):
        for s in range(K):
            c = tree.wide_count[w * K + s]
            if c > 0:
                hit[tree.wide_ref[w * K + s]:tree.wide_ref[w * K + s] + c] += 1
            elif c == 0:
                inner_refs.append(tree.wide_ref[w * K + s])
    assert np.all(hit == 1)
    assert len(set(inner_refs)) == len(inner_refs)
    assert len(inner_refs) + nmeshes == tree.num_wide
    assert tree.stack_bound == (K - 1) * (tree.max_wide_depth + 1)


@pytest.mark.parametrize("K", [2, 4, 8])
@pytest.mark.parametrize("leaf,collapse", [(1, 0), (4, 0), (8, 1), (15, 0)])
def test_restatement_invariants(orc, K, leaf, collapse):
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(3)
    tree = orc.Tree(v, t, K, leaf, collapse)
    check_tree_invariants(tree)


def test_restatement_duplicate_centroids(orc):
    # every triangle identical: keys all equal, the index tie-break builds the tree
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.zeros((300, 3), np.int32) + np.array([0, 1, 2], np.int32)
    tree = orc.Tree(v, t, 4, 4, 0)
    assert np.all(tree.keys == tree.keys[0])
    check_tree_invariants(tree)


@pytest.mark.parametrize("nt", [1, 2, 3])
def test_restatement_tiny(orc, nt):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [2, 2, 2]], np.float32)
    t = np.array([[0, 1, 2], [1, 3, 2], [2, 3, 4]], np.int32)[:nt]
    tree = orc.Tree(v, t, 4, 1, 0)
    check_tree_invariants(tree)
    q = np.array([[0.5, 0.5, 1], [3, 3, 3]], np.float32)
    r = tree.query(q)
    e = orc.brute_f64(v, t, q)
    np.testing.assert_allclose(r["dist"], e["dist"], rtol=1e-6)


def ties_ok(orc, v, t, q, tri, ref, rel=1e-6):
    """Indices equal except where FP64 confirms a tie within `rel`."""
    mm = np.nonzero(tri != ref["tri"])[0]
    if len(mm) == 0:
        return True, 0, 0.0
    d = orc.dist_to_tri_f64(v, t, q[mm], tri[mm])
    gap = (d - ref["dist"][mm]) / np.maximum(ref["dist"][mm], 1e-30)
    return bool(np.all(gap <= rel)), len(mm), float(gap.max())


@pytest.mark.parametrize("K", [2, 4, 8])
def test_restatement_query_small(orc, K):
    from gpurt_cpq import workloads as W

    v, t, q = W.small(nq=8192)
    tree = orc.Tree(v, t, K, 4, 0)
    r = tree.query(q)
    e = orc.brute_f64(v, t, q)
    rel = np.abs(r["dist"] - e["dist"]) / np.maximum(e["dist"], 1e-30)
    assert rel.max() <= 1e-6
    ok, n, gap = ties_ok(orc, v, t, q, r["tri"], e)
    assert ok, (n, gap)


def test_restatement_batch(orc):
    g = np.load(GOLDEN / "ref_meshes.npz")
    tree = orc.Tree(g["verts"], g["tris"], 4, 4, 0, vert_offsets=g["vert_offsets"],
                    tri_offsets=g["tri_offsets"])
    check_tree_invariants(tree, nmeshes=len(g["tri_offsets"]) - 1)
    qo = g["q_offsets"]
    q_mesh = np.repeat(np.arange(len(qo) - 1), np.diff(qo)).astype(np.int32)
    r = tree.query(g["queries"], q_mesh=q_mesh)
    rel = np.abs(r["dist"] - g["dist"]) / np.maximum(g["dist"], 1e-30)
    assert rel.max() <= 1e-6


def test_backward_f64_matches_finite_differences(orc):
    from gpurt_cpq import workloads as W

    v, t = W.torus(40, 16)
    rng = np.random.default_rng(3)
    q = rng.uniform(-1.5, 1.5, (200, 3)).astype(np.float32)
    e = orc.brute_f64(v, t, q)
    g = rng.normal(size=200)
    gq, gv = orc.backward_f64(v, t, q, e["tri"], e["bary"], g)
    # d/dq by central differences in FP64 (queries perturbed in float64 via scaled copies)
    h = 1e-4
    for k in range(3):
        qp = q.astype(np.float64).copy(); qp[:, k] += h
        qm = q.astype(np.float64).copy(); qm[:, k] -= h
        dp = np.array([np.sqrt(min(orc.point_tri_f64(x, v[a], v[b], v[c])[0] for a, b, c in t))
                       for x in qp[:20]])
        dm = np.array([np.sqrt(min(orc.point_tri_f64(x, v[a], v[b], v[c])[0] for a, b, c in t))
                       for x in qm[:20]])
        fd = g[:20] * (dp - dm) / (2 * h)
        np.testing.assert_allclose(gq[:20, k], fd, atol=1e-5, rtol=1e-4)


# ---------------------------------------------------------------- rays

def test_ray_known_answers(orc):
    """Hand-computed hits on the unit right triangle (0,0,0), (1,0,0), (0,1,0)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.int32)
    o = np.array([[0.25, 0.25, 1], [0.25, 0.25, 1], [2, 2, 1], [0.25, 0.25, -1], [0.5, 0.25, 3],
                  [-1, 0.25, 0]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1], [0, 0, -1], [0, 0, 2], [0, 0, -0.5], [1, 0, 0]], np.float32)
    for fp64 in (False, True):
        r = orc.ray_brute(v, t, o, d, fp64=fp64)
        np.testing.assert_array_equal(r["tri"], [0, -1, -1, 0, 0, -1])  # last: in the plane, det = 0
        np.testing.assert_allclose(r["t"][[0, 3, 4]], [1.0, 0.5, 6.0])
        np.testing.assert_allclose(r["uv"][[0, 3, 4]], [[0.25, 0.25], [0.25, 0.25], [0.5, 0.25]])
        # [tmin, tmax] and per-ray ends
        r = orc.ray_brute(v, t, o, d, tmin=0.0, tmax=0.9, fp64=fp64)
        np.testing.assert_array_equal(r["tri"], [-1, -1, -1, 0, -1, -1])
        r = orc.ray_brute(v, t, o, d, tmax_per_ray=np.full(6, 5.0, np.float32), fp64=fp64)
        np.testing.assert_array_equal(r["tri"], [0, -1, -1, 0, -1, -1])


def test_ray_reference_epsilon_rejects_small_triangles(orc):
    """triangle_hit's |det| < 1e-5 (a scene-scale constant): a triangle of
    size 1e-3 is missed with it and hit without it."""
    v = np.array([[0, 0, 0], [1e-3, 0, 0], [0, 1e-3, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.int32)
    o = np.array([[2.5e-4, 2.5e-4, 1]], np.float32)
    d = np.array([[0, 0, -1]], np.float32)
    assert orc.ray_brute(v, t, o, d)["tri"][0] == 0
    assert orc.ray_brute(v, t, o, d, det_eps=1e-5)["tri"][0] == -1


def test_ray_f32_agrees_with_f64(orc):
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(2)
    rng = np.random.default_rng(4)
    o = rng.uniform(-2, 2, (3000, 3)).astype(np.float32)
    d = rng.normal(size=(3000, 3)).astype(np.float32)
    a = orc.ray_brute(v, t, o, d)
    b = orc.ray_brute(v, t, o, d, fp64=True)
    same = a["tri"] == b["tri"]
    assert same.mean() > 0.99
    both = same & (a["tri"] >= 0)
    np.testing.assert_allclose(a["t"][both], b["t"][both], rtol=1e-5, atol=1e-6)


def test_fp64_vertex_brute_forces_match_fp32_vertex_ones(orc):
    """The FP64-vertex brute forces (for instanced scenes) give the same
    answers as the FP32-vertex ones when the vertices are FP32 values."""
    import numpy as np

    from gpurt_cpq import workloads as W

    v, t = W.icosphere(2)
    rng = np.random.default_rng(3)
    q = rng.uniform(-2, 2, (2000, 3)).astype(np.float32)
    a = orc.brute_f64(v, t, q)
    b = orc.brute_f64_dv(v.astype(np.float64), t, q)
    np.testing.assert_array_equal(a["tri"], b["tri"])
    np.testing.assert_array_equal(a["dist"], b["dist"])
    d = rng.normal(size=(2000, 3)).astype(np.float32)
    ra = orc.ray_brute(v, t, q, d, fp64=True)
    rb = orc.ray_brute_f64_dv(v.astype(np.float64), t, q, d)
    np.testing.assert_array_equal(ra["tri"], rb["tri"])
    hit = np.isfinite(ra["t"])
    np.testing.assert_array_equal(ra["t"][hit], rb["t"][hit])
    assert np.all(~np.isfinite(rb["t"][~hit]))
