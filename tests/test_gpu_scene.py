"""GPU instanced scenes (cp_scene_*): instances of a batch's meshes placed by
affine transforms, the reference's TLAS over transformed BLAS instances
(src/vk/vulkan.cpp:777-856, src/rt/rt.cpp:31-45).

The truth is the FP64 brute force over the world-space vertices, each the
FP32 matrix applied to the FP32 object vertex in FP64.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def random_similarities(n, seed, reflect=True):
    """(n, 3, 4) float32: random rotation (some reflected), scale 0.5..2, translation in [-4, 4]^3."""
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    if reflect:
        R[::3, :, 0] *= -1.0
    s = rng.uniform(0.5, 2.0, n)
    T = np.zeros((n, 3, 4))
    T[:, :, :3] = R * s[:, None, None]
    T[:, :, 3] = rng.uniform(-4, 4, (n, 3))
    return T.astype(np.float32)


def world_soup(meshes, inst_mesh, T):
    """All instances' triangles in world space, FP64 (the oracle's input)."""
    vs, ts, off = [], [], 0
    for m, t in zip(inst_mesh, T):
        v, tri = meshes[m]
        M = t.astype(np.float64)
        vs.append(v.astype(np.float64) @ M[:, :3].T + M[:, 3])
        ts.append(tri + off)
        off += v.shape[0]
    ntri = np.array([meshes[m][1].shape[0] for m in inst_mesh])
    return np.concatenate(vs), np.concatenate(ts).astype(np.int32), np.concatenate([[0], np.cumsum(ntri)])


def make_batch(cpq, cuda, meshes, K=4):
    from gpurt_cpq import workloads as W

    V, voff, T, toff, _, _ = W.concat_batch([(v, t, None) for v, t in meshes],
                                            [np.zeros((0, 3), np.float32)] * len(meshes))
    return cpq.Batch(dev(V, cuda), voff, dev(T, cuda), toff, branching=K)


def check_scene(orc, meshes, inst_mesh, T, q, r, rel=1e-6, scale=None):
    """`scale`: the length the near-surface allowance is relative to (default:
    the largest world coordinate)."""
    wv, wt, toff = world_soup(meshes, inst_mesh, T)
    ref = orc.brute_f64_dv(wv, wt, q)
    d = r.dist.cpu().numpy().astype(np.float64)
    inst = r.instance.cpu().numpy()
    tri = r.tri.cpu().numpy()
    assert np.all(inst >= 0) and np.all(tri >= 0)
    if scale is None:
        scale = np.abs(wv).max()
    # the answer is the distance to the reported triangle, never below the truth
    # by more than the float-float finish, and above it by at most the FP32
    # selection among near-equal triangles (~1e-7 of the coordinates)
    err = d - ref["dist"]
    assert np.all(err >= -1e-6 * ref["dist"] - 1e-12 * scale), err.min()
    far = ref["dist"] >= 1e-2 * scale
    assert np.all(err[far] <= rel * ref["dist"][far]), (err[far] / ref["dist"][far]).max()
    assert np.all(err <= rel * ref["dist"] + 4e-7 * scale), (err - rel * ref["dist"]).max()
    # the reported (instance, triangle) gives that distance and the point lies
    # on it, up to the FP32 rounding of the point's world coordinates
    coord = np.abs(wv).max()
    g = toff[inst] + tri
    pts = r.point.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(np.linalg.norm(pts - q, axis=1), d, rtol=2e-6, atol=2e-7 * coord)
    mm = np.nonzero(g != ref["tri"])[0]
    for i in mm[:200]:
        a, b, c = wv[wt[g[i]]]
        d2, _, _ = orc.point_tri_f64(q[i].astype(np.float64), a, b, c)
        assert abs(np.sqrt(d2) - d[i]) <= 1e-6 * d[i] + 1e-6 * scale
    for i in range(0, len(q), max(1, len(q) // 300)):
        a, b, c = wv[wt[g[i]]]
        d2, _, _ = orc.point_tri_f64(pts[i], a, b, c)
        assert np.sqrt(d2) <= 2e-7 * coord
    return ref


@pytest.mark.parametrize("K", [2, 4, 8])
def test_scene_vs_fp64(orc, cpq, cuda, K):
    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(3), W.torus(60, 24), W.heightfield(48, seed=3)[:2]]
    rng = np.random.default_rng(11)
    n = 37
    inst_mesh = rng.integers(0, len(meshes), n).astype(np.int32)
    T = random_similarities(n, seed=12)
    b = make_batch(cpq, cuda, meshes, K)
    sc = cpq.Scene(b, inst_mesh, T)
    wv, wt, _ = world_soup(meshes, inst_mesh, T)
    lo, hi = wv.min(0), wv.max(0)
    pad = 0.2 * (hi - lo)
    far = rng.uniform(lo - pad, hi + pad, (20000, 3))
    near = W.surface_points(wv.astype(np.float32), wt, 10000, rng).astype(np.float64)
    near += rng.normal(size=near.shape) * np.linalg.norm(hi - lo) * 10.0 ** rng.uniform(-6, -2, (len(near), 1))
    q = np.concatenate([far, near]).astype(np.float32)
    r = sc.query(dev(q, cuda), want_bary=True)
    check_scene(orc, meshes, inst_mesh, T, q, r)
    bary = r.bary.cpu().numpy()
    assert np.all(bary >= -1e-6) and np.all(bary.sum(1) <= 1 + 1e-6)


def test_scene_far_from_origin(orc, cpq, cuda):
    """Instances about 1000 units out: the object-space query is formed from
    q - t, so the accuracy near the surfaces is relative to the instances'
    size (~2), not to their world coordinates."""
    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(3), W.torus(60, 24)]
    rng = np.random.default_rng(41)
    n = 12
    inst_mesh = rng.integers(0, 2, n).astype(np.int32)
    T = random_similarities(n, seed=42)
    T[:, :, 3] = np.float32(1000.0) + rng.uniform(-6, 6, (n, 3)).astype(np.float32)
    sc = cpq.Scene(make_batch(cpq, cuda, meshes, 4), inst_mesh, T)
    wv, wt, _ = world_soup(meshes, inst_mesh, T)
    near = W.surface_points(wv.astype(np.float32), wt, 20000, rng).astype(np.float64)
    near += rng.normal(size=near.shape) * 10.0 ** rng.uniform(-2, 0, (len(near), 1))
    q = near.astype(np.float32)
    r = sc.query(dev(q, cuda), want_bary=True)
    # FP32 query coordinates near 1000 are themselves spaced 6e-5 apart; the
    # truth is for the FP32 queries as given
    check_scene(orc, meshes, inst_mesh, T, q, r, scale=4.0)


def test_scene_identity_matches_mesh(orc, cpq, cuda):
    """One instance at the identity gives the plain query's answers."""
    from gpurt_cpq import workloads as W

    v, t = W.torus(80, 30)
    b = make_batch(cpq, cuda, [(v, t)], 4)
    T = np.zeros((1, 3, 4), np.float32)
    T[0, :, :3] = np.eye(3)
    sc = cpq.Scene(b, [0], T)
    q = W.uniform_queries(30000, [-1.6, -1.6, -0.6], [1.6, 1.6, 0.6], seed=5)
    r = sc.query(dev(q, cuda))
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    rm = m.query(dev(q, cuda))
    np.testing.assert_allclose(r.dist.cpu().numpy(), rm.dist.cpu().numpy(), rtol=1e-6, atol=0)
    assert np.all(r.instance.cpu().numpy() == 0)
    same = (r.tri.cpu().numpy() == rm.tri.cpu().numpy()).mean()
    assert same > 0.99
    check_scene(orc, [(v, t)], [0], T, q, r)


def test_scene_many_instances_and_update(orc, cpq, cuda):
    """A few thousand small instances (deep top level), then new transforms."""
    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(1, 0.1), W.torus(12, 6, 0.1, 0.03)]
    rng = np.random.default_rng(21)
    n = 3000
    inst_mesh = rng.integers(0, 2, n).astype(np.int32)
    T = random_similarities(n, seed=22)
    T[:, :, 3] *= 5.0
    b = make_batch(cpq, cuda, meshes, 4)
    sc = cpq.Scene(b, inst_mesh, T)
    q = rng.uniform(-22, 22, (20000, 3)).astype(np.float32)
    check_scene(orc, meshes, inst_mesh, T, q, sc.query(dev(q, cuda)))
    T2 = random_similarities(n, seed=23)
    T2[:, :, 3] *= 5.0
    sc.update(T2)
    r = sc.query(dev(q, cuda))
    check_scene(orc, meshes, inst_mesh, T2, q, r)
    fresh = cpq.Scene(b, inst_mesh, T2).query(dev(q, cuda))
    assert np.array_equal(r.dist.cpu().numpy(), fresh.dist.cpu().numpy())


def test_scene_workspace_and_unsorted(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(2)]
    T = random_similarities(8, seed=2)
    sc = cpq.Scene(make_batch(cpq, cuda, meshes, 2), np.zeros(8, np.int32), T)
    q = dev(np.random.default_rng(1).uniform(-6, 6, (5000, 3)).astype(np.float32), cuda)
    r0 = sc.query(q)
    ws = torch.empty(sc.workspace_size(5000), dtype=torch.uint8, device=cuda)
    r1 = sc.query(q, workspace=ws)
    o = cpq.query_opts(sort_queries=False)
    r2 = sc.query(q, opts=o)
    assert torch.equal(r0.dist, r1.dist)
    torch.testing.assert_close(r0.dist, r2.dist, rtol=1e-6, atol=0)


def test_scene_general_affine(orc, cpq, cuda):
    """Instances that are not similarities — non-uniform scale, shear, a
    matrix that flattens the mesh onto a plane, the zero matrix — are walked
    through world-space copies, mixed with similarity instances in one scene."""
    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(2), W.torus(40, 16)]
    T = random_similarities(10, seed=5)
    T[1, :, :3] = T[1, :, :3] @ np.diag([3.0, 1.0, 0.5]).astype(np.float32)   # non-uniform scale
    T[2, 0, 1] += 0.7                                                          # shear
    T[3, :, :3] = T[3, :, :3] @ np.diag([1.0, 1.0, 0.0]).astype(np.float32)   # flattened
    T[4, :, :3] = 0.0                                                          # a point
    T[6, :, :3] = T[6, :, :3] @ np.diag([1.0, 2.0, 1.0]).astype(np.float32)
    inst_mesh = np.array([0, 1, 0, 1, 0, 1, 0, 1, 0, 1], np.int32)
    sc = cpq.Scene(make_batch(cpq, cuda, meshes, 4), inst_mesh, T)
    wv, wt, _ = world_soup(meshes, inst_mesh, T)
    rng = np.random.default_rng(6)
    lo, hi = wv.min(0), wv.max(0)
    far = rng.uniform(lo - 1, hi + 1, (15000, 3))
    near = W.surface_points(wv.astype(np.float32), wt, 15000, rng).astype(np.float64)
    near += rng.normal(size=near.shape) * 10.0 ** rng.uniform(-5, -1, (len(near), 1))
    q = np.concatenate([far, near]).astype(np.float32)
    r = sc.query(dev(q, cuda), want_bary=True)
    check_scene(orc, meshes, inst_mesh, T, q, r)
    assert set(np.unique(r.instance.cpu().numpy())) >= {1, 2, 3, 4, 6}
    # the update path re-bakes: swap two instances' matrices
    T2 = T.copy()
    T2[[1, 2]] = T[[2, 1]]
    sc.update(T2)
    check_scene(orc, meshes, inst_mesh, T2, q, sc.query(dev(q, cuda)))


def test_scene_refit_equals_rebuild(orc, cpq, cuda):
    """cp_scene_refit keeps the trees' topology (the reference's TLAS update);
    its answers are a freshly built scene's bit for bit, after every instance
    moved with its kind kept (similarities and general affine maps), and after
    two instances changed kind (the copies change: it rebuilds)."""
    import torch

    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(2), W.torus(40, 16)]
    n = 40
    inst_mesh = (np.arange(n) % 2).astype(np.int32)
    T = random_similarities(n, seed=31)
    T[5, :, :3] = T[5, :, :3] @ np.diag([3.0, 1.0, 0.5]).astype(np.float32)  # general affine
    T[9, 0, 1] += 0.7                                                         # shear
    b = make_batch(cpq, cuda, meshes, 4)
    sc = cpq.Scene(b, inst_mesh, T)
    q = np.random.default_rng(32).uniform(-7, 7, (30000, 3)).astype(np.float32)
    qd = dev(q, cuda)
    T2 = random_similarities(n, seed=33)
    T2[5, :, :3] = T2[5, :, :3] @ np.diag([2.0, 1.0, 0.7]).astype(np.float32)
    T2[9, 0, 1] += 0.4
    sc.refit(T2)
    r = sc.query(qd, want_bary=True)
    f = cpq.Scene(b, inst_mesh, T2).query(qd, want_bary=True)
    for k in ("dist", "point", "instance"):
        assert torch.equal(getattr(r, k), getattr(f, k)), k
    _same_or_tied(orc, meshes, inst_mesh, T2, q, r, f)
    check_scene(orc, meshes, inst_mesh, T2, q, r)
    T3 = T2.copy()
    T3[5] = random_similarities(1, seed=34)[0]                                 # general -> similarity
    T3[7, :, :3] = T3[7, :, :3] @ np.diag([1.0, 1.0, 2.0]).astype(np.float32)  # similarity -> general
    sc.refit(T3)
    r3 = sc.query(qd)
    f3 = cpq.Scene(b, inst_mesh, T3).query(qd)
    assert torch.equal(r3.dist, f3.dist) and torch.equal(r3.instance, f3.instance)
    _same_or_tied(orc, meshes, inst_mesh, T3, q, r3, f3)
    check_scene(orc, meshes, inst_mesh, T3, q, r3)


def _same_or_tied(orc, meshes, inst_mesh, T, q, r, f):
    """Equal triangles, except where the two trees met an exact tie in a
    different order: two triangles of one instance at the same distance
    (sharing the closest feature), whose boxes the walk may prune at equality
    depending on visit order.  There the FP64 distances agree to 1e-6."""
    tr, tf = r.tri.cpu().numpy(), f.tri.cpu().numpy()
    mm = np.nonzero(tr != tf)[0]
    assert len(mm) <= len(tr) // 100, len(mm)
    if len(mm) == 0:
        return
    wv, wt, toff = world_soup(meshes, inst_mesh, T)
    inst = r.instance.cpu().numpy()
    for i in mm:
        da = orc.point_tri_f64(q[i].astype(np.float64), *wv[wt[toff[inst[i]] + tr[i]]])[0]
        db = orc.point_tri_f64(q[i].astype(np.float64), *wv[wt[toff[inst[i]] + tf[i]]])[0]
        assert abs(np.sqrt(da) - np.sqrt(db)) <= 1e-6 * np.sqrt(db) + 1e-9, (i, da, db)


def test_scene_rejects_bad_input(cpq, cuda):
    from gpurt_cpq import workloads as W
    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE, CpError

    b = make_batch(cpq, cuda, [W.icosphere(1)], 4)
    T = random_similarities(2, seed=1)
    with pytest.raises(CpError, match="mesh id out of range") as e:
        cpq.Scene(b, [0, 1], T)
    assert e.value.status == CP_ERROR_INVALID_VALUE
    bad = T.copy()
    bad[1, 2, 3] = np.nan
    with pytest.raises(CpError, match="non-finite"):
        cpq.Scene(b, [0, 0], bad)
    sc = cpq.Scene(b, [0, 0], T)
    with pytest.raises(CpError, match="non-finite"):
        sc.update(bad)
    with pytest.raises(ValueError):
        sc.update(T[:1])


def _mt64(o, d, a, b, c):
    """FP64 Möller–Trumbore hit parameter of one ray and triangle (nan on a miss)."""
    e1, e2 = b - a, c - a
    p = np.cross(d, e2)
    det = e1 @ p
    if det == 0.0:
        return np.nan
    s = o - a
    u = (s @ p) / det
    q = np.cross(s, e1)
    v = (d @ q) / det
    if u < 0 or v < 0 or u + v > 1:
        return np.nan
    return (e2 @ q) / det


def _scene_rays(rng, wv, n):
    lo, hi = wv.min(0), wv.max(0)
    o = rng.uniform(lo - 1, hi + 1, (n, 3)).astype(np.float32)
    target = rng.uniform(lo, hi, (n, 3))
    d = (target - o).astype(np.float32)
    return o, d


def test_scene_rays_identity_matches_mesh(cpq, cuda):
    """One instance at the identity: the same hits, bit for bit, as the plain
    ray query on the mesh (identical object-space arithmetic)."""
    from gpurt_cpq import workloads as W

    v, t = W.torus(80, 30)
    T = np.zeros((1, 3, 4), np.float32)
    T[0, :, :3] = np.eye(3)
    sc = cpq.Scene(make_batch(cpq, cuda, [(v, t)], 4), [0], T)
    rng = np.random.default_rng(7)
    o, d = _scene_rays(rng, v.astype(np.float64), 30000)
    r = sc.ray_query(dev(o, cuda), dev(d, cuda))
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4).ray_query(dev(o, cuda), dev(d, cuda))
    assert torch_equal(r.t, m.t) and torch_equal(r.tri, m.tri) and torch_equal(r.uv, m.uv)
    assert np.all(r.instance.cpu().numpy()[m.tri.cpu().numpy() >= 0] == 0)


def torch_equal(a, b):
    import torch
    return bool(torch.equal(a, b))


@pytest.mark.parametrize("K", [2, 4, 8])
def test_scene_rays_vs_fp64(orc, cpq, cuda, K):
    """Similarity and general affine instances, rays aimed into the scene:
    hits against the FP64 brute force over world-space vertices."""
    from gpurt_cpq import workloads as W

    meshes = [W.icosphere(2), W.torus(40, 16)]
    T = random_similarities(12, seed=8)
    T[1, :, :3] = T[1, :, :3] @ np.diag([3.0, 1.0, 0.5]).astype(np.float32)
    T[2, 0, 1] += 0.7
    T[5, :, :3] = T[5, :, :3] @ np.diag([1.0, 1.0, 0.0]).astype(np.float32)
    inst_mesh = (np.arange(12) % 2).astype(np.int32)
    sc = cpq.Scene(make_batch(cpq, cuda, meshes, K), inst_mesh, T)
    wv, wt, toff = world_soup(meshes, inst_mesh, T)
    rng = np.random.default_rng(9)
    o, d = _scene_rays(rng, wv, 20000)
    r = sc.ray_query(dev(o, cuda), dev(d, cuda))
    ref = orc.ray_brute_f64_dv(wv, wt, o, d)
    t = r.t.cpu().numpy().astype(np.float64)
    inst, tri = r.instance.cpu().numpy(), r.tri.cpu().numpy()
    hit, hit64 = np.isfinite(t), np.isfinite(ref["t"])
    scale = 1.0 + np.abs(wv).max()
    # a hit or miss may differ only where the FP64 ray grazes a triangle's
    # boundary (barycentrics within 1e-4 of an edge) or the plane it hits
    for i in np.nonzero(hit != hit64)[0]:
        if hit64[i]:
            u, v = ref["uv"][i]
            assert min(u, v, 1 - u - v) < 1e-4, (i, u, v)
        else:
            g = toff[inst[i]] + tri[i]
            a, b, c = wv[wt[g]]
            t64 = _mt64(o[i].astype(np.float64), d[i].astype(np.float64), a, b, c)
            assert np.isnan(t64) or abs(t64 - t[i]) <= 1e-4 * scale, (i, t64, t[i])
    both = hit & hit64
    assert both.mean() > 0.3
    # the hit parameter: FP32 object-space arithmetic against FP64
    err = np.abs(t[both] - ref["t"][both])
    assert np.all(err <= 2e-5 * scale * (1.0 + ref["t"][both])), err.max()
    # another triangle than the FP64 one only where both are hit at the same t
    g = toff[inst] + tri
    for i in np.nonzero(both & (g != ref["tri"]))[0][:300]:
        a, b, c = wv[wt[g[i]]]
        t64 = _mt64(o[i].astype(np.float64), d[i].astype(np.float64), a, b, c)
        assert not np.isnan(t64) and abs(t64 - ref["t"][i]) <= 2e-5 * scale * (1 + ref["t"][i]), (i, t64)


def test_cbox_camera_rays_vs_fp64(orc, cpq, cuda):
    """The reference's Cornell box seen from its own camera (96 x 72 primary
    rays through the scene's instances) against the FP64 brute force."""
    from pathlib import Path

    from gpurt_cpq import workloads as W

    g = np.load(Path(__file__).resolve().parent / "golden" / "cbox_scene.npz")
    b = cpq.Batch(dev(g["verts"], cuda), g["vert_offsets"], dev(g["tris"], cuda), g["tri_offsets"], branching=4)
    sc = cpq.Scene(b, g["instance_primitive"], g["instance_transform"])
    o, d = W.camera_rays(96, 72, W.CBOX_EYE, W.CBOX_YFOV, W.CBOX_ASPECT)
    r = sc.ray_query(dev(o, cuda), dev(d, cuda))
    nv = np.diff(g["vert_offsets"])
    meshes = [(g["verts"][g["vert_offsets"][i]:g["vert_offsets"][i + 1]],
               g["tris"][g["tri_offsets"][i]:g["tri_offsets"][i + 1]]) for i in range(len(nv))]
    wv, wt, toff = world_soup(meshes, g["instance_primitive"], g["instance_transform"])
    ref = orc.ray_brute_f64_dv(wv, wt, o, d)
    t = r.t.cpu().numpy().astype(np.float64)
    hit, hit64 = np.isfinite(t), np.isfinite(ref["t"])
    assert 0.5 < hit64.mean() < 0.7  # the box, open toward the camera, fills 59% of the view
    for i in np.nonzero(hit != hit64)[0]:
        u, v = ref["uv"][i]
        assert hit64[i] and min(u, v, 1 - u - v) < 1e-4, (i, u, v)
    both = hit & hit64
    assert np.all(np.abs(t[both] - ref["t"][both]) <= 2e-5 * (1 + ref["t"][both])), \
        np.abs(t[both] - ref["t"][both]).max()


def test_scene_rays_any_hit_and_segments(cpq, cuda):
    from gpurt_cpq import workloads as W

    import torch

    meshes = [W.icosphere(2)]
    T = random_similarities(6, seed=10)
    T[3, :, :3] = T[3, :, :3] @ np.diag([2.0, 1.0, 1.0]).astype(np.float32)
    sc = cpq.Scene(make_batch(cpq, cuda, meshes, 4), np.zeros(6, np.int32), T)
    wv, _, _ = world_soup(meshes, np.zeros(6, np.int32), T)
    o, d = _scene_rays(np.random.default_rng(11), wv, 20000)
    od, dd = dev(o, cuda), dev(d, cuda)
    closest = sc.ray_query(od, dd)
    anyh = sc.ray_query(od, dd, opts=cpq.ray_opts(any_hit=True))
    assert torch.equal(torch.isfinite(anyh.t), torch.isfinite(closest.t))
    hit = torch.isfinite(closest.t)
    assert bool((anyh.t[hit] >= closest.t[hit]).all())
    # segment ends just before / after the closest hit
    tm = torch.where(hit, closest.t, torch.ones_like(closest.t))
    before = sc.ray_query(od, dd, tmax_per_ray=tm * 0.999, opts=cpq.ray_opts(any_hit=True))
    after = sc.ray_query(od, dd, tmax_per_ray=tm * 1.001)
    assert bool((~torch.isfinite(before.t[hit]) | (before.t[hit] < closest.t[hit])).all())
    assert torch.equal(after.t[hit], closest.t[hit])


def test_cbox_scene_vs_fp64(orc, cpq, cuda):
    """The reference's Cornell box (media/cbox, 16,720 triangles in 9
    primitives placed by 10 node instances), from the committed fixture:
    scene answers against its FP64 brute force over world-space vertices."""
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / "cbox_scene.npz")
    b = cpq.Batch(dev(g["verts"], cuda), g["vert_offsets"], dev(g["tris"], cuda), g["tri_offsets"],
                  branching=4)
    sc = cpq.Scene(b, g["instance_primitive"], g["instance_transform"])
    q = g["queries"]
    r = sc.query(dev(q, cuda), want_bary=True)
    d = r.dist.cpu().numpy().astype(np.float64)
    rel = np.abs(d - g["dist"]) / np.maximum(g["dist"], 1e-30)
    assert rel.max() <= 1e-6, rel.max()
    # the box's flat, axis-aligned faces give many exact ties (points nearest
    # to a shared edge, coplanar faces): where the answer names another
    # triangle than the brute force's first, that triangle is as close
    same = (r.instance.cpu().numpy() == g["instance"]) & (r.tri.cpu().numpy() == g["tri"])
    nv = np.diff(g["vert_offsets"])
    meshes = [(g["verts"][g["vert_offsets"][i]:g["vert_offsets"][i + 1]],
               g["tris"][g["tri_offsets"][i]:g["tri_offsets"][i + 1]]) for i in range(len(nv))]
    wv, wt, toff = world_soup(meshes, g["instance_primitive"], g["instance_transform"])
    inst, tri = r.instance.cpu().numpy(), r.tri.cpu().numpy()
    for i in np.nonzero(~same)[0]:
        a, bb, c = wv[wt[toff[inst[i]] + tri[i]]]
        d2, _, _ = orc.point_tri_f64(q[i].astype(np.float64), a, bb, c)
        assert abs(np.sqrt(d2) - g["dist"][i]) <= 1e-6 * g["dist"][i]


def test_gltf_instances_as_scene(orc, cpq, cuda, tmp_path):
    """A glTF file's primitives as a batch and its node instances as a scene:
    the same answers as the flattened world mesh."""
    from test_gltf import _scene, _write

    doc, data = _scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, "glb")))
    b = cpq.Batch(dev(s.verts, cuda), s.vert_offsets, dev(s.tris, cuda), s.tri_offsets, branching=4)
    sc = cpq.Scene(b, s.instance_primitive, s.instance_world)
    q = np.random.default_rng(3).uniform(-2, 12, (5000, 3)).astype(np.float32)
    r = sc.query(dev(q, cuda))
    meshes = [(s.verts[s.vert_offsets[i]:s.vert_offsets[i + 1]],
               s.tris[s.tri_offsets[i]:s.tri_offsets[i + 1]]) for i in range(len(s.tri_offsets) - 1)]
    check_scene(orc, meshes, s.instance_primitive, s.instance_world[:, :3, :].astype(np.float32), q, r)
