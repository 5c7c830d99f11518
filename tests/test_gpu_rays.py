"""Ray queries (cp_ray_query) against the CPU restatement and FP64.

The GPU's closest hit is the least (t, triangle index) over every triangle the
FP32 Möller–Trumbore test accepts, and its box test never rejects a box a ray
enters, so it must equal the FP32 brute force of the restatement BIT FOR BIT
(t, triangle, u, v) whatever the tree, the branching or the ray order.  FP64
agrees except for rays that graze a triangle's boundary.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def rays_for(v, n, seed):
    """Mixed rays: random origins in the padded box with random directions,
    axis-aligned directions (zero components), and rays from vertices."""
    rng = np.random.default_rng(seed)
    lo, hi = v.min(0), v.max(0)
    pad = 0.2 * (hi - lo).max()
    o = rng.uniform(lo - pad, hi + pad, (n, 3))
    d = rng.normal(size=(n, 3))
    k = n // 4
    axis = rng.integers(0, 3, k)
    d[:k] = 0.0
    d[np.arange(k), axis] = rng.choice([-1.0, 1.0], k)       # axis-aligned
    m = n // 8
    o[k:k + m] = v[rng.integers(0, v.shape[0], m)]           # from vertices
    d[k + m:k + 2 * m] *= rng.uniform(0.01, 100.0, (m, 1))   # any length
    return o.astype(np.float32), d.astype(np.float32)


def meshes():
    from gpurt_cpq import workloads as W

    rng = np.random.default_rng(7)
    rv = rng.normal(size=(300, 3)).astype(np.float32)
    rt = rng.integers(0, 300, (800, 3)).astype(np.int32)
    rt[:10] = [0, 1, 1]  # degenerate: repeated vertex
    return {"icosphere3": W.icosphere(3), "heightfield32": W.heightfield(32, seed=4), "soup": (rv, rt)}


def assert_same(r, ref):
    t = r.t.cpu().numpy()
    tri = r.tri.cpu().numpy()
    uv = r.uv.cpu().numpy()
    np.testing.assert_array_equal(t.view(np.uint32), ref["t"].view(np.uint32))
    np.testing.assert_array_equal(tri, ref["tri"])
    np.testing.assert_array_equal(uv.view(np.uint32), ref["uv"].view(np.uint32))


@pytest.mark.parametrize("name", ["icosphere3", "heightfield32", "soup"])
@pytest.mark.parametrize("K,leaf", [(2, 4), (4, 1), (4, 4), (8, 8)])
def test_rays_bit_exact_with_restatement(orc, cpq, cuda, name, K, leaf):
    v, t = meshes()[name]
    o, d = rays_for(v, 20000, 3)
    ref = orc.ray_brute(v, t, o, d)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=K, leaf_size=leaf)
    for sort in (True, False):
        r = m.ray_query(dev(o, cuda), dev(d, cuda), opts=cpq.ray_opts(sort_rays=sort))
        assert_same(r, ref)
    assert m.device_status() == 0
    hits = int((ref["tri"] >= 0).sum())
    print(f"{name} K={K} leaf={leaf}: {hits} of {len(o)} rays hit")


def test_rays_ranges_and_reference_epsilon(orc, cpq, cuda):
    """[tmin, tmax], per-ray segment ends and the reference's det threshold."""
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(3)
    o, d = rays_for(v, 20000, 5)
    rng = np.random.default_rng(6)
    seg = rng.uniform(0.0, 3.0, len(o)).astype(np.float32)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4)
    for tmin, tmax, eps in [(1e-5, 1e7, 1e-5), (0.5, 2.0, 0.0), (0.0, float("inf"), 1e-3)]:
        ref = orc.ray_brute(v, t, o, d, tmin, tmax, eps, tmax_per_ray=seg)
        r = m.ray_query(dev(o, cuda), dev(d, cuda), tmax_per_ray=dev(seg, cuda),
                        opts=cpq.ray_opts(tmin=tmin, tmax=tmax, det_epsilon=eps))
        assert_same(r, ref)


def test_any_hit_agrees_with_closest_hit(orc, cpq, cuda):
    """visibility(): the first accepted hit.  Hit or not must equal the
    closest-hit answer; the hit found is a real one in range, not closer than
    the closest."""
    from gpurt_cpq import workloads as W

    v, t = W.heightfield(64, seed=2)
    o, d = rays_for(v, 30000, 9)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    closest = m.ray_query(dev(o, cuda), dev(d, cuda))
    anyh = m.ray_query(dev(o, cuda), dev(d, cuda), opts=cpq.ray_opts(any_hit=True))
    ct, at = closest.t.cpu().numpy(), anyh.t.cpu().numpy()
    ctri, atri = closest.tri.cpu().numpy(), anyh.tri.cpu().numpy()
    np.testing.assert_array_equal(ctri >= 0, atri >= 0)
    hit = atri >= 0
    assert np.all(at[hit] >= ct[hit]) and np.all(at[~hit] == np.inf)
    # the reported hit is a real one: FP64 Möller–Trumbore of that ray and triangle
    a, b, c = (v[t[atri[hit], k]].astype(np.float64) for k in range(3))
    oo, dd = o[hit].astype(np.float64), d[hit].astype(np.float64)
    e1, e2 = b - a, c - a
    p = np.cross(dd, e2)
    det = (e1 * p).sum(1)
    s = oo - a
    q = np.cross(s, e1)
    t64 = (e2 * q).sum(1) / det
    assert np.all(np.abs(t64 - at[hit]) <= 1e-4 * (1 + np.abs(t64)))


def test_rays_agree_with_fp64(orc, cpq, cuda):
    from gpurt_cpq import workloads as W

    v, t = W.icosphere(4)
    o, d = rays_for(v, 20000, 11)
    r = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4).ray_query(dev(o, cuda), dev(d, cuda))
    ref = orc.ray_brute(v, t, o, d, fp64=True)
    tri = r.tri.cpu().numpy()
    tt = r.t.cpu().numpy().astype(np.float64)
    same = tri == ref["tri"]
    both = same & (tri >= 0)
    scale = np.linalg.norm(d, axis=1).astype(np.float64)
    err = np.abs(tt[both] - ref["t"][both]) * scale[both]
    assert err.max(initial=0) <= 1e-5 * (1 + np.abs(ref["t"][both]) * scale[both]).max(initial=1)
    # disagreements only for rays grazing a triangle's boundary in FP64
    bad = np.nonzero(~same)[0]
    uv = ref["uv"][bad]
    w = np.minimum(np.minimum(uv[:, 0], uv[:, 1]), 1 - uv[:, 0] - uv[:, 1])
    hit64 = ref["tri"][bad] >= 0
    graze = np.where(hit64, w <= 1e-4, True)
    assert graze.all(), f"{(~graze).sum()} FP64 hits well inside a triangle missed"
    print(f"fp64: {both.sum()} common hits, {len(bad)} boundary disagreements of {len(o)}")


def test_rays_large_mesh_sample(orc, cpq, cuda):
    """The large workload's 2M-triangle heightfield: a sample checked by brute force."""
    from gpurt_cpq import workloads as W

    v, t = W.heightfield(1024, seed=1)
    rng = np.random.default_rng(13)
    o = np.stack([rng.uniform(-0.1, 1.1, 400), rng.uniform(-0.1, 1.1, 400),
                  rng.uniform(-0.5, 0.5, 400)], 1).astype(np.float32)
    d = rng.normal(size=(400, 3)).astype(np.float32)
    ref = orc.ray_brute(v, t, o, d)
    m = cpq.Mesh(dev(v, cuda), dev(t, cuda), branching=4, leaf_size=4)
    assert_same(m.ray_query(dev(o, cuda), dev(d, cuda)), ref)
