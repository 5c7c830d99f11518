"""The shading restatement against the reference's own shader code, bit for bit.

oracle/make_ref_shade.py compiles the reference's rtcommon.glsl, restir.glsl,
rt.rgen and tonemap.frag as C++ (syntax rewrites only, against the GLSL environment of
oracle/glsl_shim.h) from a checkout of the reference.  GLSL leaves sin, cos,
pow and exp to the implementation, and the ray-tracing pipeline's traversal
to the driver: the shim takes both from the restatement, so everything else
is the reference's code.  These tests run both on the same inputs and
require identical results: the shader functions one by one, the tone
mapping curves, and whole
frames of rt.rgen's main (every integrator and material, Russian roulette,
Hammersley jitter, metalness, jittered later frames, ReSTIR with and without
the previous frame's reservoirs, the debug views) on a floor under a light, a
corner that inter-reflects, and the reference's Cornell box.  Skipped where
no checkout of the reference exists.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import shade as S

pytestmark = pytest.mark.skipif(S.ref_lib() is None, reason="no checkout of the reference's shaders")

FRAME = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)


def _dirs(n, seed):
    v = np.random.default_rng(seed).normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _same(a, b):
    for x, y in zip(a, b) if isinstance(a, tuple) else ((a, b),):
        np.testing.assert_array_equal(x, y)


# ------------------------------------------------------------ shader functions

def test_random_numbers():
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2**32, 5000, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 2**32, 5000, dtype=np.uint64).astype(np.uint32)
    _same(S.tea(a, b), S.tea(a, b, ref=True))
    for seed in (0, 1, 0xDEADBEEF):
        _same(S.lcg_stream(seed, 10000), S.lcg_stream(seed, 10000, ref=True))
    _same(S.radical_inverse(a), S.radical_inverse(a, ref=True))


def test_reservoir_updates():
    w = np.random.default_rng(2).random(20000).astype(np.float32)
    w[::7] = 0.0
    for seed in (3, 99):
        _same(S.reservoir_stream(seed, w), S.reservoir_stream(seed, w, ref=True))


def test_geometry():
    n = 20000
    o = (np.random.default_rng(4).random((n, 3)) * 2 - 1).astype(np.float32)
    d = _dirs(n, 5)
    tri = np.float32([[-0.4, 0.5, -0.3], [0.6, 0.6, -0.2], [0.1, 0.4, 0.7]])
    want = S.triangle_pdf(o, d, tri, ref=True)
    assert (want > 0).sum() > 500
    _same(S.triangle_pdf(o, d, tri), want)
    lo, hi = np.float32([-0.5, -0.3, -0.4]), np.float32([0.6, 0.2, 0.5])
    _same(S.hit_bbox(o * 3, d, lo, hi), S.hit_bbox(o * 3, d, lo, hi, ref=True))
    _same(S.make_tanspace(d), S.make_tanspace(d, ref=True))


@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
@pytest.mark.parametrize("rough", [0.05, 0.3, 0.8])
def test_materials(brdf, rough):
    wo = np.float32([0.45, -0.2, -0.87])
    wo /= np.linalg.norm(wo)
    wi = _dirs(50000, 7)
    got = S.material(brdf, [0.9, 0.5, 0.2], rough, wo, FRAME, wi)
    assert (got[0] > 0).mean() > 0.3
    _same(got, S.material(brdf, [0.9, 0.5, 0.2], rough, wo, FRAME, wi, ref=True))


@pytest.mark.parametrize("kind,param", [(S.UNIFORM_HEMISPHERE, 0.0), (S.COSINE_HEMISPHERE, 0.0),
                                        (S.COSPOW_HEMISPHERE, 7.0), (S.GGX_SAMPLE, 0.3), (S.BP_SAMPLE, 0.2),
                                        (S.TRIANGLE_SAMPLE, 0.0)])
def test_samplers(kind, param):
    wo = np.float32([0.3, 0.1, -0.95])
    wo /= np.linalg.norm(wo)
    _same(S.sample(kind, 50000, 8, FRAME, param, wo=wo), S.sample(kind, 50000, 8, FRAME, param, wo=wo, ref=True))


def test_tonemapping():
    c = np.concatenate([np.linspace(0.0, 4.0, 4001), np.geomspace(4.0, 1e4, 500)]).astype(np.float32)
    for kind in (S.FILMIC, S.EXPONENTIAL, S.NO_TONEMAP):
        for exposure, gamma in ((1.0, 2.2), (0.37, 1.0), (3.0, 2.4)):
            _same(S.tonemap(c, kind, exposure, gamma), S.tonemap(c, kind, exposure, gamma, ref=True))


# ------------------------------------------------------------------ frames

def _scenes():
    import test_shade_oracle as T

    return {"floor": (T.floor_and_light(), T.CAM), "corner": (T.corner_and_light(), T.CAM),
            "cbox": (T.cbox_shade_scene(), S.camera(eye=(0.0, 0.0, 19.992091970966317), target=(0.0, 0.0, 0.0),
                                                    up=(0, 1, 0), yfov=0.7175414562225342, width=16, height=12))}


@pytest.fixture(scope="module")
def scenes():
    return _scenes()


def _frame_pair(sc, cam, **kw):
    a = sc.render(cam, gbuffer=True, **kw)
    b = sc.render(cam, gbuffer=True, ref=True, **kw)
    return a, b


@pytest.mark.parametrize("name", ["floor", "corner", "cbox"])
@pytest.mark.parametrize("integrator", [S.DIRECT, S.MATERIAL, S.MIS, S.RESTIR_DIRECT, S.RESTIR])
@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_frames_bit_exact(scenes, name, integrator, brdf):
    sc, cam = scenes[name]
    a, b = _frame_pair(sc, cam, integrator=integrator, brdf=brdf, samples=4, seed=11)
    _same(a, b)
    assert a[0].max() > 0.0


@pytest.mark.parametrize("integrator", [S.DIRECT, S.MATERIAL, S.MIS, S.RESTIR_DIRECT, S.RESTIR])
@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
@pytest.mark.parametrize("normal_map", [False, True])
def test_textured_frames_bit_exact(integrator, brdf, normal_map):
    """Textured materials (albedo, emission, metal / roughness, normal maps)
    through the reference's own mat_info, hit_info, shade_info and
    light_sample: the restatement's frames equal them bit for bit."""
    import test_shade_oracle as T

    sc = T.textured_scene()
    for metal in (False, True):
        a, b = _frame_pair(sc, T.CAM, integrator=integrator, brdf=brdf, samples=4, seed=17,
                           use_normal_map=normal_map, use_metalness=metal)
        _same(a, b)
        assert a[0].max() > 0.0


@pytest.mark.parametrize("opts", [dict(use_rr=False, max_depth=5), dict(qmc=True, frame=3, max_frame=16),
                                  dict(use_metalness=True, integrator=S.MIS), dict(frame=2, env=(0.2, 0.3, 0.4)),
                                  dict(integrator=S.RESTIR, new_samples=7, temporal_multiplier=3)])
def test_frame_options_bit_exact(scenes, opts):
    sc, cam = scenes["corner"]
    kw = dict(integrator=S.MIS, samples=4, seed=12)
    kw.update(opts)
    if kw.get("frame", 0) > 0:  # a later frame blends into the previous image
        base = np.random.default_rng(13).random((cam.height, cam.width, 3)).astype(np.float32)
        a = sc.render(cam, image=base.copy(), **kw)
        b = sc.render(cam, image=base.copy(), ref=True, **kw)
        _same(a, b)
    else:
        _same(*_frame_pair(sc, cam, **kw))


@pytest.mark.parametrize("integrator", [S.RESTIR_DIRECT, S.RESTIR])
def test_restir_across_frames_bit_exact(scenes, integrator):
    """Four frames of temporal reuse: images, first-hit buffers and the
    reservoirs handed to the next frame all identical."""
    sc, cam = scenes["floor"]
    states = [S.TemporalState(cam), S.TemporalState(cam)]
    imgs = [np.zeros((cam.height, cam.width, 3), np.float32) for _ in range(2)]
    for frame in range(4):
        outs = []
        for k, ref in enumerate((False, True)):
            _, g = sc.render(cam, integrator=integrator, samples=2, frame=frame, seed=40 + frame, image=imgs[k],
                             gbuffer=True, temporal=states[k], ref=ref)
            outs.append(g)
        _same(imgs[0], imgs[1])
        _same(outs[0], outs[1])
        assert states[0].out_res.tobytes() == states[1].out_res.tobytes()
        for k in range(2):
            states[k].advance(outs[k], cam)
    assert states[0].prev_res["n_seen"].max() > states[0].prev_res["n_seen"].min()


@pytest.mark.parametrize("view", [1, 2, 3])
def test_debug_views_bit_exact(scenes, view):
    sc, cam = scenes["floor"]
    st = [S.TemporalState(cam), S.TemporalState(cam)]
    for k, ref in enumerate((False, True)):
        _, g = sc.render(cam, integrator=S.DIRECT, samples=1, gbuffer=True, ref=ref)
        st[k].advance(g, cam)
    a = sc.render(cam, integrator=S.DIRECT, samples=1, frame=1, seed=5, debug_view=view, temporal=st[0])
    b = sc.render(cam, integrator=S.DIRECT, samples=1, frame=1, seed=5, debug_view=view, temporal=st[1], ref=True)
    _same(a, b)


# ------------------------------------------------- the ray query's arithmetic

def test_ray_restatement_matches_triangle_hit():
    """The FP32 ray restatement that the GPU ray kernels match bit for bit
    (cpq_oracle.c, det epsilon 1e-5, t >= 0) against the reference's own
    triangle_hit: the same hits, and o + t d is the shader's hit point."""
    from oracle import oracle as O

    rng = np.random.default_rng(21)
    tri = np.float32([[-0.4, 0.5, -0.3], [0.6, 0.6, -0.2], [0.1, 0.4, 0.7]])
    n = 50000
    o = (rng.random((n, 3)) * 4 - 2).astype(np.float32)
    # half the rays aimed at points of the triangle, half at random
    b = rng.random((n, 2))
    b = np.where(b.sum(1, keepdims=True) > 1, 1 - b, b)
    target = tri[0] + b[:, :1] * (tri[1] - tri[0]) + b[:, 1:] * (tri[2] - tri[0])
    d = np.where(np.arange(n)[:, None] % 2 == 0, target - o, rng.normal(size=(n, 3)))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    hit, p = S.triangle_hit_ref(o, d, tri)
    r = O.ray_brute(tri, np.int32([[0, 1, 2]]), o, d, tmin=0.0, tmax=float("inf"), det_eps=1e-5)
    mine = r["tri"] >= 0
    assert hit.sum() > 20000
    np.testing.assert_array_equal(mine, hit)
    t = r["t"][hit].astype(np.float32)[:, None]
    np.testing.assert_array_equal(o[hit] + t * d[hit], p[hit])
