"""GPU path tracer (cp_shade_*) against the CPU restatement, bit for bit.

The restatement (oracle/shade_oracle.c) is the reference's rt.rgen,
rtcommon.glsl, restir.glsl and tonemap.frag restated in FP32, and equals the
reference's own shader code compiled as C++ bit for bit (test_shade_ref.py).
The CUDA kernels trace through the library's BVH, whose hits equal the
restatement's brute force over all triangles bit for bit, and shade with the
same operations in the same order without multiply-add contraction, so every
pixel must be identical: images, first-hit buffers and ReSTIR's reservoirs,
for every integrator, material and frame option, over several frames of
temporal reuse, on a floor under a light, a corner that inter-reflects and
the reference's Cornell box.  All calls go through the C ABI.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import shade as S

pytestmark = pytest.mark.gpu


def _gpu_scene(sc, cuda):
    import torch

    from gpurt_cpq import shading as G

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)

    return G.ShadeScene(d(sc.verts), d(sc.normals), d(sc.obj), d(sc.albedo), d(sc.emissive), d(sc.metal_rough))


def _cam(cam):
    from gpurt_cpq import shading as G

    return G.ShadeCamera.from_buffer_copy(cam)


def _same(got, want, what="image"):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape
    bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))
    assert len(bad[0]) == 0, (f"{what}: {len(bad[0])} of {got.size} values differ, first at "
                              f"{tuple(int(b[0]) for b in bad)}: {got[tuple(b[0] for b in bad)]} vs "
                              f"{want[tuple(b[0] for b in bad)]}")


def _scenes():
    import test_shade_oracle as T

    return {"floor": (T.floor_and_light(), T.CAM), "corner": (T.corner_and_light(), T.CAM),
            "cbox": (T.cbox_shade_scene(), S.camera(eye=(0.0, 0.0, 19.992091970966317), target=(0.0, 0.0, 0.0),
                                                    up=(0, 1, 0), yfov=0.7175414562225342, width=16, height=12))}


@pytest.fixture(scope="module")
def scenes(cuda):
    return {k: (sc, cam, _gpu_scene(sc, cuda)) for k, (sc, cam) in _scenes().items()}


def _pair(sc, gs, cam, **kw):
    want = sc.render(cam, gbuffer=True, **kw)
    img, g = gs.render(_cam(cam), gbuffer=True, **kw)
    return (img.cpu().numpy(), g.cpu().numpy()), want


@pytest.mark.parametrize("name", ["floor", "corner", "cbox"])
@pytest.mark.parametrize("integrator", [S.DIRECT, S.MATERIAL, S.MIS, S.RESTIR_DIRECT, S.RESTIR])
@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_frames_bit_exact(scenes, name, integrator, brdf):
    sc, cam, gs = scenes[name]
    (img, g), (wimg, wg) = _pair(sc, gs, cam, integrator=integrator, brdf=brdf, samples=4, seed=11)
    _same(img, wimg)
    _same(g, wg, "first-hit buffer")
    assert img.max() > 0.0


@pytest.mark.parametrize("opts", [dict(use_rr=False, max_depth=5), dict(qmc=True, frame=3, max_frame=16),
                                  dict(use_metalness=True, integrator=S.MIS), dict(frame=2, env=(0.2, 0.3, 0.4)),
                                  dict(integrator=S.RESTIR, new_samples=7, temporal_multiplier=3),
                                  dict(max_depth=0), dict(integrator=S.MIS, brdf=S.GGX, max_depth=12, samples=9)])
def test_frame_options_bit_exact(scenes, opts, cuda):
    import torch

    sc, cam, gs = scenes["corner"]
    kw = dict(integrator=S.MIS, samples=4, seed=12)
    kw.update(opts)
    if kw.get("frame", 0) > 0:  # a later frame blends into the previous image
        base = np.random.default_rng(13).random((cam.height, cam.width, 3)).astype(np.float32)
        want = sc.render(cam, image=base.copy(), **kw)
        got = gs.render(_cam(cam), image=torch.from_numpy(base.copy()).to(cuda), **kw)
        _same(got.cpu().numpy(), want)
    else:
        (img, g), (wimg, wg) = _pair(sc, gs, cam, **kw)
        _same(img, wimg)
        _same(g, wg, "first-hit buffer")


@pytest.mark.parametrize("integrator", [S.RESTIR_DIRECT, S.RESTIR])
def test_restir_across_frames_bit_exact(scenes, integrator, cuda):
    """Four frames of temporal reuse: images, first-hit buffers and the
    reservoirs handed to the next frame all identical."""
    import torch

    from gpurt_cpq import shading as G

    sc, cam, gs = scenes["floor"]
    ost, gst = S.TemporalState(cam), G.TemporalState(_cam(cam), cuda)
    oimg = np.zeros((cam.height, cam.width, 3), np.float32)
    gimg = torch.zeros((cam.height, cam.width, 3), dtype=torch.float32, device=cuda)
    for frame in range(4):
        _, og = sc.render(cam, integrator=integrator, samples=2, frame=frame, seed=40 + frame, image=oimg,
                          gbuffer=True, temporal=ost)
        _, gg = gs.render(_cam(cam), integrator=integrator, samples=2, frame=frame, seed=40 + frame, image=gimg,
                          gbuffer=True, temporal=gst)
        _same(gimg.cpu().numpy(), oimg)
        _same(gg.cpu().numpy(), og, "first-hit buffer")
        assert gst.out_res.cpu().numpy().tobytes() == ost.out_res.tobytes(), f"reservoirs of frame {frame}"
        ost.advance(og, cam)
        gst.advance(gg, _cam(cam))
    assert ost.prev_res["n_seen"].max() > ost.prev_res["n_seen"].min()


@pytest.mark.parametrize("view", [1, 2, 3])
def test_debug_views_bit_exact(scenes, view, cuda):
    from gpurt_cpq import shading as G

    sc, cam, gs = scenes["floor"]
    ost, gst = S.TemporalState(cam), G.TemporalState(_cam(cam), cuda)
    _, og = sc.render(cam, integrator=S.DIRECT, samples=1, gbuffer=True)
    _, gg = gs.render(_cam(cam), integrator=S.DIRECT, samples=1, gbuffer=True)
    ost.advance(og, cam)
    gst.advance(gg, _cam(cam))
    want = sc.render(cam, integrator=S.DIRECT, samples=1, frame=1, seed=5, debug_view=view, temporal=ost)
    got = gs.render(_cam(cam), integrator=S.DIRECT, samples=1, frame=1, seed=5, debug_view=view, temporal=gst)
    _same(got.cpu().numpy(), want)


def test_cornell_box_larger_frame_bit_exact(scenes):
    """The reference's Cornell box at 64 x 48, 8 samples per pixel, MIS and
    ReSTIR: many paths per pixel through 16,720 triangles."""
    sc, _, gs = scenes["cbox"]
    cam = S.camera(eye=(0.0, 0.0, 19.992091970966317), target=(0.0, 0.0, 0.0), up=(0, 1, 0),
                   yfov=0.7175414562225342, width=64, height=48)
    for integrator in (S.MIS, S.RESTIR):
        (img, g), (wimg, wg) = _pair(sc, gs, cam, integrator=integrator, samples=8, seed=3)
        _same(img, wimg)
        _same(g, wg, "first-hit buffer")


def _gpu_textured(sc, cuda):
    import torch

    g = _gpu_scene(sc, cuda)
    g.set_textures(texcoords=torch.from_numpy(sc.texcoords).to(cuda), tangents=torch.from_numpy(sc.tangents).to(cuda),
                   textures=sc.textures, obj_tex=sc.obj_tex)
    return g


@pytest.mark.parametrize("integrator", [S.DIRECT, S.MATERIAL, S.MIS, S.RESTIR_DIRECT, S.RESTIR])
@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_textured_frames_bit_exact(cuda, integrator, brdf):
    """Textured albedo, emission, metal / roughness and normal maps, with the
    normal map on and off and metalness on and off: every pixel and first
    hit equal to the restatement."""
    import test_shade_oracle as T

    sc = T.textured_scene()
    gs = _gpu_textured(sc, cuda)
    for normal_map in (False, True):
        for metal in (False, True):
            (img, g), (wimg, wg) = _pair(sc, gs, T.CAM, integrator=integrator, brdf=brdf, samples=4, seed=17,
                                         use_normal_map=normal_map, use_metalness=metal)
            _same(img, wimg)
            _same(g, wg, "first-hit buffer")
            assert img.max() > 0.0


def test_textured_larger_frame_and_refusals(cuda):
    """A 48 x 36 textured frame at 8 samples per pixel through every
    integrator option at once; then textures replaced by none give the
    untextured frame; bad texture indices and sizes are refused."""
    import torch

    from gpurt_cpq import CpError

    import test_shade_oracle as T

    sc = T.textured_scene(seed=9)
    gs = _gpu_textured(sc, cuda)
    cam = S.camera(eye=(0.1, 0.8, 1.5), target=(0.0, 0.2, -0.3), up=(0, 1, 0), yfov=1.0, width=48, height=36)
    for integrator in (S.MIS, S.RESTIR):
        (img, g), (wimg, wg) = _pair(sc, gs, cam, integrator=integrator, samples=8, seed=2, use_normal_map=True)
        _same(img, wimg)
        _same(g, wg, "first-hit buffer")
    plain = S.Scene(sc.verts, sc.normals, sc.obj, sc.albedo, sc.emissive, sc.metal_rough)
    gs.set_textures()
    _same(gs.render(_cam(cam), integrator=S.MIS, samples=2, seed=4).cpu().numpy(),
          plain.render(cam, integrator=S.MIS, samples=2, seed=4))
    bad = sc.obj_tex.copy()
    bad[1, 0] = len(sc.textures)
    with pytest.raises(CpError, match="names texture"):
        gs.set_textures(texcoords=torch.from_numpy(sc.texcoords).to(cuda), textures=sc.textures, obj_tex=bad)
    with pytest.raises(CpError, match="size"):
        gs.set_textures(textures=[np.zeros((0, 4, 4), np.uint8)])
    # texels in host memory: refused before the decode kernel could read them
    from ctypes import c_void_p

    from gpurt_cpq._lib import lib
    host = np.zeros(4 * 4 * 4, np.uint8)
    size = np.int32([[4, 4]])
    assert lib.cp_shade_scene_textures(gs._h, None, None, 1, c_void_p(size.ctypes.data), c_void_p(host.ctypes.data),
                                       None, None) != 0
    assert b"device memory" in lib.cp_last_error_string()
    # the refused calls left the scene as it was (no textures)
    _same(gs.render(_cam(cam), integrator=S.MIS, samples=2, seed=4).cpu().numpy(),
          plain.render(cam, integrator=S.MIS, samples=2, seed=4))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_tonemap_bit_exact(cuda, kind):
    import torch

    from gpurt_cpq import shading as G

    x = np.concatenate([np.linspace(0.0, 20.0, 4001), np.random.default_rng(2).exponential(1.5, 4000)])
    x = x.astype(np.float32)
    for exposure, gamma in ((1.0, 2.2), (0.35, 1.8), (3.0, 2.4)):
        got = G.tonemap(torch.from_numpy(x).to(cuda), kind, exposure, gamma).cpu().numpy()
        _same(got, S.tonemap(x, kind, exposure, gamma), f"tone map {kind}")


def test_scene_and_render_refusals(cuda):
    import torch

    from gpurt_cpq import CpError
    from gpurt_cpq import shading as G

    import test_shade_oracle as T

    sc = T.floor_and_light()
    dark = S.Scene(sc.verts, sc.normals, sc.obj, sc.albedo, np.zeros_like(sc.emissive), sc.metal_rough)
    gd = _gpu_scene(dark, cuda)
    assert gd.n_lights == 0
    with pytest.raises(CpError):  # every integrator but material sampling needs a light
        gd.render(_cam(T.CAM), integrator=S.DIRECT)
    img = gd.render(_cam(T.CAM), integrator=S.MATERIAL, samples=2)
    _same(img.cpu().numpy(), dark.render(T.CAM, integrator=S.MATERIAL, samples=2))
    gs = _gpu_scene(sc, cuda)
    assert gs.n_lights == 1
    for bad in (dict(samples=0), dict(integrator=5), dict(brdf=2), dict(qmc=True, max_frame=0)):
        with pytest.raises(CpError):
            gs.render(_cam(T.CAM), **bad)
    obj = torch.from_numpy(sc.obj.copy()).to(cuda)
    obj[0] = 7  # names an object that does not exist
    with pytest.raises(CpError):
        G.ShadeScene(*(torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (sc.verts, sc.normals)), obj,
                     *(torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (sc.albedo, sc.emissive,
                                                                                   sc.metal_rough)))
