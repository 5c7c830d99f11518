"""The shading restatement (oracle/shade_oracle.c) against known answers and
the mathematics the reference's shaders implement (rtcommon.glsl, rt.rgen,
restir.glsl).

The shaders cannot run here (Vulkan), so parity with the reference itself is
unpinned; these tests pin the restatement instead:
  - random numbers: TEA and the lcg against an independent Python
    restatement, the radical inverse against hand values;
  - the restatement's own sin / cos / pow / exp within 2 ulp of FP64, and
    its tone mapping against the FP64 formulas of tonemap.frag;
  - samplers: unit directions in the right hemisphere with the analytic
    moments of their densities;
  - materials: each pdf integrates over the upper hemisphere to its
    sampler's acceptance rate, and the sampler's directions reproduce the
    pdf (E[g(wi)] against quadrature of g * pdf), for Blinn-Phong and GGX;
  - triangle and light pdfs integrate to 1 over the sphere;
  - direct lighting per pixel against an FP64 quadrature over the light's
    area with the material formulas written independently here;
  - integrators: direct lighting, material sampling, MIS and both ReSTIR
    modes estimate the same image of a floor under an area light, with and
    without Russian roulette; in a corner that inter-reflects, material
    sampling, ReSTIR and MIS to depth 8 agree; ReSTIR reusing the previous
    frame's reservoirs stays unbiased; a mirror floor reflects the light
    exactly.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import shade as S

FRAME = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)  # T, B, N = x, y, z


# ---------------------------------------------------------------- random numbers

def _tea_py(v0: int, v1: int) -> int:
    m = 0xFFFFFFFF
    s0 = 0
    for _ in range(16):
        s0 = (s0 + 0x9E3779B9) & m
        v0 = (v0 + ((((v1 << 4) & m) + 0xA341316C) ^ ((v1 + s0) & m) ^ ((v1 >> 5) + 0xC8013EA4))) & m
        v1 = (v1 + ((((v0 << 4) & m) + 0xAD90777D) ^ ((v0 + s0) & m) ^ ((v0 >> 5) + 0x7E95761E))) & m
    return v0


def test_tea_matches_python_restatement():
    rng = np.random.default_rng(5)
    a = rng.integers(0, 2**32, 200, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 2**32, 200, dtype=np.uint64).astype(np.uint32)
    a[:3] = [0, 1, 0xFFFFFFFF]
    b[:3] = [0, 0, 0xFFFFFFFF]
    got = S.tea(a, b)
    assert [int(x) for x in got] == [_tea_py(int(x), int(y)) for x, y in zip(a, b)]


def test_lcg_stream():
    u, f = S.lcg_stream(0, 4)
    s, want = 0, []
    for _ in range(4):
        s = (1664525 * s + 1013904223) % 2**32
        want.append(s & 0xFFFFFF)
    assert u.tolist() == want
    assert want[0] == 1013904223 & 0xFFFFFF
    np.testing.assert_array_equal(f, np.asarray(want, np.float32) / np.float32(2**24))
    # randf lies in [0, 1) for every state of a long stream
    _, f = S.lcg_stream(12345, 1 << 16)
    assert f.min() >= 0.0 and f.max() < 1.0


def test_radical_inverse_known_values():
    got = S.radical_inverse([0, 1, 2, 3, 4, 5, 0x80000000, 0xFFFFFFFF])
    np.testing.assert_array_equal(got, np.float32([0.0, 0.5, 0.25, 0.75, 0.125, 0.625, 2.0**-32, 1.0]))


# ------------------------------------------------------------------ own math

def test_sin_cos_within_two_ulp():
    x = np.linspace(0.0, 6.3, 200001, dtype=np.float32)
    x = np.concatenate([x, np.float32(2.0 * 3.141592) * np.random.default_rng(2).random(50000, np.float32)])
    for got, ref in ((S.sin(x), np.sin(x.astype(np.float64))), (S.cos(x), np.cos(x.astype(np.float64)))):
        ulp = np.spacing(np.maximum(np.abs(ref), 2.0**-24).astype(np.float32)).astype(np.float64)
        assert (np.abs(got - ref) / ulp).max() <= 2.0


def test_pow_within_two_ulp():
    rng = np.random.default_rng(3)
    x = rng.random(200000, np.float32)
    y = np.concatenate([rng.random(100000, np.float32) * 200.0, np.float32(1.0) / (rng.random(100000, np.float32)
                                                                                    * 100.0 + 1.0)])
    ref = np.power(x.astype(np.float64), y.astype(np.float64))
    got = S.pow(x, y)
    keep = ref > 1e-30
    ulp = np.spacing(ref[keep].astype(np.float32)).astype(np.float64)
    assert (np.abs(got[keep] - ref[keep]) / ulp).max() <= 2.0
    assert S.pow(np.float32([0.0, 0.0, 1.0, 0.5]), np.float32([5.0, 0.25, 7.0, 1.0])).tolist() == [0.0, 0.0, 1.0,
                                                                                                   0.5]


def test_pow_exact_cases():
    """x^1 = x, x^(1/2) = the correctly rounded square root, and integer
    powers 2..64 (FP64 products) within one ulp of FP64."""
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.random(50000, np.float32), rng.random(1000, np.float32) * np.float32(3.0)])
    np.testing.assert_array_equal(S.pow(x, np.full_like(x, 1.0)), x)
    np.testing.assert_array_equal(S.pow(x, np.full_like(x, 0.5)), np.sqrt(x))
    for n in (2, 3, 5, 10, 17, 64):
        ref = np.power(x.astype(np.float64), float(n))
        keep = (ref > 1e-30) & (ref < 1e30)
        got = S.pow(x, np.full_like(x, float(n)))
        ulp = np.spacing(ref[keep].astype(np.float32)).astype(np.float64)
        assert (np.abs(got[keep] - ref[keep]) / ulp).max() <= 1.0, n
    # a non-integer exponent next to an integer takes the general path
    ref = np.power(x.astype(np.float64), float(np.float32(2.5)))
    got = S.pow(x, np.full_like(x, 2.5))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert (np.abs(got - ref) / ulp).max() <= 2.0


def test_exp_within_two_ulp():
    x = np.concatenate([-np.linspace(0.0, 80.0, 200001, dtype=np.float32),
                        np.linspace(0.0, 80.0, 1001, dtype=np.float32)])
    ref = np.exp(x.astype(np.float64))
    got = S.exp(x)
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert (np.abs(got - ref) / ulp).max() <= 2.0
    assert S.exp(np.float32([0.0]))[0] == 1.0


# -------------------------------------------------------------- tone mapping

def _filmic64(c):
    A, B, C, D, E, F = 0.15, 0.50, 0.10, 0.20, 0.02, 0.30
    return (c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F) - E / F


def test_tonemap_against_fp64_formulas():
    c = np.concatenate([np.linspace(0.0, 4.0, 4001), np.geomspace(4.0, 1e4, 500)]).astype(np.float32)
    c64 = c.astype(np.float64)
    for exposure, gamma in ((1.0, 2.2), (0.37, 1.0), (3.0, 2.4)):
        e = np.float32(exposure)
        want = (1.0 - np.exp(-c64 * np.float64(e))) ** (1.0 / np.float64(np.float32(gamma)))
        got = S.tonemap(c, S.EXPONENTIAL, exposure, gamma).astype(np.float64)
        np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-6)
        want = np.maximum(_filmic64(c64 * e) / _filmic64(11.2), 0.0) ** (1.0 / np.float64(np.float32(gamma)))
        got = S.tonemap(c, S.FILMIC, exposure, gamma).astype(np.float64)
        # at black the curve's constant terms cancel in FP32 to ~7e-9 instead
        # of 0 (the shader's formula in FP32), which the gamma power lifts
        away = c64 * e >= 1e-3
        np.testing.assert_allclose(got[away], want[away], rtol=1e-5, atol=1e-5)
        assert 0.0 <= got[0] < 1e-3
        assert np.all(np.diff(got[:4001]) >= 0)  # monotone
    img = np.random.default_rng(4).random((3, 5, 3), np.float32) * 3
    np.testing.assert_array_equal(S.tonemap(img, S.NO_TONEMAP), img)
    # the filmic curve reaches white at 11.2 / exposure
    assert abs(S.tonemap(np.float32([11.2]), S.FILMIC, 1.0, 2.2)[0] - 1.0) < 1e-6
    with pytest.raises(ValueError):
        S.tonemap(img, 3)


# ------------------------------------------------------------------ samplers

N_SAMP = 200000


def _se(x):
    return x.std() / np.sqrt(len(x))


@pytest.mark.parametrize("kind,param,axis,mean", [
    (S.UNIFORM_HEMISPHERE, 0.0, 1, 0.5),        # cos theta uniform, about the frame's y axis
    (S.COSINE_HEMISPHERE, 0.0, 2, 2.0 / 3.0),
    (S.COSPOW_HEMISPHERE, 3.0, 2, 4.0 / 5.0),   # E[cos] = (e + 1) / (e + 2)
    (S.COSPOW_HEMISPHERE, 20.0, 2, 21.0 / 22.0),
])
def test_hemisphere_samplers(kind, param, axis, mean):
    d, ok = S.sample(kind, N_SAMP, 77, FRAME, param)
    assert ok.all()
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
    c = d[:, axis].astype(np.float64)
    assert c.min() >= 0.0
    assert abs(c.mean() - mean) < 5 * _se(c)
    # azimuth uniform: the two other components average to zero
    for k in {0, 1, 2} - {axis}:
        assert abs(d[:, k].mean()) < 5 * _se(d[:, k].astype(np.float64))


def test_triangle_sample_uniform():
    b, ok = S.sample(S.TRIANGLE_SAMPLE, N_SAMP, 9, FRAME)
    assert ok.all() and b.min() >= -1e-7
    np.testing.assert_allclose(b.sum(1), 1.0, atol=1e-6)
    for k in range(3):
        assert abs(b[:, k].mean() - 1.0 / 3.0) < 5 * _se(b[:, k].astype(np.float64))
        # second moment of a barycentric under the uniform density: 1/6
        assert abs((b[:, k].astype(np.float64) ** 2).mean() - 1.0 / 6.0) < 5 * _se(b[:, k].astype(np.float64) ** 2)


def _hemisphere_grid(n_cos=1024, n_phi=1024):
    c = (np.arange(n_cos) + 0.5) / n_cos
    p = (np.arange(n_phi) + 0.5) / n_phi * 2 * np.pi
    C, P = np.meshgrid(c, p, indexing="ij")
    s = np.sqrt(1 - C * C)
    w = np.stack([s * np.cos(P), s * np.sin(P), C], -1).reshape(-1, 3)
    return w.astype(np.float32), (1.0 / n_cos) * (2 * np.pi / n_phi)


WO = np.float32([0.45, -0.2, -0.87])  # incoming direction (towards the surface)
WO = WO / np.linalg.norm(WO)


@pytest.mark.parametrize("brdf,rough", [(S.BLINN_PHONG, 0.5), (S.BLINN_PHONG, 0.15), (S.GGX, 0.6), (S.GGX, 0.35)])
def test_material_pdf_matches_its_sampler(brdf, rough):
    kind = S.BP_SAMPLE if brdf == S.BLINN_PHONG else S.GGX_SAMPLE
    d, ok = S.sample(kind, N_SAMP, 1234, FRAME, rough, wo=WO)
    grid, dw = _hemisphere_grid()
    pdf, ev = S.material(brdf, [1, 1, 1], rough, WO, FRAME, grid)
    pdf = pdf.astype(np.float64)
    # the pdf over the upper hemisphere integrates to the sampler's acceptance rate
    acc = ok.mean()
    se_acc = np.sqrt(acc * (1 - acc) / N_SAMP) + 1e-4
    assert abs(pdf.sum() * dw - acc) < 5 * se_acc + 2e-3
    # and the accepted directions follow it: E[g(wi) 1{ok}] = integral of g pdf
    for g in (lambda w: w[:, 2], lambda w: w[:, 0] ** 2, lambda w: w[:, 0] * w[:, 1] + w[:, 2] ** 3):
        est = np.where(ok, g(d.astype(np.float64)), 0.0)
        quad = (g(grid.astype(np.float64)) * pdf).sum() * dw
        assert abs(est.mean() - quad) < 5 * _se(est) + 2e-3
    # the throughput of a sampled bounce, eval / pdf, averages to the hemisphere integral of eval
    p_s, e_s = S.material(brdf, [1, 1, 1], rough, WO, FRAME, d[ok])
    keep = p_s > 0
    tp = np.zeros(N_SAMP)
    tp[np.flatnonzero(ok)[keep]] = e_s[keep, 0] / p_s[keep]
    assert abs(tp.mean() - ev[:, 0].astype(np.float64).sum() * dw) < 5 * _se(tp) + 2e-3
    # energy: no material returns more than arrives
    assert ev[:, 0].astype(np.float64).sum() * dw <= 1.0 + 1e-2


def test_materials_vanish_below_the_surface():
    w = np.float32([[0.3, 0.1, -0.5], [0.0, 0.0, -1.0]])
    for brdf in (S.BLINN_PHONG, S.GGX):
        pdf, ev = S.material(brdf, [0.5, 0.6, 0.7], 0.4, WO, FRAME, w)
        assert (pdf == 0).all() and (ev == 0).all()
        # and above it when the view comes from below
        pdf, ev = S.material(brdf, [0.5, 0.6, 0.7], 0.4, -WO, FRAME, np.float32([[0, 0, 1]]))
        assert (pdf == 0).all() and (ev == 0).all()


def test_blinn_phong_eval_is_albedo_times_pdf():
    grid, _ = _hemisphere_grid(64, 64)
    pdf, ev = S.material(S.BLINN_PHONG, [0.25, 0.5, 0.75], 0.3, WO, FRAME, grid)
    np.testing.assert_array_equal(ev, np.float32([0.25, 0.5, 0.75]) * pdf[:, None])


# ---------------------------------------------------------- triangles, boxes, frames

def _sphere_dirs(n, seed):
    v = np.random.default_rng(seed).normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def test_triangle_pdf_integrates_to_one():
    tri = np.float32([[-0.4, 0.5, -0.3], [0.6, 0.6, -0.2], [0.1, 0.4, 0.7]])
    n = 400000
    d = _sphere_dirs(n, 11)
    pdf = S.triangle_pdf(np.zeros((n, 3), np.float32), d, tri).astype(np.float64)
    est = pdf * 4 * np.pi
    assert abs(est.mean() - 1.0) < 5 * _se(est)


def test_hit_bbox_against_fp64_slabs():
    rng = np.random.default_rng(21)
    n = 20000
    o = (rng.random((n, 3)) * 4 - 2).astype(np.float32)
    d = _sphere_dirs(n, 22)
    lo, hi = np.float32([-0.5, -0.3, -0.4]), np.float32([0.6, 0.2, 0.5])
    got = S.hit_bbox(o, d, lo, hi)
    o64, d64 = o.astype(np.float64), d.astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        t0, t1 = (lo - o64) / d64, (hi - o64) / d64
    tn = np.maximum(np.fmin(t0, t1).max(1), 0.0)
    tf = np.fmax(t0, t1).min(1)
    clear = np.abs(tn - tf) > 1e-4  # away from grazing cases
    assert clear.mean() > 0.95
    np.testing.assert_array_equal(got[clear], (tn <= tf)[clear])
    assert got.any() and not got.all()


def test_make_tanspace_orthonormal():
    n = _sphere_dirs(5000, 31)
    n[:4] = [[1, 0, 0], [0, 1, 0], [0, 0, -1], [0.6, 0.8, 0]]
    t, b = S.make_tanspace(n)
    for a in (t, b):
        np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-6)
    for x, y in ((t, n), (b, n), (t, b)):
        assert np.abs((x * y).sum(1)).max() < 1e-6
    np.testing.assert_allclose(b, np.cross(n, t), atol=1e-6)


# ------------------------------------------------------------------- scenes

def _quad(y, half, up, x0=0.0, z0=0.0):
    """Two triangles of the square |x - x0|, |z - z0| <= half at height y,
    wound so their geometric normal is +y (up) or -y."""
    a, b = [x0 - half, y, z0 - half], [x0 + half, y, z0 - half]
    c, d = [x0 + half, y, z0 + half], [x0 - half, y, z0 + half]
    tris = [[a, d, c], [a, c, b]] if up else [[a, b, c], [a, c, d]]
    n = [0, 1, 0] if up else [0, -1, 0]
    return np.float32(tris), np.float32([[n] * 3] * 2)


def floor_and_light(rough=0.5, albedo=(0.8, 0.7, 0.6), light_e=(6.0, 6.0, 6.0)):
    fv, fn = _quad(0.0, 1.0, True)
    lv, ln = _quad(1.0, 0.25, False, x0=0.2)
    return S.Scene(np.concatenate([fv, lv]), np.concatenate([fn, ln]), [0, 0, 1, 1],
                   albedo=[albedo, (0, 0, 0)], emissive=[(0, 0, 0), light_e], metal_rough=[(0, rough), (0, 0.5)])


CAM = S.camera(eye=(0.0, 0.9, 1.6), target=(0.0, 0.0, 0.0), up=(0, 1, 0), yfov=0.9, width=12, height=9)


def textured_scene(seed=5):
    """A floor and a back wall under an emissive quad, every material
    textured: checker albedo and random metal / roughness on the floor, an
    albedo texture on the wall, a normal map on both, an emission texture on
    the light.  Texture coordinates repeat past [0, 1] and go negative;
    tangents flip sign between the floor's two triangles."""
    rng = np.random.default_rng(seed)
    fv, fn = _quad(0.0, 1.0, True)
    wv = np.float32([[[-1, 0, -1], [1, 0, -1], [1, 1.2, -1]], [[-1, 0, -1], [1, 1.2, -1], [-1, 1.2, -1]]])
    wn = np.float32([[[0, 0, 1]] * 3] * 2)
    lv, ln = _quad(1.0, 0.25, False, x0=0.2)
    verts = np.concatenate([fv, wv, lv])
    normals = np.concatenate([fn, wn, ln])
    obj = [0, 0, 1, 1, 2, 2]
    tc = np.concatenate([(fv[..., [0, 2]] + 1.0) * 1.3, wv[..., [0, 1]] * 0.8 - 0.3, (lv[..., [0, 2]] - 0.2) * 2.0 + 0.5])
    tg = np.zeros((6, 3, 4), np.float32)
    tg[0, :, :] = [1, 0, 0, 1]
    tg[1, :, :] = [1, 0, 0, -1]
    tg[2:4, :, :] = [1, 0, 0, 1]
    tg[4:, :, :] = [0, 0, 1, 1]
    checker = np.where((np.add.outer(np.arange(8), np.arange(8)) % 2)[..., None] == 0,
                       rng.integers(150, 256, (8, 8, 4)), rng.integers(20, 90, (8, 8, 4))).astype(np.uint8)
    wall = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    metal_rough = np.stack([rng.integers(0, 256, (4, 4)), rng.integers(40, 256, (4, 4)),
                            np.zeros((4, 4)), np.full((4, 4), 255)], -1).astype(np.uint8)
    normal = np.stack([rng.integers(100, 156, (4, 4)), rng.integers(100, 156, (4, 4)),
                       rng.integers(220, 256, (4, 4)), np.full((4, 4), 255)], -1).astype(np.uint8)
    emit = rng.integers(180, 256, (2, 2, 4), dtype=np.uint8)
    textures = [checker, wall, metal_rough, normal, emit]
    obj_tex = [[0, -1, 2, 3], [1, -1, -1, 3], [-1, 4, -1, -1]]
    return S.Scene(verts, normals, obj, albedo=[(0.8, 0.7, 0.6), (0.5, 0.5, 0.5), (0, 0, 0)],
                   emissive=[(0, 0, 0), (0, 0, 0), (6.0, 6.0, 6.0)],
                   metal_rough=[(0.2, 0.5), (0.0, 0.7), (0.0, 0.5)], texcoords=tc, tangents=tg,
                   textures=textures, obj_tex=obj_tex)


def _texture_numpy(im, u, v, lut):
    """Bilinear at level 0 with repeat addressing of the sRGB-decoded
    texels, in FP32, operations in the restatement's order."""
    f32 = np.float32
    h, w = im.shape[:2]

    def wrap(x):
        with np.errstate(invalid="ignore"):
            f = (x - np.floor(x)).astype(f32)
        return np.where((f >= 0) & (f < 1), f, f32(0))

    fx = wrap(u) * f32(w) - f32(0.5)
    fy = wrap(v) * f32(h) - f32(0.5)
    x0, y0 = np.floor(fx), np.floor(fy)
    ax, ay = (fx - x0).astype(f32), (fy - y0).astype(f32)
    i0, j0 = x0.astype(np.int64), y0.astype(np.int64)
    i0 = np.where(i0 < 0, w - 1, i0)
    j0 = np.where(j0 < 0, h - 1, j0)
    i1 = np.where(i0 + 1 == w, 0, i0 + 1)
    j1 = np.where(j0 + 1 == h, 0, j0 + 1)
    dec = np.concatenate([lut[im[..., :3]], (im[..., 3:] / f32(255)).astype(f32)], -1).astype(f32)
    t00, t10, t01, t11 = dec[j0, i0], dec[j0, i1], dec[j1, i0], dec[j1, i1]
    ax, ay = ax[:, None], ay[:, None]
    one = f32(1)
    return ((t00 * (one - ax) + t10 * ax) * (one - ay) + (t01 * (one - ax) + t11 * ax) * ay).astype(f32)


def test_texture_sampling():
    """The restatement's texture(): the sRGB decode within 6 ulp of FP64 (its
    FP32 base (c + 0.055) / 1.055 rounds once or twice and the 2.4th power
    scales that error by 2.4), and
    the bilinear repeat blend equal to an independent FP32 version of it,
    including coordinates far outside [0, 1], negative, on texel centres
    and edges, and NaN / infinite (which read the texel at 0)."""
    lut = S.srgb_decode()
    c = np.arange(256) / 255.0
    ref = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
    ulp = np.spacing(np.maximum(ref, 1e-30).astype(np.float32)).astype(np.float64)
    assert (np.abs(lut - ref) / ulp).max() <= 6.0
    assert lut[0] == 0.0 and lut[255] == 1.0
    rng = np.random.default_rng(3)
    for h, w in ((1, 1), (1, 5), (7, 3), (16, 16)):
        im = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        u = np.concatenate([rng.uniform(-3, 4, 300), (np.arange(w) + 0.5) / w, np.arange(w + 1) / w,
                            [-1e-9, 1e-9, -0.0, 1e7, -1e7, np.nan, np.inf, -np.inf]]).astype(np.float32)
        v = np.concatenate([rng.uniform(-3, 4, 300), rng.uniform(0, 1, w), rng.uniform(0, 1, w + 1),
                            [0.5, 0.5, 0.5, 0.5, 0.5, 0.25, np.nan, 2.5]]).astype(np.float32)
        got = S.texture(im, u, v)
        want = _texture_numpy(im, u, v, lut)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        assert np.isfinite(got).all()


def test_textures_change_the_frame():
    """Each texture kind reaches the image: without the albedo checker, the
    emission texture or the normal map the frame differs."""
    sc = textured_scene()
    base = sc.render(CAM, integrator=S.MIS, samples=4, seed=3, use_normal_map=True)
    assert base.max() > 0.0
    for k in range(4):
        tex = sc.obj_tex.copy()
        if (tex[:, k] < 0).all():
            continue
        tex[:, k] = -1
        alt = S.Scene(sc.verts, sc.normals, sc.obj, sc.albedo, sc.emissive, sc.metal_rough, texcoords=sc.texcoords,
                      tangents=sc.tangents, textures=sc.textures, obj_tex=tex)
        img = alt.render(CAM, integrator=S.MIS, samples=4, seed=3, use_normal_map=True)
        assert not np.array_equal(img, base), k
    flat = sc.render(CAM, integrator=S.MIS, samples=4, seed=3, use_normal_map=False)
    assert not np.array_equal(flat, base)


def test_light_pdf_integrates_to_one():
    sc = floor_and_light()
    n = 400000
    d = _sphere_dirs(n, 41)
    p = np.tile(np.float32([0.1, 0.0, 0.2]), (n, 1))
    est = sc.light_pdf(p, d).astype(np.float64) * 4 * np.pi
    assert abs(est.mean() - 1.0) < 5 * _se(est)


def _rows(sc, seeds, **kw):
    """Per-seed renders reduced to the mean of each image row (channel 0)."""
    return np.stack([sc.render(CAM, seed=s, **kw)[..., 0].mean(1) for s in seeds]).astype(np.float64)


@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_integrators_agree_on_direct_lighting(brdf):
    """Floor under an area light, nothing to bounce off twice: direct
    lighting, material sampling to depth 2, MIS to depth 2 (and to depth 8
    with Russian roulette) and ReSTIR's direct-only mode all estimate the
    same image.  Compared per image row and over the whole image, each
    against the standard error of the per-seed means."""
    sc = floor_and_light()
    seeds = range(1, 9)
    ref = _rows(sc, seeds, integrator=S.DIRECT, brdf=brdf, samples=96, use_rr=False)
    assert ref.mean(0).max() > 0.05  # the floor is lit
    for integ, depth, rr in ((S.MATERIAL, 2, False), (S.MIS, 2, False), (S.MIS, 8, True),
                             (S.RESTIR_DIRECT, 8, False), (S.RESTIR, 8, True)):
        got = _rows(sc, seeds, integrator=integ, brdf=brdf, samples=96, max_depth=depth, use_rr=rr)
        _agree(got, ref, (integ, depth, rr))


def _agree(got, ref, what):
    n = got.shape[0]
    se = np.sqrt(ref.var(0, ddof=1) / n + got.var(0, ddof=1) / n)
    lit = se > 0  # rows the light reaches; rows of clear colour agree to rounding
    np.testing.assert_allclose(got.mean(0)[~lit], ref.mean(0)[~lit], rtol=1e-5)
    z = np.abs(got.mean(0) - ref.mean(0))[lit] / se[lit]
    assert z.max() < 5.0, (what, z)
    whole_se = np.sqrt(ref.mean(1).var(ddof=1) / n + got.mean(1).var(ddof=1) / n)
    assert abs(got.mean() - ref.mean()) < 5 * whole_se, what


def corner_and_light(brdf_rough=0.6, albedo=0.35):
    """A floor and two walls meeting in a corner under an area light: light
    reaches the camera after several bounces."""
    fv, fn = _quad(0.0, 1.0, True)
    # the wall x = -1 (normal +x) and the wall z = -1 (normal +z), as rotated floors
    wx = fv[..., [1, 0, 2]].copy()
    wx[..., 0] -= 1.0
    wx[..., 1] += 1.0
    wz = fv[..., [0, 2, 1]].copy()
    wz[..., 2] -= 1.0
    wz[..., 1] += 1.0
    nx = np.broadcast_to(np.float32([1, 0, 0]), (2, 3, 3))
    nz = np.broadcast_to(np.float32([0, 0, 1]), (2, 3, 3))
    lv, ln = _quad(1.2, 0.2, False, x0=0.1, z0=0.1)
    a = (albedo,) * 3
    return S.Scene(np.concatenate([fv, wx, wz, lv]), np.concatenate([fn, nx, nz, ln]), [0, 0, 1, 1, 2, 2, 3, 3],
                   albedo=[a, a, a, (0, 0, 0)], emissive=[(0, 0, 0)] * 3 + [(8.0, 8.0, 8.0)],
                   metal_rough=[(0, brdf_rough)] * 3 + [(0, 0.5)])


@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_integrators_agree_with_interreflection(brdf):
    """ReSTIR and material sampling to the same depth count the same paths;
    MIS to that depth differs from them only by part of the paths of the
    last bounce, negligible at albedo 0.35 and depth 8."""
    sc = corner_and_light()
    seeds = range(11, 19)
    ref = _rows(sc, seeds, integrator=S.MATERIAL, brdf=brdf, samples=64, max_depth=8, use_rr=False)
    one = _rows(sc, seeds, integrator=S.MATERIAL, brdf=brdf, samples=64, max_depth=2, use_rr=False)
    assert ref.mean() > one.mean() * 1.02  # inter-reflection adds light
    for integ, rr in ((S.RESTIR, False), (S.MIS, False), (S.MIS, True)):
        got = _rows(sc, seeds, integrator=integ, brdf=brdf, samples=64, max_depth=8, use_rr=rr)
        _agree(got, ref, (integ, rr))


def test_view_projection_maps_first_hits_to_their_pixels():
    sc = floor_and_light()
    _, g = sc.render(CAM, integrator=S.DIRECT, samples=1, gbuffer=True)
    hit = np.abs(g[..., 3:6]).sum(-1) > 0
    M = S.view_projection(CAM).astype(np.float64)
    p = np.concatenate([g[..., :3].astype(np.float64), np.ones(g.shape[:2] + (1,))], -1) @ M.T
    uv = (p[..., :2] / p[..., 3:4] + 1.0) * 0.5 * np.float64([CAM.width, CAM.height])
    ys, xs = np.mgrid[0:CAM.height, 0:CAM.width]
    np.testing.assert_allclose(uv[hit], np.stack([xs, ys], -1)[hit] + 0.5, atol=1e-3)


def _frames(sc, seed, nframes=4, temporal=False, cam=CAM, **kw):
    """nframes accumulated frames of a still camera (frames after the first
    jitter their rays); row means of the image, and the temporal state."""
    st = S.TemporalState(cam) if temporal else None
    img = np.zeros((cam.height, cam.width, 3), np.float32)
    n_first = None
    for frame in range(nframes):
        _, g = sc.render(cam, frame=frame, seed=seed * 16 + frame, image=img, gbuffer=True, temporal=st, **kw)
        if st is not None:
            if frame == 0:
                n_first = st.out_res["n_seen"].copy()
            st.advance(g, cam)
    return img[..., 0].mean(1).astype(np.float64), st, n_first


def test_restir_temporal_reuse_is_unbiased():
    """ReSTIR direct-only reusing the previous frame's reservoirs
    (rt.rgen:456-479), over four accumulated frames of a still camera,
    estimates what direct lighting does over the same frames; reuse did take
    place."""
    sc = floor_and_light()
    seeds = range(21, 29)
    ref = np.stack([_frames(sc, sd, integrator=S.DIRECT, samples=24, use_rr=False)[0] for sd in seeds])
    rows = [_frames(sc, sd, temporal=True, integrator=S.RESTIR_DIRECT, samples=24, use_rr=False)[0]
            for sd in seeds]
    _agree(np.stack(rows), ref, "restir temporal")
    # reuse took place: with one sample per frame (so that reuse within the
    # pixel cannot fill the reservoir) the candidates a floor pixel's
    # reservoir has seen grow by 4 per reused frame: 4 in frame 0, 16 in
    # frame 3.  The shader reuses only a previous hit within 0.1 of this one,
    # so the pixels must be finer than that on the floor (96 x 72 here).
    fine = S.camera(eye=(0.0, 0.9, 1.6), target=(0.0, 0.0, 0.0), up=(0, 1, 0), yfov=0.9, width=96, height=72)
    _, st, n0 = _frames(sc, 99, temporal=True, cam=fine, integrator=S.RESTIR_DIRECT, samples=1, use_rr=False)
    lit = n0 > 0
    assert (n0[lit] == 4).all()
    n3 = st.prev_res["n_seen"][lit]
    assert n3.max() == 16 and (n3 == 16).mean() > 0.8, np.bincount(n3)


def test_debug_view_shows_the_previous_buffers():
    """debug_view 1-3 (rt.rgen:647-671): each pixel shows the previous
    frame's position, normal or albedo at its first hit reprojected; with a
    still camera that is the pixel's own previous value; misses are 0."""
    sc = floor_and_light()
    st = S.TemporalState(CAM)
    _, g0 = sc.render(CAM, integrator=S.DIRECT, samples=1, gbuffer=True)
    st.advance(g0, CAM)
    hit = np.abs(g0[..., 3:6]).sum(-1) > 0
    for view in (1, 2, 3):
        img = sc.render(CAM, integrator=S.DIRECT, samples=1, frame=1, seed=5, debug_view=view, temporal=st)
        same = (img == g0[..., 3 * (view - 1):3 * view]).all(-1)
        assert same[hit].mean() > 0.9, view
        np.testing.assert_array_equal(img[~hit], 0.0)


def test_primary_misses_and_emitters():
    sc = floor_and_light()
    cam = S.camera(eye=(0.2, 0.5, 0.0), target=(0.2, 2.0, 0.0), up=(0, 0, 1), yfov=0.3, width=4, height=4)
    img = sc.render(cam, integrator=S.DIRECT, samples=2, clear=(0.1, 0.2, 0.3))
    # looking straight up at the light: every pixel sees its emission
    np.testing.assert_array_equal(img, np.full((4, 4, 3), 6.0, np.float32))
    cam = S.camera(eye=(0.0, 0.5, 0.0), target=(0.0, 0.5, 5.0), up=(0, 1, 0), yfov=0.2, width=4, height=4)
    for integ in (S.DIRECT, S.MATERIAL, S.MIS, S.RESTIR):
        img = sc.render(cam, integrator=integ, samples=2, clear=(0.1, 0.2, 0.3))
        np.testing.assert_array_equal(img, np.broadcast_to(np.float32([0.1, 0.2, 0.3]), (4, 4, 3)))


def test_mirror_floor_reflects_the_light_exactly():
    sc = floor_and_light(rough=0.0, albedo=(0.5, 0.25, 1.0))
    # the mirror image of the light (centre (0.2, 1, 0)) is at (0.2, -1, 0)
    cam = S.camera(eye=(0.2, 0.4, 0.0), target=(0.2, -1.0, 0.0), up=(0, 0, 1), yfov=0.1, width=3, height=3)
    img = sc.render(cam, integrator=S.MATERIAL, samples=1, max_depth=3, use_rr=False)
    np.testing.assert_allclose(img, np.broadcast_to(np.float32([3.0, 1.5, 6.0]), (3, 3, 3)), rtol=1e-6)


def test_qmc_jitter_is_seed_independent():
    """With Hammersley jitter (rt.rgen:553-555) a mirror render draws no
    random numbers, so two seeds give the same frame; with random jitter on a
    later frame they do not."""
    sc = floor_and_light(rough=0.0)
    kw = dict(integrator=S.MATERIAL, samples=4, max_depth=3, use_rr=False, frame=2, max_frame=8)
    a = sc.render(CAM, qmc=True, seed=1, **kw)
    b = sc.render(CAM, qmc=True, seed=2, **kw)
    np.testing.assert_array_equal(a, b)
    c = sc.render(CAM, qmc=False, seed=1, **kw)
    d = sc.render(CAM, qmc=False, seed=2, **kw)
    assert not np.array_equal(c, d)


def test_metalness_mixes_albedo():
    fv, fn = _quad(0.0, 1.0, True)
    lv, ln = _quad(1.0, 0.25, False)
    sc = S.Scene(np.concatenate([fv, lv]), np.concatenate([fn, ln]), [0, 0, 1, 1],
                 albedo=[(0.8, 0.4, 0.2), (0, 0, 0)], emissive=[(0, 0, 0), (5, 5, 5)],
                 metal_rough=[(0.25, 0.5), (0, 0.5)])
    _, g = sc.render(CAM, integrator=S.DIRECT, samples=1, use_metalness=True, gbuffer=True)
    on_floor = (np.abs(g[..., 3:6]).sum(-1) > 0) & (np.abs(g[..., 1]) < 1e-6)
    want = np.float32(0.04) * np.float32(0.75) + np.float32([0.8, 0.4, 0.2]) * np.float32(0.25)
    np.testing.assert_allclose(g[on_floor][:, 6:9], np.broadcast_to(want, (on_floor.sum(), 3)), rtol=1e-6)


def test_render_is_deterministic_and_blends_frames():
    sc = floor_and_light()
    a = sc.render(CAM, integrator=S.MIS, samples=4, seed=7)
    b = sc.render(CAM, integrator=S.MIS, samples=4, seed=7)
    np.testing.assert_array_equal(a, b)
    c = sc.render(CAM, integrator=S.MIS, samples=4, seed=8)
    assert not np.array_equal(a, c)
    # frame 1 blends half and half into the previous image: rendered onto
    # zeros it leaves half its own average, onto `a` that plus half of `a`
    img = a.copy()
    half_new = sc.render(CAM, integrator=S.MIS, samples=4, seed=9, frame=1)
    sc.render(CAM, integrator=S.MIS, samples=4, seed=9, frame=1, image=img)
    np.testing.assert_array_equal(img, a * np.float32(0.5) + half_new)


def test_gbuffer_holds_first_hit():
    sc = floor_and_light()
    img, g = sc.render(CAM, integrator=S.DIRECT, samples=1, gbuffer=True)
    hit = np.abs(g[..., 3:6]).sum(-1) > 0
    assert hit.any()
    np.testing.assert_allclose(np.linalg.norm(g[hit][:, 3:6], axis=1), 1.0, atol=1e-6)
    on_floor = hit & (np.abs(g[..., 1]) < 1e-6)
    np.testing.assert_allclose(g[on_floor][:, 6:9], np.broadcast_to(np.float32([0.8, 0.7, 0.6]),
                                                                     (on_floor.sum(), 3)))


def test_render_refuses_bad_arguments():
    sc = floor_and_light()
    for kw in ({"integrator": 5}, {"brdf": 2}, {"samples": 0}, {"qmc": True, "max_frame": 0}):
        with pytest.raises(ValueError):
            sc.render(CAM, **kw)
    dark = S.Scene(*[a for a in (_quad(0.0, 1.0, True))], [0, 0], albedo=[(1, 1, 1)], emissive=[(0, 0, 0)],
                   metal_rough=[(0, 0.5)])
    with pytest.raises(ValueError):  # light sampling with no light
        dark.render(CAM, integrator=S.DIRECT)
    dark.render(CAM, integrator=S.MATERIAL, samples=1)  # material sampling needs none


# ------------------------------------------------------- the reference's scene

def cbox_shade_scene():
    """The reference's Cornell box (media/cbox/cbox.gltf, from the committed
    fixture): one object per instance, world-space vertices and normals (the
    inverse-transpose of the instance matrix), the primitive's material."""
    from pathlib import Path

    z = np.load(Path(__file__).resolve().parent / "golden" / "cbox_scene.npz")
    voff, toff = z["vert_offsets"], z["tri_offsets"]
    V, N, Tr = [], [], []
    albedo, emissive, mr, obj = [], [], [], []
    for i, (j, T) in enumerate(zip(z["instance_primitive"], z["instance_transform"])):
        v = z["verts"][voff[j]:voff[j + 1]].astype(np.float64)
        n = z["normals"][voff[j]:voff[j + 1]].astype(np.float64)
        tri = z["tris"][toff[j]:toff[j + 1]]
        M = T.astype(np.float64)
        V.append((v @ M[:, :3].T + M[:, 3])[tri])
        N.append((n @ np.linalg.inv(M[:, :3]))[tri])
        obj.append(np.full(len(tri), i, np.int32))
        albedo.append(z["prim_albedo"][j])
        emissive.append(z["prim_emissive"][j])
        mr.append(z["prim_metal_rough"][j])
    return S.Scene(np.concatenate(V), np.concatenate(N), np.concatenate(obj), albedo, emissive, mr)


def test_gltf_world_shading_matches_the_fixture_scene(cpq, reference_root):
    """The library's reader, flattened by GltfScene.world_shading, gives the
    shading scene built here from the fixture (the reference's Cornell box)."""
    path = reference_root / "media" / "cbox" / "cbox.gltf"
    if not path.exists():
        pytest.skip("reference media not present")
    w = cpq.load_gltf(str(path)).world_shading()
    sc = cbox_shade_scene()
    np.testing.assert_allclose(w["verts"].reshape(-1, 9), sc.verts, rtol=0, atol=1e-5)
    np.testing.assert_allclose(w["normals"].reshape(-1, 9), sc.normals, rtol=0, atol=1e-5)
    np.testing.assert_array_equal(w["obj"], sc.obj)
    np.testing.assert_array_equal(w["materials"][:, 0:3], sc.albedo)
    np.testing.assert_array_equal(w["materials"][:, 3:6], sc.emissive)
    np.testing.assert_array_equal(w["materials"][:, 6:8], sc.metal_rough)


# the glTF's camera (node CamInst): on the +z axis looking down -z, vertical
# field of view 0.7175 rad at 4:3
CBOX_CAM = S.camera(eye=(0.0, 0.0, 19.992091970966317), target=(0.0, 0.0, 0.0), up=(0, 1, 0),
                    yfov=0.7175414562225342, width=32, height=24)


def test_cbox_renders():
    sc = cbox_shade_scene()
    img, g = sc.render(CBOX_CAM, integrator=S.DIRECT, samples=4, gbuffer=True, seed=3)
    assert np.isfinite(img).all() and img.min() >= 0.0
    # the ceiling light in view, at its emission exactly
    assert (img == 10.0).all(-1).sum() >= 1
    # the red and the green wall
    alb = g[..., 6:9]
    red = np.abs(alb - np.float32([1.0, 0.0, 1.0718736e-4])).max(-1) < 1e-6
    green = np.abs(alb - np.float32([0.054592282, 1.0, 0.0])).max(-1) < 1e-6
    assert red.sum() >= 4 and green.sum() >= 4
    assert (img[red][:, 0] >= img[red][:, 1]).all() and img[red][:, 0].mean() > 2 * img[red][:, 1].mean() + 1e-6
    assert img[green][:, 1].mean() > 2 * img[green][:, 0].mean()
    # indirect light and the mirror sphere's reflections add to direct light
    mis = sc.render(CBOX_CAM, integrator=S.MIS, samples=4, seed=3)
    assert np.isfinite(mis).all() and mis.min() >= 0.0
    assert mis.mean() > img.mean()


def _bp_eval64(albedo, rough, wo, n, wi):
    """Blinn-Phong eval of rtcommon.glsl:255-270 in FP64, independently of
    the restatement (wi: (k, 3))."""
    o_dn = -wo @ n
    i_dn = wi @ n
    h = wi - wo
    h /= np.linalg.norm(h, axis=-1, keepdims=True)
    e = 1.0 / rough
    pdf = (e + 1) / (2 * 3.141592) * np.maximum(h @ n, 0) ** e / (4 * (h @ -wo))
    return np.where((o_dn > 0) & (i_dn > 0), pdf, 0.0)[:, None] * albedo


def _ggx_eval64(albedo, rough, wo, n, wi):
    """GGX eval of rtcommon.glsl:281-324 in FP64."""
    o_dn = -wo @ n
    i_dn = wi @ n
    h = wi - wo
    h /= np.linalg.norm(h, axis=-1, keepdims=True)
    a2 = rough * rough
    n_dh = np.maximum(h @ n, 0)
    b = n_dh * n_dh * (a2 - 1) + 1
    d = a2 / (3.141592 * b * b)
    g = 2 * o_dn * i_dn / (o_dn * np.sqrt(a2 + (1 - a2) * i_dn * i_dn) + i_dn * np.sqrt(a2 + (1 - a2) * o_dn * o_dn))
    f = albedo + (1 - albedo) * ((1 - i_dn) ** 5)[:, None]
    ev = f * (d * g / (4 * o_dn))[:, None]
    return np.where(((o_dn > 0) & (i_dn > 0))[:, None], ev, 0.0)


@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
def test_direct_lighting_matches_quadrature(brdf):
    """Each floor pixel's direct-lighting estimate (rt.rgen:392-412) against
    an FP64 midpoint quadrature of the same integral over the light's area,
    sum of eval(wi) L |n_light . wi| / r^2 dA, written independently here."""
    albedo, rough, emit = np.float64([0.8, 0.7, 0.6]), 0.5, 6.0
    sc = floor_and_light(rough=rough, albedo=tuple(albedo), light_e=(emit,) * 3)
    _, g = sc.render(CAM, integrator=S.DIRECT, samples=1, gbuffer=True)
    seeds = range(31, 39)
    imgs = np.stack([sc.render(CAM, integrator=S.DIRECT, brdf=brdf, samples=128, seed=s)
                     for s in seeds]).astype(np.float64)
    mean, se = imgs.mean(0), imgs.std(0, ddof=1) / np.sqrt(len(seeds))
    # the light: y = 1, x in [-0.05, 0.45], z in [-0.25, 0.25], facing down
    k = 96
    u = (np.arange(k) + 0.5) / k
    X, Z = np.meshgrid(-0.05 + 0.5 * u, -0.25 + 0.5 * u, indexing="ij")
    lp = np.stack([X.ravel(), np.ones(k * k), Z.ravel()], -1)
    dA = (0.5 / k) ** 2
    eye = np.float64(list(CAM.eye))
    ev = _bp_eval64 if brdf == S.BLINN_PHONG else _ggx_eval64
    checked = 0
    for y in range(CAM.height):
        for x in range(CAM.width):
            p = g[y, x, :3].astype(np.float64)
            if abs(p[1]) > 1e-6 or not np.any(g[y, x, 3:6]):
                continue  # not the floor
            wo = (p - eye) / np.linalg.norm(p - eye)
            d = lp - p
            r2 = (d * d).sum(1)
            wi = d / np.sqrt(r2)[:, None]
            want = (ev(albedo, rough, wo, np.float64([0, 1, 0]), wi) * (emit * np.abs(wi[:, 1]) / r2 * dA)[:, None]).sum(0)
            z = np.abs(mean[y, x] - want) / (se[y, x] + 1e-4 * want + 1e-9)
            assert z.max() < 5.0, (brdf, y, x, mean[y, x], want, se[y, x])
            checked += 1
    assert checked >= 40
