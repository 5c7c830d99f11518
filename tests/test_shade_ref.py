"""The shading restatement against the reference's own shader code.

oracle/make_ref_shade.py compiles the reference's rtcommon.glsl and
restir.glsl as C++ (syntax rewrites only, against oracle/glsl_shim.h) from a
checkout of the reference; these tests run both on the same inputs.  Where
the shader uses only IEEE operations and sqrt (random numbers, reservoir
updates, the triangle pdf, the slab test, the tangent frame, triangle
sampling) the two agree bit for bit; where it calls pow, sin or cos (the
materials and hemisphere samplers) the restatement's own routines stand
against the C library's, so results agree to a few ulp and sampled
directions to 1e-5.  Skipped where no checkout of the reference exists.
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


def test_random_numbers_bit_exact():
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2**32, 5000, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 2**32, 5000, dtype=np.uint64).astype(np.uint32)
    np.testing.assert_array_equal(S.tea(a, b), S.tea(a, b, ref=True))
    for seed in (0, 1, 0xDEADBEEF):
        for x, y in zip(S.lcg_stream(seed, 10000), S.lcg_stream(seed, 10000, ref=True)):
            np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(S.radical_inverse(a), S.radical_inverse(a, ref=True))


def test_reservoir_updates_bit_exact():
    w = np.random.default_rng(2).random(20000).astype(np.float32)
    w[::7] = 0.0
    for seed in (3, 99):
        for x, y in zip(S.reservoir_stream(seed, w), S.reservoir_stream(seed, w, ref=True)):
            np.testing.assert_array_equal(x, y)


def test_geometry_bit_exact():
    n = 20000
    rng = np.random.default_rng(4)
    o = (rng.random((n, 3)) * 2 - 1).astype(np.float32)
    d = _dirs(n, 5)
    tri = np.float32([[-0.4, 0.5, -0.3], [0.6, 0.6, -0.2], [0.1, 0.4, 0.7]])
    got, want = S.triangle_pdf(o, d, tri), S.triangle_pdf(o, d, tri, ref=True)
    assert (want > 0).sum() > 500
    np.testing.assert_array_equal(got, want)
    lo, hi = np.float32([-0.5, -0.3, -0.4]), np.float32([0.6, 0.2, 0.5])
    np.testing.assert_array_equal(S.hit_bbox(o * 3, d, lo, hi), S.hit_bbox(o * 3, d, lo, hi, ref=True))
    for x, y in zip(S.make_tanspace(d), S.make_tanspace(d, ref=True)):
        np.testing.assert_array_equal(x, y)


def test_triangle_sampling_bit_exact():
    for x, y in zip(S.sample(S.TRIANGLE_SAMPLE, 50000, 6, FRAME), S.sample(S.TRIANGLE_SAMPLE, 50000, 6, FRAME,
                                                                                ref=True)):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("brdf", [S.BLINN_PHONG, S.GGX])
@pytest.mark.parametrize("rough", [0.05, 0.3, 0.8])
def test_materials_agree(brdf, rough):
    wo = np.float32([0.45, -0.2, -0.87])
    wo /= np.linalg.norm(wo)
    wi = _dirs(50000, 7)
    p0, e0 = S.material(brdf, [0.9, 0.5, 0.2], rough, wo, FRAME, wi)
    p1, e1 = S.material(brdf, [0.9, 0.5, 0.2], rough, wo, FRAME, wi, ref=True)
    np.testing.assert_array_equal(p0 == 0, p1 == 0)
    np.testing.assert_allclose(p0, p1, rtol=2e-6, atol=1e-30)
    np.testing.assert_allclose(e0, e1, rtol=2e-6, atol=1e-30)


@pytest.mark.parametrize("kind,param", [(S.UNIFORM_HEMISPHERE, 0.0), (S.COSINE_HEMISPHERE, 0.0),
                                        (S.COSPOW_HEMISPHERE, 7.0), (S.GGX_SAMPLE, 0.3), (S.BP_SAMPLE, 0.2)])
def test_samplers_agree(kind, param):
    wo = np.float32([0.3, 0.1, -0.95])
    wo /= np.linalg.norm(wo)
    d0, ok0 = S.sample(kind, 50000, 8, FRAME, param, wo=wo)
    d1, ok1 = S.sample(kind, 50000, 8, FRAME, param, wo=wo, ref=True)
    # the same random numbers drive both: directions agree to the ulps of sin/cos/pow
    np.testing.assert_allclose(d0, d1, rtol=0, atol=1e-5)
    # acceptance can differ only for directions grazing the surface
    diff = ok0 != ok1
    assert diff.mean() < 1e-4 and np.all(np.abs(d1[diff] @ FRAME[2]) < 1e-5)
