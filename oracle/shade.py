"""ORACLE — test infrastructure only.

ctypes wrapper of the FP32 restatement of the reference's path-tracer
shading math (oracle/shade_oracle.c: rtcommon.glsl, rt.rgen, restir.glsl).
Only tests/ may import this module; the product never does.

Everything here runs either on the restatement or (``ref=True``) on the
reference's own rtcommon.glsl, restir.glsl and rt.rgen compiled as C++
(make_ref_shade.py), which share only what GLSL leaves to the
implementation (sin / cos / pow / exp and the ray tracer); the tests
require the two to agree bit for bit, and pin the mathematics besides (pdf
normalisation, sampler/pdf agreement, unbiased integrators agreeing in
expectation, a quadrature of direct lighting).
"""
from __future__ import annotations

import ctypes
from ctypes import Structure, byref, c_float, c_int32, c_int64, c_uint32, c_void_p

import numpy as np

from . import oracle as _o

# orc_sh_sample kinds
UNIFORM_HEMISPHERE, COSINE_HEMISPHERE, COSPOW_HEMISPHERE, GGX_SAMPLE, BP_SAMPLE, TRIANGLE_SAMPLE = range(6)
BLINN_PHONG, GGX = 0, 1
DIRECT, MATERIAL, MIS, RESTIR_DIRECT, RESTIR = range(5)


class ShadeScene(Structure):
    _fields_ = [("nt", c_int64), ("verts", c_void_p), ("normals", c_void_p), ("obj", c_void_p),
                ("nobj", c_int32), ("albedo", c_void_p), ("emissive", c_void_p), ("metal_rough", c_void_p),
                ("texcoords", c_void_p), ("tangents", c_void_p), ("obj_tex", c_void_p), ("ntex", c_int32),
                ("tex_size", c_void_p), ("tex_off", c_void_p), ("texels", c_void_p)]


class ShadeCamera(Structure):
    _fields_ = [("eye", c_float * 3), ("right", c_float * 3), ("up", c_float * 3), ("fwd", c_float * 3),
                ("tan_half_y", c_float), ("aspect", c_float), ("width", c_int32), ("height", c_int32)]


class ShadeParams(Structure):
    _fields_ = [("clear", c_float * 3), ("env", c_float * 3), ("samples", c_int32), ("max_depth", c_int32),
                ("qmc", c_int32), ("integrator", c_int32), ("brdf", c_int32), ("use_rr", c_int32),
                ("use_metalness", c_int32), ("frame", c_int32), ("max_frame", c_int32),
                ("new_samples", c_int32), ("temporal_multiplier", c_int32), ("use_temporal", c_int32),
                ("debug_view", c_int32), ("seed", c_uint32), ("use_normal_map", c_int32)]


class ShadeTemporal(Structure):
    _fields_ = [("prev_pv", c_void_p), ("prev_gbuf", c_void_p), ("prev_res", c_void_p), ("out_res", c_void_p)]


# orc_shade_reservoir
RESERVOIR = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 3), ("emissive", "<f4", 3), ("w_sum", "<f4"),
                      ("w", "<f4"), ("n_seen", "<u4")])
assert RESERVOIR.itemsize == 48


class TemporalState:
    """ReSTIR's state between frames: the previous frame's view-projection,
    first-hit buffer and reservoirs.  `advance` makes this frame's outputs
    the next frame's inputs."""

    def __init__(self, camera: "ShadeCamera"):
        self.h, self.w = camera.height, camera.width
        self.prev_pv = view_projection(camera)
        self.prev_gbuf = None
        self.prev_res = None
        self.out_res = np.zeros((self.h, self.w), RESERVOIR)

    def advance(self, gbuf, camera: "ShadeCamera"):
        self.prev_gbuf = np.ascontiguousarray(gbuf, np.float32)
        self.prev_res = self.out_res
        self.out_res = np.zeros((self.h, self.w), RESERVOIR)
        self.prev_pv = view_projection(camera)

    def _struct(self) -> ShadeTemporal:
        return ShadeTemporal(_p(self.prev_pv), _p(self.prev_gbuf), _p(self.prev_res), _p(self.out_res))


def _L():
    return _o.lib()


_ref = None


def ref_lib():
    """The reference's own shading functions (rtcommon.glsl, restir.glsl)
    compiled as C++ into oracle/_ref by make_ref_shade.py, or None where no
    checkout of the reference exists."""
    global _ref
    if _ref is None:
        from . import make_ref_shade

        path = make_ref_shade.build()
        if path is None:
            _ref = False
        else:
            L = ctypes.CDLL(str(path))
            P = c_void_p
            for name, args in [("ref_tea", [c_int64, P, P, P]), ("ref_lcg_stream", [c_uint32, c_int64, P, P]),
                               ("ref_radical_inverse", [c_int64, P, P]),
                               ("ref_sample", [c_int32, c_int64, c_uint32, P, c_float, P, P, P]),
                               ("ref_material", [c_int32, c_int64, P, c_float, P, P, P, P, P]),
                               ("ref_triangle_pdf", [c_int64, P, P, P, P]), ("ref_hit_bbox", [c_int64, P, P, P, P, P]),
                               ("ref_make_tanspace", [c_int64, P, P, P]),
                               ("ref_triangle_hit", [c_int64, P, P, P, P, P]),
                               ("ref_reservoir_stream", [c_uint32, c_int64, P, P, P])]:
                getattr(L, name).argtypes = args
                getattr(L, name).restype = None
            L.ref_render.argtypes = [P] * 6
            L.ref_render.restype = c_int32
            L.ref_tonemap.argtypes = [c_int32, c_float, c_float, c_int64, P, P]
            L.ref_tonemap.restype = c_int32
            _ref = L
    return _ref or None


def _fn(name: str, ref: bool):
    """orc_sh_<name> of the restatement, or ref_<name> of the reference's code."""
    if ref:
        L = ref_lib()
        if L is None:
            raise RuntimeError("the reference's shaders are not available here")
        return getattr(L, "ref_" + name)
    return getattr(_L(), "orc_sh_" + name)


def _p(a):
    return _o._p(a)


def _v3(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 3))


def tea(v0, v1, ref: bool = False) -> np.ndarray:
    a = np.ascontiguousarray(v0, np.uint32)
    b = np.ascontiguousarray(v1, np.uint32)
    out = np.empty(a.shape[0], np.uint32)
    _fn("tea", ref)(a.shape[0], _p(a), _p(b), _p(out))
    return out


def lcg_stream(seed: int, n: int, ref: bool = False):
    u = np.empty(n, np.uint32)
    f = np.empty(n, np.float32)
    _fn("lcg_stream", ref)(seed, n, _p(u), _p(f))
    return u, f


def radical_inverse(bits, ref: bool = False) -> np.ndarray:
    b = np.ascontiguousarray(bits, np.uint32)
    out = np.empty(b.shape[0], np.float32)
    _fn("radical_inverse", ref)(b.shape[0], _p(b), _p(out))
    return out


def reservoir_stream(seed: int, weights, ref: bool = False):
    """res_update over `weights` from one lcg stream: the selected index and
    w_sum after each update."""
    w = np.ascontiguousarray(weights, np.float32)
    chosen = np.empty(w.shape[0], np.int32)
    ws = np.empty(w.shape[0], np.float32)
    _fn("reservoir_stream", ref)(seed, w.shape[0], _p(w), _p(chosen), _p(ws))
    return chosen, ws


def _math(kind, x, y=None):
    xx = np.ascontiguousarray(x, np.float32)
    yy = np.ascontiguousarray(y if y is not None else np.zeros_like(xx), np.float32)
    out = np.empty(xx.shape[0], np.float32)
    _L().orc_sh_math(kind, xx.shape[0], _p(xx), _p(yy), _p(out))
    return out


def sin(x):
    return _math(0, x)


def cos(x):
    return _math(1, x)


def pow(x, y):  # noqa: A001 - the restatement's own pow
    return _math(2, x, y)


def exp(x):
    return _math(3, x)


FILMIC, EXPONENTIAL, NO_TONEMAP = range(3)


def tonemap(img, kind: int = EXPONENTIAL, exposure: float = 1.0, gamma: float = 2.2, ref: bool = False) -> np.ndarray:
    """tonemap.frag per colour component; defaults as effect.h:25-27."""
    a = np.ascontiguousarray(img, np.float32)
    out = np.empty_like(a)
    if _fn("tonemap", ref)(kind, exposure, gamma, a.size, _p(a), _p(out)) != 0:
        raise ValueError("unknown tone mapping")
    return out


def sample(kind: int, n: int, seed: int, frame, param: float = 0.0, wo=None, ref: bool = False):
    """n draws of one sampler from one lcg stream: (directions or barycentrics, ok)."""
    f = np.ascontiguousarray(np.asarray(frame, np.float32).reshape(9))
    w = None if wo is None else np.ascontiguousarray(np.asarray(wo, np.float32).reshape(3))
    dirs = np.empty((n, 3), np.float32)
    ok = np.empty(n, np.uint8)
    _fn("sample", ref)(kind, n, seed, _p(f), param, _p(w), _p(dirs), _p(ok))
    return dirs, ok.astype(bool)


def material(brdf: int, albedo, roughness: float, wo, frame, wi, ref: bool = False):
    """(pdf, eval) of MAT_pdf / MAT_eval for directions wi at one shading point."""
    a = np.ascontiguousarray(np.asarray(albedo, np.float32).reshape(3))
    w = np.ascontiguousarray(np.asarray(wo, np.float32).reshape(3))
    f = np.ascontiguousarray(np.asarray(frame, np.float32).reshape(9))
    d = _v3(wi)
    pdf = np.empty(d.shape[0], np.float32)
    ev = np.empty((d.shape[0], 3), np.float32)
    _fn("material", ref)(brdf, d.shape[0], _p(a), roughness, _p(w), _p(f), _p(d), _p(pdf), _p(ev))
    return pdf, ev


def triangle_pdf(o, d, tri, ref: bool = False) -> np.ndarray:
    oo, dd = _v3(o), _v3(d)
    t = np.ascontiguousarray(np.asarray(tri, np.float32).reshape(9))
    out = np.empty(oo.shape[0], np.float32)
    _fn("triangle_pdf", ref)(oo.shape[0], _p(oo), _p(dd), _p(t), _p(out))
    return out


def triangle_hit_ref(o, d, tri):
    """The reference's own triangle_hit (rtcommon.glsl:181-202) per ray:
    (hit, hit point)."""
    oo, dd = _v3(o), _v3(d)
    t = np.ascontiguousarray(np.asarray(tri, np.float32).reshape(9))
    hit = np.empty(oo.shape[0], np.uint8)
    p = np.zeros_like(oo)
    _fn("triangle_hit", True)(oo.shape[0], _p(oo), _p(dd), _p(t), _p(hit), _p(p))
    return hit.astype(bool), p


def hit_bbox(o, d, bmin, bmax, ref: bool = False) -> np.ndarray:
    oo, dd = _v3(o), _v3(d)
    lo = np.ascontiguousarray(np.asarray(bmin, np.float32).reshape(3))
    hi = np.ascontiguousarray(np.asarray(bmax, np.float32).reshape(3))
    out = np.empty(oo.shape[0], np.uint8)
    _fn("hit_bbox", ref)(oo.shape[0], _p(oo), _p(dd), _p(lo), _p(hi), _p(out))
    return out.astype(bool)


def make_tanspace(n, ref: bool = False):
    nn = _v3(n)
    t = np.empty_like(nn)
    b = np.empty_like(nn)
    _fn("make_tanspace", ref)(nn.shape[0], _p(nn), _p(t), _p(b))
    return t, b


def texture_pack(images):
    """RGBA8 images (h, w, 4) uint8 -> (tex_size (n, 2) [w, h], tex_off (n + 1), texels)."""
    images = [np.ascontiguousarray(im, np.uint8) for im in images]
    for im in images:
        assert im.ndim == 3 and im.shape[2] == 4 and im.shape[0] > 0 and im.shape[1] > 0
    size = np.asarray([[im.shape[1], im.shape[0]] for im in images], np.int32).reshape(-1, 2)
    off = np.zeros(len(images) + 1, np.int64)
    off[1:] = np.cumsum([im.shape[0] * im.shape[1] for im in images])
    texels = np.concatenate([im.reshape(-1) for im in images]) if images else np.zeros(4, np.uint8)
    return size, off, np.ascontiguousarray(texels)


class Scene:
    """World-space triangles with per-vertex normals and a material per object
    (albedo, emission, metalness, roughness factors); an object whose
    emission factor has a component above zero is a light.  Objects'
    triangles are contiguous.  Optional: per-vertex texture coordinates
    (nt, 3, 2) and tangents (nt, 3, 4: xyz, w), RGBA8 sRGB textures (a list of
    (h, w, 4) uint8 images) and per object the texture replacing each factor
    (obj_tex (nobj, 4): albedo, emissive, metal_rough, normal; -1 none)."""

    def __init__(self, verts, normals, obj, albedo, emissive, metal_rough, *, texcoords=None, tangents=None,
                 textures=None, obj_tex=None):
        self.verts = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 9))
        self.normals = np.ascontiguousarray(np.asarray(normals, np.float32).reshape(-1, 9))
        self.obj = np.ascontiguousarray(obj, np.int32)
        self.albedo = np.ascontiguousarray(np.asarray(albedo, np.float32).reshape(-1, 3))
        self.emissive = np.ascontiguousarray(np.asarray(emissive, np.float32).reshape(-1, 3))
        self.metal_rough = np.ascontiguousarray(np.asarray(metal_rough, np.float32).reshape(-1, 2))
        nt = self.verts.shape[0]
        self.texcoords = None if texcoords is None else np.ascontiguousarray(
            np.asarray(texcoords, np.float32).reshape(nt, 6))
        self.tangents = None if tangents is None else np.ascontiguousarray(
            np.asarray(tangents, np.float32).reshape(nt, 12))
        self.textures = list(textures or [])
        self.obj_tex = None if obj_tex is None else np.ascontiguousarray(
            np.asarray(obj_tex, np.int32).reshape(-1, 4))
        if self.obj_tex is not None:
            assert self.obj_tex.shape[0] == self.albedo.shape[0]
            assert self.obj_tex.max() < len(self.textures) and self.obj_tex.min() >= -1
        self.tex_size, self.tex_off, self.texels = texture_pack(self.textures)

        def ptr(a):
            return None if a is None else a.ctypes.data

        self._s = ShadeScene(nt, self.verts.ctypes.data, self.normals.ctypes.data,
                             self.obj.ctypes.data, self.albedo.shape[0], self.albedo.ctypes.data,
                             self.emissive.ctypes.data, self.metal_rough.ctypes.data, ptr(self.texcoords),
                             ptr(self.tangents), ptr(self.obj_tex), len(self.textures), self.tex_size.ctypes.data,
                             self.tex_off.ctypes.data, self.texels.ctypes.data)

    def light_pdf(self, p, d) -> np.ndarray:
        pp, dd = _v3(p), _v3(d)
        out = np.empty(pp.shape[0], np.float32)
        _L().orc_sh_light_pdf(byref(self._s), pp.shape[0], _p(pp), _p(dd), _p(out))
        return out

    def render(self, camera: ShadeCamera, *, integrator=DIRECT, brdf=BLINN_PHONG, samples=8, max_depth=8,
               use_rr=True, qmc=False, use_metalness=False, frame=0, max_frame=256, new_samples=4,
               temporal_multiplier=16, use_temporal=True, debug_view=0, clear=(0.3, 0.3, 0.3),
               env=(0.0, 0.0, 0.0), seed=1, image=None, gbuffer=False, temporal: TemporalState | None = None,
               use_normal_map=False, ref: bool = False):
        """One frame, the reference's defaults unless given (rt.h:38-53;
        env_scale 0).  Returns the image (height, width, 3) and, if asked,
        the first-hit buffer (height, width, 9).  `temporal` carries ReSTIR's
        reservoirs between frames (its out_res is written).  With `ref` the
        frame comes from the reference's own rt.rgen compiled as C++
        (make_ref_shade.py) instead of the restatement."""
        p = ShadeParams((c_float * 3)(*clear), (c_float * 3)(*env), samples, max_depth, int(qmc), integrator,
                        brdf, int(use_rr), int(use_metalness), frame, max_frame, new_samples,
                        temporal_multiplier, int(use_temporal), debug_view, seed, int(use_normal_map))
        img = np.zeros((camera.height, camera.width, 3), np.float32) if image is None else image
        assert img.dtype == np.float32 and img.flags.c_contiguous and img.shape == (camera.height, camera.width, 3)
        g = np.zeros((camera.height, camera.width, 9), np.float32) if gbuffer else None
        ts = None if temporal is None else temporal._struct()
        rc = _fn("render", ref)(byref(self._s), byref(camera), byref(p), _p(img), _p(g),
                                None if ts is None else byref(ts))
        if rc != 0:
            raise ValueError("orc_sh_render refused its arguments")
        return (img, g) if gbuffer else img


def texture(image, u, v) -> np.ndarray:
    """The restatement's texture() on one RGBA8 sRGB image at arrays of
    (u, v): (n, 4) float32."""
    im = np.ascontiguousarray(image, np.uint8)
    u = np.ascontiguousarray(u, np.float32).reshape(-1)
    v = np.ascontiguousarray(v, np.float32).reshape(-1)
    out = np.empty((u.shape[0], 4), np.float32)
    fn = _L().orc_sh_texture
    for i in range(u.shape[0]):
        fn(im.shape[1], im.shape[0], _p(im), c_float(u[i]), c_float(v[i]), _p(out[i]))
    return out


def srgb_decode() -> np.ndarray:
    """The restatement's sRGB decode of each 8-bit value (256 floats)."""
    fn = _L().orc_sh_srgb_decode
    fn.restype = c_float
    return np.asarray([fn(i) for i in range(256)], np.float32)


def camera(eye, target, up, yfov: float, width: int, height: int) -> ShadeCamera:
    """Pinhole camera at eye looking at target (row 0 at the top)."""
    e = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - e
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    c3 = lambda v: (c_float * 3)(*[float(x) for x in v])  # noqa: E731
    return ShadeCamera(c3(e), c3(r), c3(u), c3(f), float(np.tan(0.5 * yfov)), width / height, width, height)


def view_projection(cam: ShadeCamera) -> np.ndarray:
    """4 x 4 row-major matrix taking a world point to the clip coordinates
    whose (x/w + 1)/2, (y/w + 1)/2 are the camera's image coordinates (row 0
    at the top), the inverse of the renderer's camera ray; w is the depth."""
    e, r, u, f = (np.asarray(v, np.float64) for v in (cam.eye, cam.right, cam.up, cam.fwd))
    sx, sy = cam.tan_half_y * cam.aspect, cam.tan_half_y
    m = np.zeros((4, 4))
    m[0, :3], m[0, 3] = r / sx, -np.dot(e, r) / sx
    m[1, :3], m[1, 3] = -u / sy, np.dot(e, u) / sy
    m[3, :3], m[3, 3] = f, -np.dot(e, f)
    return np.ascontiguousarray(m, np.float32)
