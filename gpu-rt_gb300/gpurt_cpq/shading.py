"""The reference's path tracer on the GPU (cp_shade_* of include/cpq.h).

Its ray-generation shader (src/shaders/rt/rt.rgen:567-677: camera rays, the
five integrators, Russian roulette, frame blending, ReSTIR with temporal
reuse, debug views) and tone mapping (src/shaders/tonemap.frag) as CUDA
kernels over the library's BVH, rendering into a device image instead of a
swapchain.  Defaults are the reference's UI defaults (src/rt/rt.h:38-53, with
the environment scale 0).
"""
from __future__ import annotations

from ctypes import byref, c_float, c_int32, c_void_p

import numpy as np
import torch

from ._lib import ShadeCamera, ShadeParams, check, lib
from .mesh import _check_dev, _ptr, _stream

DIRECT, MATERIAL, MIS, RESTIR_DIRECT, RESTIR = range(5)
BLINN_PHONG, GGX = 0, 1
FILMIC, EXPONENTIAL, NO_TONEMAP = range(3)
RESERVOIR_BYTES = 48  # cp_shade_reservoir: pos, normal, emissive (3 floats each), w_sum, w, n_seen


def camera(eye, target, up, yfov: float, width: int, height: int) -> ShadeCamera:
    """Pinhole camera at `eye` looking at `target` (row 0 at the top); yfov in radians."""
    e = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - e
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)

    def c3(v):
        return (c_float * 3)(*[float(x) for x in v])

    return ShadeCamera(c3(e), c3(r), c3(u), c3(f), float(np.tan(0.5 * yfov)), width / height, width, height)


def view_projection(cam: ShadeCamera) -> np.ndarray:
    """4 x 4 row-major matrix taking a world point to clip coordinates whose
    ((x/w + 1)/2, (y/w + 1)/2) are the camera's image coordinates (row 0 at
    the top): the inverse of the renderer's camera ray; w is the depth."""
    e, r, u, f = (np.asarray(v, np.float64) for v in (cam.eye, cam.right, cam.up, cam.fwd))
    sx, sy = cam.tan_half_y * cam.aspect, cam.tan_half_y
    m = np.zeros((4, 4))
    m[0, :3], m[0, 3] = r / sx, -np.dot(e, r) / sx
    m[1, :3], m[1, 3] = -u / sy, np.dot(e, u) / sy
    m[3, :3], m[3, 3] = f, -np.dot(e, f)
    return np.ascontiguousarray(m, np.float32)


class TemporalState:
    """ReSTIR's state between frames on the device: the previous frame's
    view-projection, first-hit buffer and reservoirs.  `advance` makes this
    frame's outputs the next frame's inputs."""

    def __init__(self, cam: ShadeCamera, device):
        self.h, self.w = cam.height, cam.width
        self.device = device
        self.prev_pv = view_projection(cam)
        self.prev_gbuf = None
        self.prev_res = None
        self.out_res = torch.zeros(self.h * self.w * RESERVOIR_BYTES, dtype=torch.uint8, device=device)

    def advance(self, gbuf: torch.Tensor, cam: ShadeCamera) -> None:
        self.prev_gbuf = gbuf.contiguous()
        self.prev_res = self.out_res
        self.out_res = torch.zeros_like(self.prev_res)
        self.prev_pv = view_projection(cam)


class ShadeScene:
    """World-space triangles with per-vertex normals and one constant
    material per object; an object whose emission has a component above
    zero is a light (its triangles contiguous).  Device tensors: verts and
    normals (T, 9) or (T, 3, 3) float32, obj (T,) int32, albedo and emissive
    (O, 3), metal_rough (O, 2) float32."""

    def __init__(self, verts: torch.Tensor, normals: torch.Tensor, obj: torch.Tensor, albedo: torch.Tensor,
                 emissive: torch.Tensor, metal_rough: torch.Tensor, stream=None):
        v = verts.reshape(-1, 9).contiguous()
        n = normals.reshape(-1, 9).contiguous()
        _check_dev(v, "verts", torch.float32, 9)
        _check_dev(n, "normals", torch.float32, 9)
        if n.shape[0] != v.shape[0]:
            raise ValueError("normals must match verts")
        o = obj.contiguous()
        _check_dev(o, "obj", torch.int32, None)
        al, em, mr = albedo.contiguous(), emissive.contiguous(), metal_rough.contiguous()
        _check_dev(al, "albedo", torch.float32, 3)
        _check_dev(em, "emissive", torch.float32, 3)
        _check_dev(mr, "metal_rough", torch.float32, 2)
        h = c_void_p()
        check(lib.cp_shade_scene_create(_ptr(v), _ptr(n), _ptr(o), v.shape[0], _ptr(al), _ptr(em), _ptr(mr),
                                        al.shape[0], _stream(stream), byref(h)), "cp_shade_scene_create")
        self._h = h
        self.num_triangles = v.shape[0]
        self.device = v.device

    def set_textures(self, *, texcoords: torch.Tensor | None = None, tangents: torch.Tensor | None = None,
                     textures=(), obj_tex=None, stream=None) -> None:
        """cp_shade_scene_textures: device texcoords (T, 3, 2) and tangents
        (T, 3, 4) float32, a list of RGBA8 sRGB images ((h, w, 4) uint8,
        numpy or tensors; uploaded here) and per object the texture replacing
        its albedo, emission, metal / roughness and its normal map
        ((O, 4) int, -1 none)."""
        tc = None if texcoords is None else texcoords.reshape(-1, 6).contiguous()
        tg = None if tangents is None else tangents.reshape(-1, 12).contiguous()
        if tc is not None:
            _check_dev(tc, "texcoords", torch.float32, 6)
        if tg is not None:
            _check_dev(tg, "tangents", torch.float32, 12)
        ims = [torch.as_tensor(np.ascontiguousarray(np.asarray(im, dtype=np.uint8))) for im in textures]
        for im in ims:
            if im.dim() != 3 or im.shape[2] != 4:
                raise ValueError("each texture must be (h, w, 4) uint8")
        size = np.asarray([[im.shape[1], im.shape[0]] for im in ims], np.int32).reshape(-1, 2)
        texels = (torch.cat([im.reshape(-1) for im in ims]).to(self.device) if ims
                  else torch.zeros(4, dtype=torch.uint8, device=self.device))
        ot = None if obj_tex is None else np.ascontiguousarray(np.asarray(obj_tex, np.int32).reshape(-1, 4))
        check(lib.cp_shade_scene_textures(self._h, _ptr(tc), _ptr(tg), len(ims), c_void_p(size.ctypes.data),
                                          _ptr(texels), None if ot is None else c_void_p(ot.ctypes.data),
                                          _stream(stream)), "cp_shade_scene_textures")

    @property
    def n_lights(self) -> int:
        n = c_int32()
        check(lib.cp_shade_scene_lights(self._h, byref(n)), "cp_shade_scene_lights")
        return n.value

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib.cp_shade_scene_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, cam: ShadeCamera, *, integrator=DIRECT, brdf=BLINN_PHONG, samples=8, max_depth=8,
               use_rr=True, qmc=False, use_metalness=False, frame=0, max_frame=256, new_samples=4,
               temporal_multiplier=16, use_temporal=True, debug_view=0, clear=(0.3, 0.3, 0.3),
               env=(0.0, 0.0, 0.0), seed=1, image: torch.Tensor | None = None, gbuffer: bool = False,
               temporal: TemporalState | None = None, use_normal_map=False, stream=None):
        """One frame; returns the image (height, width, 3) and, with `gbuffer`,
        the first-hit buffer (height, width, 9), as device tensors.  `image`
        is blended into when frame > 0.  `temporal` carries ReSTIR's state
        between frames (its out_res is written)."""
        p = ShadeParams((c_float * 3)(*clear), (c_float * 3)(*env), samples, max_depth, int(qmc), integrator,
                        brdf, int(use_rr), int(use_metalness), frame, max_frame, new_samples,
                        temporal_multiplier, int(use_temporal), debug_view, seed, int(use_normal_map))
        shape = (cam.height, cam.width, 3)
        img = torch.zeros(shape, dtype=torch.float32, device=self.device) if image is None else image
        if tuple(img.shape) != shape or img.dtype != torch.float32 or not img.is_contiguous():
            raise ValueError(f"image must be a contiguous float32 tensor of shape {shape}")
        g = torch.zeros((cam.height, cam.width, 9), dtype=torch.float32, device=self.device) if gbuffer else None
        pv = pg = pr = orr = None
        if temporal is not None:
            pv = temporal.prev_pv
            pg, pr, orr = temporal.prev_gbuf, temporal.prev_res, temporal.out_res
        pv_ptr = c_void_p(pv.ctypes.data) if pv is not None else c_void_p(None)
        check(lib.cp_shade_render(self._h, byref(cam), byref(p), _ptr(img), _ptr(g), pv_ptr, _ptr(pg), _ptr(pr),
                                  _ptr(orr), _stream(stream)), "cp_shade_render")
        return (img, g) if gbuffer else img


def tonemap(img: torch.Tensor, kind: int = EXPONENTIAL, exposure: float = 1.0, gamma: float = 2.2,
            stream=None) -> torch.Tensor:
    """tonemap.frag per colour component (FILMIC, EXPONENTIAL or NO_TONEMAP)."""
    src = img.contiguous()
    if not src.is_cuda or src.dtype != torch.float32:
        raise ValueError("img must be a float32 CUDA tensor")
    out = torch.empty_like(src)
    check(lib.cp_shade_tonemap(kind, exposure, gamma, src.numel(), _ptr(src), _ptr(out), _stream(stream)),
          "cp_shade_tonemap")
    return out
