"""glTF 2.0 ingest (cp_gltf_*): triangle primitives, their placement, and
for shading their vertex normals, texture coordinates and tangents, material
factors and texture references (images are not decoded).

``load_gltf`` copies what the library read into numpy arrays; ``world_mesh``
flattens the instances into one world-space triangle soup for
:class:`~gpurt_cpq.Mesh`, and the per-primitive arrays feed
:class:`~gpurt_cpq.Batch` (object space) directly.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_int32, c_void_p
from dataclasses import dataclass

import numpy as np

from ._lib import check, lib


@dataclass
class GltfScene:
    verts: np.ndarray          # (V, 3) float32, object space, all primitives
    tris: np.ndarray           # (T, 3) int32, local to each primitive
    vert_offsets: np.ndarray   # (P + 1,) int64
    tri_offsets: np.ndarray    # (P + 1,) int64
    instance_primitive: np.ndarray  # (I,) int32
    instance_world: np.ndarray      # (I, 4, 4) float32, row-major
    normals: np.ndarray        # (V, 3) float32, object space; zero where a primitive has none
    materials: np.ndarray      # (P, 8) float32: base colour rgb, emission rgb, metalness, roughness
    texcoords: np.ndarray | None = None  # (V, 2) float32 TEXCOORD_0, zero where absent
    tangents: np.ndarray | None = None   # (V, 4) float32 TANGENT (xyz, w), zero where absent
    prim_tex: np.ndarray | None = None   # (P, 4) int32 glTF texture of base colour, emission, metal / rough, normal; -1
    tex_image: np.ndarray | None = None  # (textures,) int32 image of each texture, -1 if none
    image_uri: list | None = None        # per image its "uri" ("" if none)
    image_view: np.ndarray | None = None  # (images,) int32 "bufferView" of each image, -1 if none

    def world_mesh(self) -> tuple[np.ndarray, np.ndarray]:
        """All instances in world space as one mesh (vertices, triangles)."""
        vs, ts, base = [], [], 0
        for p, w in zip(self.instance_primitive, self.instance_world):
            v = self.verts[self.vert_offsets[p]:self.vert_offsets[p + 1]].astype(np.float64)
            t = self.tris[self.tri_offsets[p]:self.tri_offsets[p + 1]]
            vs.append((v @ w[:3, :3].T.astype(np.float64) + w[:3, 3]).astype(np.float32))
            ts.append(t + base)
            base += v.shape[0]
        if not vs:
            return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
        return np.concatenate(vs), np.concatenate(ts).astype(np.int32)


    def world_shading(self) -> dict[str, np.ndarray]:
        """All instances in world space for shading, one object per instance
        (as Scene::load adds objects): per triangle its three vertices
        ``verts`` (T, 3, 3), normals ``normals`` (T, 3, 3; the instance's
        inverse-transpose applied, not renormalised), texture coordinates
        ``texcoords`` (T, 3, 2) and tangents ``tangents`` (T, 3, 4; xyz under
        the inverse-transpose as the shader's modelIT, w kept) and its object
        ``obj`` (T,); per object its primitive's ``materials`` (I, 8) and
        glTF texture references ``obj_tex`` (I, 4)."""
        vs, ns, tcs, tgs, obj, mats, otex = [], [], [], [], [], [], []
        for i, (p, w) in enumerate(zip(self.instance_primitive, self.instance_world)):
            lo, hi = self.vert_offsets[p], self.vert_offsets[p + 1]
            t = self.tris[self.tri_offsets[p]:self.tri_offsets[p + 1]]
            m = w[:3, :4].astype(np.float64)
            v = self.verts[lo:hi].astype(np.float64) @ m[:, :3].T + m[:, 3]
            inv = np.linalg.inv(m[:, :3])
            n = self.normals[lo:hi].astype(np.float64) @ inv
            vs.append(v[t])
            ns.append(n[t])
            tc = self.texcoords[lo:hi] if self.texcoords is not None else np.zeros((hi - lo, 2), np.float32)
            tg = self.tangents[lo:hi].astype(np.float64) if self.tangents is not None else np.zeros((hi - lo, 4))
            tg = np.concatenate([tg[:, :3] @ inv, tg[:, 3:]], 1)
            tcs.append(tc[t])
            tgs.append(tg[t])
            obj.append(np.full(len(t), i, np.int32))
            mats.append(self.materials[p])
            otex.append(self.prim_tex[p] if self.prim_tex is not None else np.full(4, -1, np.int32))
        if not vs:
            z = np.zeros((0, 3, 3), np.float32)
            return {"verts": z, "normals": z.copy(), "texcoords": np.zeros((0, 3, 2), np.float32),
                    "tangents": np.zeros((0, 3, 4), np.float32), "obj": np.zeros(0, np.int32),
                    "materials": np.zeros((0, 8), np.float32), "obj_tex": np.zeros((0, 4), np.int32)}
        return {"verts": np.concatenate(vs).astype(np.float32), "normals": np.concatenate(ns).astype(np.float32),
                "texcoords": np.concatenate(tcs).astype(np.float32), "tangents": np.concatenate(tgs).astype(np.float32),
                "obj": np.concatenate(obj), "materials": np.stack(mats).astype(np.float32),
                "obj_tex": np.stack(otex).astype(np.int32)}


def _array(ptr, count, dtype):
    if count == 0:
        return np.zeros(0, dtype)
    ct = np.ctypeslib.as_ctypes_type(dtype)
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape=(count,)).copy()


def load_gltf(path: str) -> GltfScene:
    h = c_void_p()
    check(lib.cp_gltf_load(str(path).encode(), byref(h)), "cp_gltf_load")
    try:
        n = c_int32()
        pv, pt, pvo, pto = c_void_p(), c_void_p(), c_void_p(), c_void_p()
        check(lib.cp_gltf_primitives(h, byref(n), byref(pv), byref(pt), byref(pvo), byref(pto)),
              "cp_gltf_primitives")
        voff = _array(pvo, n.value + 1, np.int64)
        toff = _array(pto, n.value + 1, np.int64)
        verts = _array(pv, int(voff[-1]) * 3, np.float32).reshape(-1, 3)
        tris = _array(pt, int(toff[-1]) * 3, np.int32).reshape(-1, 3)
        ni = c_int32()
        ip, iw = c_void_p(), c_void_p()
        check(lib.cp_gltf_instances(h, byref(ni), byref(ip), byref(iw)), "cp_gltf_instances")
        prim = _array(ip, ni.value, np.int32)
        world = _array(iw, ni.value * 16, np.float32).reshape(-1, 4, 4)
        ns = c_int32()
        pn, pm = c_void_p(), c_void_p()
        check(lib.cp_gltf_shading(h, byref(ns), byref(pn), byref(pm)), "cp_gltf_shading")
        normals = _array(pn, int(voff[-1]) * 3, np.float32).reshape(-1, 3)
        materials = _array(pm, ns.value * 8, np.float32).reshape(-1, 8)
        nt_, ntex, nim = c_int32(), c_int32(), c_int32()
        ptc, ptg, ppt, pti, puri, pview = (c_void_p() for _ in range(6))
        check(lib.cp_gltf_textures(h, byref(nt_), byref(ptc), byref(ptg), byref(ppt), byref(ntex), byref(pti),
                                   byref(nim), byref(puri), byref(pview)), "cp_gltf_textures")
        texcoords = _array(ptc, int(voff[-1]) * 2, np.float32).reshape(-1, 2)
        tangents = _array(ptg, int(voff[-1]) * 4, np.float32).reshape(-1, 4)
        prim_tex = _array(ppt, nt_.value * 4, np.int32).reshape(-1, 4)
        tex_image = _array(pti, ntex.value, np.int32)
        uris = ctypes.cast(puri, ctypes.POINTER(ctypes.c_char_p)) if nim.value else None
        image_uri = [uris[i].decode("utf-8", "replace") for i in range(nim.value)] if uris else []
        image_view = _array(pview, nim.value, np.int32)
        return GltfScene(verts, tris, voff, toff, prim, world, normals, materials, texcoords, tangents, prim_tex,
                         tex_image, image_uri, image_view)
    finally:
        lib.cp_gltf_free(h)
