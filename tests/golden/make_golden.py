"""Generate the golden fixtures under tests/golden/.

Run from the repository root:  python tests/golden/make_golden.py

1. kat_point_triangle.json — hand-computed point-triangle known answers.  The
   expected values below are written out by hand from the geometry (they are
   not computed by the oracle), so they pin the oracle's FP64 routine and the
   GPU kernel independently.
2. ref_meshes.npz — the triangle meshes of the reference's own demo scenes
   media/cube.gltf (12 triangles) and media/mis_test/mis_test.gltf (1,544
   triangles, 7 meshes), read from a checkout of the reference (glTF 2.0:
   POSITION accessors and uint16/uint32 index accessors, mesh space), plus
   seeded queries and their FP64 brute-force answers.  Regenerating needs the
   reference checkout (REFERENCE_ROOT, default /root/reference); the committed
   file is what the tests read.
3. small_sample.npz — FP64 brute-force answers for the first 4,096 queries of
   the small workload (icosphere level 4, queries U[-2,2]^3, seed 0), and the
   exact bytes of its vertex array, as a cross-platform regression anchor.
4. cbox_scene.npz — the reference's media/cbox/cbox.gltf as instances: its 9
   triangle primitives (16,720 triangles, mesh space), one instance per
   (node, primitive) with the node's world matrix (glTF matrix or TRS,
   composed down the node tree, rounded to FP32 3 x 4), seeded queries and
   their FP64 brute-force answers over the world-space vertices (the FP32
   matrix applied to the FP32 vertex in FP64); for shading, each vertex's
   normal and each primitive's material factors (base colour, emission,
   metalness, roughness, glTF defaults where absent).  Needs the reference
   checkout.
"""
from __future__ import annotations

import base64
import json
import os
import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "gpu-rt_gb300"))

R2 = 2.0 ** 0.5

# (a, b, c, q, expected distance, expected closest point, expected barycentrics or None)
KATS = [
    # right triangle in z = 0
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.25, 0.25, 1], 1.0, [0.25, 0.25, 0], [0.5, 0.25, 0.25]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.25, 0.25, -2], 2.0, [0.25, 0.25, 0], [0.5, 0.25, 0.25]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, -1, 0], R2, [0, 0, 0], [1, 0, 0]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [2, -1, 0], R2, [1, 0, 0], [0, 1, 0]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, 2, 0], R2, [0, 1, 0], [0, 0, 1]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, -1, 0], 1.0, [0.5, 0, 0], [0.5, 0.5, 0]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], 0.5 ** 0.5, [0.5, 0.5, 0], [0, 0.5, 0.5]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, 0.5, 3], 10.0 ** 0.5, [0, 0.5, 0], [0.5, 0, 0.5]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 1, 0], 0.0, [0, 1, 0], [0, 0, 1]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.25, 0.5, 0], 0.0, [0.25, 0.5, 0], [0.25, 0.25, 0.5]),
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0], 0.0, [0.5, 0.5, 0], [0, 0.5, 0.5]),
    # obtuse triangle: the foot of the perpendicular lies past the long edge's ends
    ([0, 0, 0], [4, 0, 0], [2, 1, 0], [2, -3, 4], 5.0, [2, 0, 0], [0.5, 0.5, 0]),
    # far from the origin, a distance of exactly 2^-10 (all values exact in FP32)
    ([1000, 1000, 1000], [1001, 1000, 1000], [1000, 1001, 1000], [1000.25, 1000.25, 1000 + 2.0 ** -10],
     2.0 ** -10, [1000.25, 1000.25, 1000], [0.5, 0.25, 0.25]),
    # degenerate triangles: collinear, repeated vertex, single point
    ([0, 0, 0], [1, 0, 0], [2, 0, 0], [1.5, 1, 0], 1.0, [1.5, 0, 0], None),
    ([0, 0, 0], [0, 0, 0], [0, 2, 0], [1, 1, 0], 1.0, [0, 1, 0], None),
    ([1, 1, 1], [1, 1, 1], [1, 1, 1], [1, 1, 3], 2.0, [1, 1, 1], None),
]

# two triangles sharing edge (1,0,0)-(0,1,0); the query sits exactly above the
# shared edge's midpoint, so both are at distance 1: the smaller index wins
TIE_MESH = {
    "verts": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]],
    "tris": [[0, 1, 2], [1, 3, 2]],
    "queries": [[0.5, 0.5, 1.0], [0.5, 0.5, -1.0]],
    "dist": [1.0, 1.0],
    "tri": [0, 0],
}


def write_kats():
    cases = [{"a": a, "b": b, "c": c, "q": q, "dist": d, "point": p, "bary": w}
             for a, b, c, q, d, p, w in KATS]
    with open(HERE / "kat_point_triangle.json", "w") as f:
        json.dump({"cases": cases, "tie_mesh": TIE_MESH}, f, indent=1)


def _gltf_meshes(path: Path, shading: bool = False):
    """Triangle primitives in file order: (positions, triangles), and with
    `shading` also the vertex normals and the material factors the
    reference reads (scene.cpp:286-299) with glTF's defaults: base colour
    1, emission 0, metalness 1, roughness 1."""
    g = json.loads(path.read_text())
    bufs = []
    for b in g["buffers"]:
        uri = b["uri"]
        if uri.startswith("data:"):
            bufs.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            bufs.append((path.parent / uri).read_bytes())

    def accessor(i):
        a = g["accessors"][i]
        bv = g["bufferViews"][a["bufferView"]]
        data = bufs[bv["buffer"]]
        off = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        ncomp = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}[a["type"]]
        fmt = {5126: "f", 5123: "H", 5125: "I", 5121: "B"}[a["componentType"]]
        size = struct.calcsize(fmt)
        stride = bv.get("byteStride", size * ncomp)
        out = np.empty((a["count"], ncomp), dtype=np.float64 if fmt == "f" else np.int64)
        for k in range(a["count"]):
            out[k] = struct.unpack_from("<" + fmt * ncomp, data, off + k * stride)
        return out

    meshes = []
    for m in g["meshes"]:
        for prim in m["primitives"]:
            if prim.get("mode", 4) != 4:
                continue
            pos = accessor(prim["attributes"]["POSITION"]).astype(np.float32)
            idx = accessor(prim["indices"]).reshape(-1, 3).astype(np.int32)
            if not shading:
                meshes.append((pos, idx))
                continue
            nrm = accessor(prim["attributes"]["NORMAL"]).astype(np.float32)
            mat = g["materials"][prim["material"]]
            pbr = mat.get("pbrMetallicRoughness", {})
            albedo = np.float32(pbr.get("baseColorFactor", [1, 1, 1, 1])[:3])
            emissive = np.float32(mat.get("emissiveFactor", [0, 0, 0]))
            mr = np.float32([pbr.get("metallicFactor", 1.0), pbr.get("roughnessFactor", 1.0)])
            meshes.append((pos, idx, nrm, albedo, emissive, mr))
    return meshes


def _gltf_instances(path: Path):
    """One (primitive index, 4 x 4 world matrix) per node primitive, depth-first
    from the default scene's roots; primitives numbered as _gltf_meshes
    returns them (triangle lists in file order)."""
    g = json.loads(path.read_text())
    first, k = [], 0
    for m in g["meshes"]:
        first.append(k)
        k += sum(1 for p in m["primitives"] if p.get("mode", 4) == 4)

    def local(n):
        if "matrix" in n:
            return np.array(n["matrix"], np.float64).reshape(4, 4).T  # column-major
        t = np.array(n.get("translation", [0, 0, 0]), np.float64)
        x, y, z, w = n.get("rotation", [0, 0, 0, 1])
        s = np.array(n.get("scale", [1, 1, 1]), np.float64)
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        M = np.eye(4)
        M[:3, :3] = R * s[None, :]
        M[:3, 3] = t
        return M

    out = []

    def visit(i, parent):
        n = g["nodes"][i]
        W = parent @ local(n)
        if "mesh" in n:
            j = first[n["mesh"]]
            for p in g["meshes"][n["mesh"]]["primitives"]:
                if p.get("mode", 4) == 4:
                    out.append((j, W))
                    j += 1
        for c in n.get("children", []):
            visit(c, W)

    for r in g["scenes"][g.get("scene", 0)]["nodes"]:
        visit(r, np.eye(4))
    return out


def write_cbox_scene(ref_root: Path):
    from oracle import oracle as O

    path = ref_root / "media" / "cbox" / "cbox.gltf"
    meshes = _gltf_meshes(path)
    inst = _gltf_instances(path)
    prim = np.array([j for j, _ in inst], np.int32)
    T = np.stack([W[:3, :4] for _, W in inst]).astype(np.float32)
    wv, wt, off = [], [], 0
    for j, t in zip(prim, T):
        v, tri = meshes[j]
        t64 = t.astype(np.float64)
        wv.append(v.astype(np.float64) @ t64[:, :3].T + t64[:, 3])
        wt.append(tri + off)
        off += len(v)
    wv, wt = np.concatenate(wv), np.concatenate(wt).astype(np.int32)
    rng = np.random.default_rng(11)
    lo, hi = wv.min(0), wv.max(0)
    c, h = 0.5 * (lo + hi), 0.6 * (hi - lo)
    far = c - h + 2 * h * rng.random((4096, 3))
    k = rng.integers(0, len(wt), 2048)
    r1, r2 = np.sqrt(rng.random(2048)), rng.random(2048)
    a, b, cc = (wv[wt[k, j]] for j in range(3))
    near = (1 - r1)[:, None] * a + (r1 * (1 - r2))[:, None] * b + (r1 * r2)[:, None] * cc
    near += rng.normal(0.0, 0.01, near.shape)
    q = np.concatenate([far, near]).astype(np.float32)
    bf = O.brute_f64_dv(wv, wt, q)
    ntri = np.array([len(meshes[j][1]) for j in prim])
    toff_i = np.concatenate([[0], np.cumsum(ntri)])
    inst_of = np.searchsorted(toff_i, bf["tri"], side="right") - 1
    V = np.concatenate([m[0] for m in meshes])
    TT = np.concatenate([m[1] for m in meshes])
    voff = np.concatenate([[0], np.cumsum([len(m[0]) for m in meshes])]).astype(np.int64)
    toff = np.concatenate([[0], np.cumsum([len(m[1]) for m in meshes])]).astype(np.int64)
    shade = _gltf_meshes(path, shading=True)
    np.savez_compressed(HERE / "cbox_scene.npz", verts=V, tris=TT, vert_offsets=voff, tri_offsets=toff,
                        instance_primitive=prim, instance_transform=T, queries=q, dist=bf["dist"],
                        instance=inst_of.astype(np.int32), tri=(bf["tri"] - toff_i[inst_of]).astype(np.int32),
                        normals=np.concatenate([m[2] for m in shade]),
                        prim_albedo=np.stack([m[3] for m in shade]),
                        prim_emissive=np.stack([m[4] for m in shade]),
                        prim_metal_rough=np.stack([m[5] for m in shade]),
                        source=np.array(str(path.relative_to(ref_root))))


def write_ref_meshes(ref_root: Path):
    from oracle import oracle as O

    files = [ref_root / "media" / "cube.gltf", ref_root / "media" / "mis_test" / "mis_test.gltf"]
    meshes = []
    for f in files:
        meshes += _gltf_meshes(f)
    rng = np.random.default_rng(7)
    voff, toff, qoff = [0], [0], [0]
    V, T, Q, D, I = [], [], [], [], []
    for v, t in meshes:
        lo, hi = v.min(0), v.max(0)
        c, h = 0.5 * (lo + hi), 0.75 * (hi - lo) + 1e-3
        q = (c - h + 2 * h * rng.random((512, 3))).astype(np.float32)
        bf = O.brute_f64(v, t, q)
        V.append(v); T.append(t); Q.append(q); D.append(bf["dist"]); I.append(bf["tri"])
        voff.append(voff[-1] + len(v)); toff.append(toff[-1] + len(t)); qoff.append(qoff[-1] + len(q))
    np.savez_compressed(HERE / "ref_meshes.npz", verts=np.concatenate(V), tris=np.concatenate(T),
                        queries=np.concatenate(Q), dist=np.concatenate(D), tri=np.concatenate(I),
                        vert_offsets=np.array(voff, np.int64), tri_offsets=np.array(toff, np.int64),
                        q_offsets=np.array(qoff, np.int64),
                        source=np.array([str(f.relative_to(ref_root)) for f in files]))


def write_small_sample():
    from gpurt_cpq import workloads as W
    from oracle import oracle as O

    v, t, q = W.small()
    q = q[:4096]
    bf = O.brute_f64(v, t, q)
    np.savez_compressed(HERE / "small_sample.npz", verts=v, tris=t, queries=q, dist=bf["dist"],
                        tri=bf["tri"])


if __name__ == "__main__":
    write_kats()
    ref = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))
    if (ref / "media" / "cube.gltf").exists():
        write_ref_meshes(ref)
        write_cbox_scene(ref)
    else:
        print("reference checkout not found; ref_meshes.npz left as committed")
    write_small_sample()
    print("fixtures written to", HERE)
