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


def _gltf_meshes(path: Path):
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
            meshes.append((pos, idx))
    return meshes


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
    else:
        print("reference checkout not found; ref_meshes.npz left as committed")
    write_small_sample()
    print("fixtures written to", HERE)
