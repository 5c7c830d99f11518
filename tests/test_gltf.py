"""glTF ingest (cp_gltf_*): the reference's shipped scenes and synthetic files.

The host reader must give the primitives the reference's Scene::parse_mesh
builds (src/scene/scene.cpp:48-315) — checked against the committed fixture
made from the reference's media — and place them as glTF nodes say.
"""
from __future__ import annotations

import base64
import json
import struct
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_reference_scenes_match_fixture(cpq, reference_root):
    REF_MEDIA = reference_root / "media"
    if not (REF_MEDIA / "cube.gltf").exists():
        pytest.skip("reference media not present")
    g = np.load(GOLDEN / "ref_meshes.npz")
    scenes = [cpq.load_gltf(str(REF_MEDIA / "cube.gltf")),
              cpq.load_gltf(str(REF_MEDIA / "mis_test" / "mis_test.gltf"))]
    np.testing.assert_array_equal(np.concatenate([s.verts for s in scenes]), g["verts"])
    np.testing.assert_array_equal(np.concatenate([s.tris for s in scenes]), g["tris"])
    offs = np.concatenate([[0], np.cumsum(np.concatenate([np.diff(s.tri_offsets) for s in scenes]))])
    np.testing.assert_array_equal(offs, g["tri_offsets"])
    assert len(scenes[0].instance_primitive) == 1  # the cube node; light and camera have no mesh


def test_cbox_reader_matches_fixture(cpq, reference_root):
    """The reference's Cornell box: primitives and node instances as the
    fixture's independent Python reader (tests/golden/make_golden.py) made
    them."""
    path = reference_root / "media" / "cbox" / "cbox.gltf"
    if not path.exists():
        pytest.skip("reference media not present")
    g = np.load(GOLDEN / "cbox_scene.npz")
    s = cpq.load_gltf(str(path))
    np.testing.assert_array_equal(s.verts, g["verts"])
    np.testing.assert_array_equal(s.tris, g["tris"])
    np.testing.assert_array_equal(s.vert_offsets, g["vert_offsets"])
    np.testing.assert_array_equal(s.tri_offsets, g["tri_offsets"])
    np.testing.assert_array_equal(s.instance_primitive, g["instance_primitive"])
    np.testing.assert_array_equal(s.instance_world[:, :3, :].astype(np.float32), g["instance_transform"])
    # shading inputs: normals, and the material factors with glTF's defaults
    np.testing.assert_array_equal(s.normals, g["normals"])
    np.testing.assert_array_equal(s.materials[:, 0:3], g["prim_albedo"])
    np.testing.assert_array_equal(s.materials[:, 3:6], g["prim_emissive"])
    np.testing.assert_array_equal(s.materials[:, 6:8], g["prim_metal_rough"])


def _write(tmp: Path, doc: dict, bin_data: bytes, mode: str) -> Path:
    """mode: "data" (base64 URI), "file" (external .bin) or "glb"."""
    doc = json.loads(json.dumps(doc))
    doc["asset"] = {"version": "2.0"}
    if mode == "glb":
        doc["buffers"] = [{"byteLength": len(bin_data)}]
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        bd = bin_data + b"\0" * (-len(bin_data) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bd), 0x004E4942) + bd
        p = tmp / "scene.glb"
        p.write_bytes(struct.pack("<4sII", b"glTF", 2, 12 + len(body)) + body)
        return p
    if mode == "data":
        uri = "data:application/octet-stream;base64," + base64.b64encode(bin_data).decode()
    else:
        (tmp / "my data.bin").write_bytes(bin_data)
        uri = "my%20data.bin"
    doc["buffers"] = [{"byteLength": len(bin_data), "uri": uri}]
    p = tmp / "scene.gltf"
    p.write_text(json.dumps(doc))
    return p


def _scene():
    """A quad as TRIANGLES (uint16), a strip (uint8), a fan (uint32) and an
    unindexed triangle with interleaved 24-byte vertices; two nodes place the
    quad mesh (TRS, and a matrix child), one places the others."""
    quad = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    qidx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    strip = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1], [0, 2, 1]], np.float32)
    sidx = np.array([0, 1, 2, 3, 4], np.uint8)
    fan = np.array([[0, 0, 2], [1, 0, 2], [1, 1, 2], [0, 1, 2]], np.float32)
    fidx = np.array([0, 1, 2, 3], np.uint32)
    inter = np.zeros((3, 6), np.float32)
    inter[:, :3] = [[5, 5, 5], [6, 5, 5], [5, 6, 5]]
    inter[:, 3:] = 9.0  # another attribute interleaved
    chunks, views = [], []

    def add(arr, stride=None):
        off = sum(len(c) for c in chunks)
        b = arr.tobytes()
        chunks.append(b + b"\0" * (-len(b) % 4))
        v = {"buffer": 0, "byteOffset": off, "byteLength": len(b)}
        if stride:
            v["byteStride"] = stride
        views.append(v)
        return len(views) - 1

    acc = []

    def accessor(view, ctype, count, typ, off=0):
        acc.append({"bufferView": view, "componentType": ctype, "count": count, "type": typ,
                    "byteOffset": off})
        return len(acc) - 1

    a_q = accessor(add(quad), 5126, 4, "VEC3")
    a_qi = accessor(add(qidx), 5123, 6, "SCALAR")
    a_s = accessor(add(strip), 5126, 5, "VEC3")
    a_si = accessor(add(sidx), 5121, 5, "SCALAR")
    a_f = accessor(add(fan), 5126, 4, "VEC3")
    a_fi = accessor(add(fidx), 5125, 4, "SCALAR")
    a_i = accessor(add(inter, stride=24), 5126, 3, "VEC3")
    doc = {
        "scene": 0,
        "scenes": [{"nodes": [0, 2]}],
        "nodes": [
            {"mesh": 0, "translation": [10, 0, 0], "rotation": [0, 0, 0.7071067811865476, 0.7071067811865476],
             "scale": [2, 2, 2], "children": [1]},
            {"mesh": 0, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 3, 1]},
            {"mesh": 1},
        ],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": a_q}, "indices": a_qi}]},
            {"primitives": [{"attributes": {"POSITION": a_s}, "indices": a_si, "mode": 5},
                            {"attributes": {"POSITION": a_f}, "indices": a_fi, "mode": 6},
                            {"attributes": {"POSITION": a_q}, "indices": a_qi, "mode": 1},  # lines: skipped
                            {"attributes": {"POSITION": a_i}}]},
        ],
        "accessors": acc,
        "bufferViews": views,
    }
    return doc, b"".join(chunks)


@pytest.mark.parametrize("mode", ["data", "file", "glb"])
def test_synthetic_scene(cpq, tmp_path, mode):
    doc, data = _scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, mode)))
    np.testing.assert_array_equal(s.vert_offsets, [0, 4, 9, 13, 16])
    np.testing.assert_array_equal(s.tri_offsets, [0, 2, 5, 7, 8])
    np.testing.assert_array_equal(s.tris[:2], [[0, 1, 2], [0, 2, 3]])
    np.testing.assert_array_equal(s.tris[2:5], [[0, 1, 2], [1, 2, 3], [2, 3, 4]])  # strip
    np.testing.assert_array_equal(s.tris[5:7], [[0, 1, 2], [0, 2, 3]])             # fan
    np.testing.assert_array_equal(s.tris[7], [0, 1, 2])                            # unindexed
    np.testing.assert_array_equal(s.verts[13:16], [[5, 5, 5], [6, 5, 5], [5, 6, 5]])  # stride 24
    # instances: node 0 (quad), its child node 1 (quad), node 2 (3 primitives)
    np.testing.assert_array_equal(s.instance_primitive, [0, 0, 1, 2, 3])
    rz = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64)
    w0 = np.eye(4)
    w0[:3, :3] = rz * 2
    w0[:3, 3] = [10, 0, 0]
    w1 = w0 @ np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 3], [0, 0, 0, 1]], np.float64)
    np.testing.assert_allclose(s.instance_world[0], w0, atol=1e-6)
    np.testing.assert_allclose(s.instance_world[1], w1, atol=1e-6)
    np.testing.assert_allclose(s.instance_world[2], np.eye(4), atol=0)
    v, t = s.world_mesh()
    assert v.shape == (4 + 4 + 5 + 4 + 3, 3) and t.shape == (2 + 2 + 3 + 2 + 1, 3)
    np.testing.assert_allclose(v[1], [10, 2, 0], atol=1e-5)       # (1,0,0) rotated, scaled, moved
    np.testing.assert_allclose(v[4 + 1], [10, 2, 6], atol=1e-5)   # child: z + 3 before the parent's scale


def _append(doc, data, arr, ctype, typ):
    """Append an accessor over `arr` to a document from _scene()."""
    b = arr.tobytes()
    doc["bufferViews"].append({"buffer": 0, "byteOffset": len(data), "byteLength": len(b)})
    doc["accessors"].append({"bufferView": len(doc["bufferViews"]) - 1, "componentType": ctype,
                             "count": len(arr), "type": typ})
    return len(doc["accessors"]) - 1, data + b + b"\0" * (-len(b) % 4)


def _shading_scene():
    doc, data = _scene()
    qn = np.float32([[0, 0, 1], [0, 0.6, 0.8], [0, 0, -1], [1, 0, 0]])
    a_qn, data = _append(doc, data, qn, 5126, "VEC3")
    a_fn, data = _append(doc, data, qn[:2], 5126, "VEC3")  # fewer normals than the fan's 4 vertices
    doc["meshes"][0]["primitives"][0]["attributes"]["NORMAL"] = a_qn
    doc["meshes"][0]["primitives"][0]["material"] = 0
    doc["meshes"][1]["primitives"][0]["material"] = 1
    doc["meshes"][1]["primitives"][1]["attributes"]["NORMAL"] = a_fn
    doc["meshes"][1]["primitives"][3]["material"] = 0
    doc["materials"] = [{"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.25, 0.125, 1.0], "metallicFactor": 0.0,
                                                  "roughnessFactor": 0.3},
                         "emissiveFactor": [1.0, 2.0, 3.0]},
                        {"pbrMetallicRoughness": {"roughnessFactor": 0.7}}]
    return doc, data, qn


@pytest.mark.parametrize("mode", ["data", "file", "glb"])
def test_shading_inputs(cpq, tmp_path, mode):
    """Vertex normals (zero past the NORMAL accessor's count, or without one)
    and material factors with glTF's defaults, as parse_mesh reads them."""
    doc, data, qn = _shading_scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, mode)))
    assert s.normals.shape == s.verts.shape
    np.testing.assert_array_equal(s.normals[0:4], qn)                    # quad
    np.testing.assert_array_equal(s.normals[4:9], np.zeros((5, 3)))      # strip: no NORMAL
    np.testing.assert_array_equal(s.normals[9:11], qn[:2])               # fan: two normals,
    np.testing.assert_array_equal(s.normals[11:13], np.zeros((2, 3)))    # then zeros
    np.testing.assert_array_equal(s.normals[13:16], np.zeros((3, 3)))
    mat0 = [0.5, 0.25, 0.125, 1.0, 2.0, 3.0, 0.0, 0.3]
    np.testing.assert_array_equal(s.materials, np.float32([
        mat0,
        [1, 1, 1, 0, 0, 0, 1, 0.7],   # strip: material 1, defaults but its roughness
        [1, 1, 1, 0, 0, 0, 1, 1],     # fan: no material
        mat0,                         # unindexed triangle: material 0
    ]))


def test_shading_input_errors(cpq, tmp_path):
    from gpurt_cpq._lib import CpError

    for change, msg in (
        (lambda d: d["meshes"][0]["primitives"][0].__setitem__("material", 5), "material index out of range"),
        (lambda d: d["materials"][0]["pbrMetallicRoughness"].__setitem__("baseColorFactor", "red"), "not an array"),
        (lambda d: d["materials"][0].__setitem__("emissiveFactor", [1, "x", 3]), "non-number"),
        (lambda d: d["accessors"][d["meshes"][0]["primitives"][0]["attributes"]["NORMAL"]].__setitem__(
            "type", "VEC2"), "NORMAL must be FLOAT VEC3"),
    ):
        doc, data, _ = _shading_scene()
        change(doc)
        with pytest.raises(CpError, match=msg):
            cpq.load_gltf(str(_write(tmp_path, doc, data, "data")))


def _texture_scene():
    doc, data, qn = _shading_scene()
    tc = np.float32([[0, 0], [1, 0], [1, 1], [0, 1]])
    tg = np.float32([[1, 0, 0, 1], [1, 0, 0, 1], [1, 0, 0, -1], [0, 1, 0, 1]])
    a_tc, data = _append(doc, data, tc, 5126, "VEC2")
    a_tc_short, data = _append(doc, data, tc[:3], 5126, "VEC2")  # fewer than the fan's vertices
    a_tc_u16, data = _append(doc, data, np.uint16([[0, 0], [65535, 0], [65535, 65535], [0, 65535]]), 5123, "VEC2")
    a_tg, data = _append(doc, data, tg, 5126, "VEC4")
    prims = doc["meshes"]
    prims[0]["primitives"][0]["attributes"].update(TEXCOORD_0=a_tc, TANGENT=a_tg)
    prims[1]["primitives"][1]["attributes"]["TEXCOORD_0"] = a_tc_short
    prims[1]["primitives"][0]["attributes"]["TEXCOORD_0"] = a_tc_u16  # normalised shorts: not read
    doc["materials"][0]["pbrMetallicRoughness"].update(baseColorTexture={"index": 1},
                                                       metallicRoughnessTexture={"index": 2})
    doc["materials"][0]["emissiveTexture"] = {"index": 0}
    doc["materials"][0]["normalTexture"] = {"index": 1, "scale": 1.0}
    doc["materials"][1]["normalTexture"] = {"index": 2}
    doc["textures"] = [{"source": 0}, {"source": 1, "sampler": 0}, {"source": 7}]
    doc["images"] = [{"uri": "albedo.jpg"}, {"bufferView": 0, "mimeType": "image/png"}]
    return doc, data, tc, tg


@pytest.mark.parametrize("mode", ["data", "glb"])
def test_texture_inputs(cpq, tmp_path, mode):
    """TEXCOORD_0 and TANGENT paired with the vertices as the normals are
    (zero past the accessor's count, without one, or when not FLOAT VEC2 /
    VEC4, as parse_mesh skips the types it does not read), each primitive's
    texture references, each texture's image and each image's uri or view."""
    doc, data, tc, tg = _texture_scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, mode)))
    assert s.texcoords.shape == (s.verts.shape[0], 2) and s.tangents.shape == (s.verts.shape[0], 4)
    np.testing.assert_array_equal(s.texcoords[0:4], tc)
    np.testing.assert_array_equal(s.tangents[0:4], tg)
    np.testing.assert_array_equal(s.texcoords[4:9], np.zeros((5, 2)))   # strip: unsigned shorts, not read
    np.testing.assert_array_equal(s.texcoords[9:12], tc[:3])            # fan: three, then zero
    np.testing.assert_array_equal(s.texcoords[12:], np.zeros((s.verts.shape[0] - 12, 2)))
    np.testing.assert_array_equal(s.tangents[4:], np.zeros((s.verts.shape[0] - 4, 4)))
    np.testing.assert_array_equal(s.prim_tex, np.int32([[1, 0, 2, 1], [-1, -1, -1, 2], [-1, -1, -1, -1],
                                                        [1, 0, 2, 1]]))
    np.testing.assert_array_equal(s.tex_image, [0, 1, -1])
    assert s.image_uri == ["albedo.jpg", ""]
    np.testing.assert_array_equal(s.image_view, [-1, 0])
    # world space: texture coordinates per triangle corner, tangents under the
    # instance's inverse-transpose with w kept, the texture references per object
    w = s.world_shading()
    T = w["verts"].shape[0]
    assert w["texcoords"].shape == (T, 3, 2) and w["tangents"].shape == (T, 3, 4)
    assert w["obj_tex"].shape == (len(s.instance_primitive), 4)
    i0 = int(np.nonzero(s.instance_primitive == 0)[0][0])
    m = s.instance_world[i0][:3, :3].astype(np.float64)
    t0 = s.tris[s.tri_offsets[0]:s.tri_offsets[1]]
    first = int(np.nonzero(w["obj"] == i0)[0][0])
    want = np.concatenate([tg[t0[0], :3] @ np.linalg.inv(m), tg[t0[0], 3:]], 1)
    np.testing.assert_allclose(w["tangents"][first], want, rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(w["texcoords"][first], tc[t0[0]])
    np.testing.assert_array_equal(w["obj_tex"][i0], s.prim_tex[0])


def test_texture_input_errors(cpq, tmp_path):
    from gpurt_cpq._lib import CpError

    for change, msg in (
        (lambda d: d["materials"][0]["pbrMetallicRoughness"].__setitem__("baseColorTexture", {"index": 3}),
         "baseColorTexture index out of range"),
        (lambda d: d["materials"][1].__setitem__("normalTexture", {"index": -2}), "normalTexture index out of range"),
        (lambda d: d["accessors"][d["meshes"][0]["primitives"][0]["attributes"]["TANGENT"]].__setitem__(
            "count", 999), "past the end"),
    ):
        doc, data, _, _ = _texture_scene()
        change(doc)
        with pytest.raises(CpError, match=msg):
            cpq.load_gltf(str(_write(tmp_path, doc, data, "data")))


def test_errors_are_reported(cpq, tmp_path):
    from gpurt_cpq._lib import CP_ERROR_INVALID_VALUE, CpError

    with pytest.raises(CpError) as e:
        cpq.load_gltf(str(tmp_path / "missing.gltf"))
    assert e.value.status == CP_ERROR_INVALID_VALUE and "cannot open" in str(e.value)
    (tmp_path / "bad.gltf").write_text('{"meshes": [}')
    with pytest.raises(CpError, match="JSON"):
        cpq.load_gltf(str(tmp_path / "bad.gltf"))
    doc, data = _scene()
    doc["accessors"][1]["count"] = 1000  # past its bufferView
    with pytest.raises(CpError, match="past the end"):
        cpq.load_gltf(str(_write(tmp_path, doc, data, "data")))
    doc, data = _scene()
    doc["accessors"][0]["count"] = 2  # indices now reach past the vertices
    with pytest.raises(CpError, match="past 2 vertices"):
        cpq.load_gltf(str(_write(tmp_path, doc, data, "file")))


@pytest.mark.gpu
def test_gltf_scene_queries(orc, cpq, cuda, tmp_path):
    """A loaded scene, flattened to world space, through cp_mesh_create and
    cp_query, checked in FP64."""
    import torch

    doc, data = _scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, "glb")))
    v, t = s.world_mesh()
    m = cpq.Mesh(torch.from_numpy(v).to(cuda), torch.from_numpy(t).to(cuda), branching=4)
    q = np.random.default_rng(3).uniform(-2, 12, (5000, 3)).astype(np.float32)
    r = m.query(torch.from_numpy(q).to(cuda))
    ref = orc.brute_f64(v, t, q)
    d = r.dist.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(d - ref["dist"]) / np.maximum(ref["dist"], 1e-30)) <= 1e-6


@pytest.mark.gpu
def test_gltf_textured_render(cpq, cuda, tmp_path):
    """A textured glTF scene through the path: read, flattened to world space,
    rendered by the path tracer with textures (the file's images stood in for
    by synthetic RGBA8 images in glTF texture order) and normal maps, equal
    pixel for pixel to the restatement."""
    import torch

    from gpurt_cpq import shading as G

    from oracle import shade as S

    doc, data, _, _ = _texture_scene()
    s = cpq.load_gltf(str(_write(tmp_path, doc, data, "glb")))
    w = s.world_shading()
    rng = np.random.default_rng(4)
    images = [rng.integers(0, 256, (3 + k, 4 + 2 * k, 4), dtype=np.uint8) for k in range(len(s.tex_image))]
    mats = w["materials"]
    sc = S.Scene(w["verts"], w["normals"], w["obj"], mats[:, 0:3], mats[:, 3:6], mats[:, 6:8],
                 texcoords=w["texcoords"], tangents=w["tangents"], textures=images, obj_tex=w["obj_tex"])

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)

    gs = G.ShadeScene(d(w["verts"]), d(w["normals"]), d(w["obj"]), d(mats[:, 0:3]), d(mats[:, 3:6]),
                      d(mats[:, 6:8]))
    gs.set_textures(texcoords=d(w["texcoords"]), tangents=d(w["tangents"]), textures=images, obj_tex=w["obj_tex"])
    lo, hi = w["verts"].reshape(-1, 3).min(0), w["verts"].reshape(-1, 3).max(0)
    c = (lo + hi) / 2
    cam = S.camera(eye=tuple(c + np.float32([0.0, 0.0, 1.6]) * float((hi - lo).max())), target=tuple(c),
                   up=(0, 1, 0), yfov=0.9, width=24, height=18)
    for integrator in (S.DIRECT, S.MIS, S.RESTIR):
        want = sc.render(cam, integrator=integrator, samples=4, seed=5, use_normal_map=True)
        got = gs.render(G.ShadeCamera.from_buffer_copy(cam), integrator=integrator, samples=4, seed=5,
                        use_normal_map=True).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), integrator
        assert want.max() > 0.0


def test_malformed_files_never_crash(cpq, tmp_path):
    """Seeded mutations of valid .gltf and .glb files — truncation, byte
    flips, numbers in the JSON replaced by huge, negative or fractional
    values — load cleanly or raise CpError; the process never crashes and no
    index reaches past its vertices."""
    import re

    from gpurt_cpq._lib import CpError

    rng = np.random.default_rng(2024)
    doc, data = _scene()
    gl = _write(tmp_path, doc, data, "data").read_bytes()
    glb = _write(tmp_path, doc, data, "glb").read_bytes()
    numbers = [m.start() for m in re.finditer(rb"\d+", gl)]
    outcomes = {"ok": 0, "error": 0}
    for k in range(400):
        src, ext = (gl, ".gltf") if k % 2 == 0 else (glb, ".glb")
        b = bytearray(src)
        kind = k % 5
        if kind == 0:
            b = b[: int(rng.integers(1, len(b)))]
        elif kind == 1:
            for _ in range(int(rng.integers(1, 8))):
                b[int(rng.integers(0, len(b)))] ^= 1 << int(rng.integers(0, 8))
        elif kind == 2 and ext == ".gltf":
            at = numbers[int(rng.integers(0, len(numbers)))]
            end = at
            while end < len(b) and chr(b[end]).isdigit():
                end += 1
            b[at:end] = [b"4294967295", b"-1", b"99999999999999999999", b"0.5", b"1e300"][int(rng.integers(0, 5))]
        elif kind == 3 and ext == ".glb":
            # damage the chunk headers (lengths and types)
            for off in (12, 16, 20 + int.from_bytes(src[12:16], "little")):
                if off + 4 <= len(b):
                    b[off:off + 4] = int(rng.integers(0, 2**32)).to_bytes(4, "little")
        else:
            cut = int(rng.integers(0, len(b)))
            b = b[:cut] + b[cut + int(rng.integers(1, 64)):]
        f = tmp_path / f"m{k}{ext}"
        f.write_bytes(bytes(b))
        try:
            s = cpq.load_gltf(str(f))
        except CpError:
            outcomes["error"] += 1
            continue
        outcomes["ok"] += 1
        nv = np.diff(s.vert_offsets)
        for p in range(len(nv)):
            t = s.tris[s.tri_offsets[p]:s.tri_offsets[p + 1]]
            assert t.size == 0 or (t.min() >= 0 and t.max() < nv[p])
        assert np.all(s.instance_primitive >= 0) and np.all(s.instance_primitive < len(nv))
    assert outcomes["error"] > 0 and outcomes["ok"] > 0
