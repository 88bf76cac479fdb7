"""glTF scene input (solrt_gltf_*, the counterpart of scene::load_scene,
src/scene/mod.rs:138-295). Host-side parsing only, no GPU: round trips of
scenes written by scenes.write_gltf in every container form, node
hierarchies (matrix and translation-rotation-scale, first match in node
order as calc_mesh_global_transform, src/scene/mod.rs:106-136), vertex and
material defaults, error reporting, and the reference's own cornell.gltf /
tunnel.gltf (when the reference tree is present) against an independent
numpy reading of the same files."""
import base64
import json
import os
import struct

import numpy as np
import pytest

from helpers import S, reference_path

REF_MODELS = reference_path("assets", "models")


def _arrays_equal(a, b):
    assert np.array_equal(a.vertices.view(np.uint8), b.vertices.view(np.uint8))
    assert np.array_equal(a.indices, b.indices)
    assert np.array_equal(a.sections, b.sections)
    assert np.array_equal(a.materials.view(np.uint8), b.materials.view(np.uint8))


def _with_uv(d):
    d.vertices["uv"][:, 0] = np.linspace(0, 1, len(d.vertices), dtype=np.float32)
    d.vertices["uv"][:, 1] = np.linspace(1, 0, len(d.vertices), dtype=np.float32)
    d.vertices["color"][:, 3] = 0.5
    return d


@pytest.mark.parametrize("form", ["base64", "external", "glb", "u16"])
def test_round_trip(solrt, tmp_path, form):
    d = _with_uv(S.cornell())
    path = tmp_path / ("scene.glb" if form == "glb" else "scene.gltf")
    S.write_gltf(d, str(path), external_bin=form == "external", index_type="u16" if form == "u16" else "u32")
    g = solrt.load_scene(str(path))
    _arrays_equal(g.data, d)
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    assert (g.data.instances["transform"] == eye).all() and (g.data.instances["transform_it"] == eye).all()
    assert np.array_equal(g.data.instances["id"], np.arange(len(d.sections)))
    assert g.camera(1.0) is None
    g.close()


def test_camera_from_view(solrt, tmp_path):
    """The camera node's matrix is the view matrix as is; yfov is passed to a
    degrees-based perspective (Camera::from_view + update_persp)."""
    d = S.cornell()
    view = np.array(solrt.camera_look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, -1, 0), 40.0, 1.0).view)
    S.write_gltf(d, str(tmp_path / "c.gltf"), view=view, yfov=40.0, znear=0.1, zfar=1000.0)
    g = solrt.load_scene(str(tmp_path / "c.gltf"))
    c = g.camera(1.0)
    ref = solrt.camera_look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, -1, 0), 40.0, 1.0)
    for f in ("view", "view_inverse", "projection", "projection_inverse"):
        assert np.array_equal(np.array(getattr(c, f)), np.array(getattr(ref, f))), f


def _quat(axis, deg):
    axis = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    h = np.radians(deg) / 2
    return [*(axis * np.sin(h)), np.cos(h)]


def _trs(t=(0, 0, 0), q=(0, 0, 0, 1), s=(1, 1, 1)):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(s)[None, :]
    M[:3, 3] = t
    return M


def _triangle_doc(nodes, extra_mesh_nodes=()):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], "<f4")
    blob = pos.tobytes()
    doc = {"asset": {"version": "2.0"}, "nodes": nodes,
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
           "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"}],
           "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": len(blob)}],
           "buffers": [{"byteLength": len(blob),
                        "uri": "data:application/octet-stream;base64," + base64.b64encode(blob).decode()}]}
    return doc


def test_node_hierarchy_trs(solrt, tmp_path):
    """Global transform = product of the matrices on the path from the first
    node (in node order) whose subtree holds the mesh; later nodes holding the
    same mesh are ignored."""
    t0, q1, s2 = (0.5, -1.0, 2.0), _quat((1, 2, 3), 37.0), (2.0, 0.5, 1.5)
    m3 = _trs((9, 9, 9))
    nodes = [{"name": "unrelated", "translation": [5, 5, 5]},
             {"children": [2], "translation": list(t0)},
             {"children": [3], "rotation": list(q1)},
             {"mesh": 0, "scale": list(s2)},
             {"mesh": 0, "matrix": list(m3.T.reshape(-1))}]
    p = tmp_path / "h.gltf"
    p.write_text(json.dumps(_triangle_doc(nodes)))
    g = solrt.load_scene(str(p))
    M = _trs(t=t0) @ _trs(q=q1) @ _trs(s=s2)
    got = g.data.instances["transform"][0].reshape(4, 4).T.astype(np.float64)
    assert np.allclose(got, M, rtol=0, atol=1e-6)
    assert np.array_equal(g.data.instances["transform"][0], M.T.reshape(-1).astype(np.float32))
    git = g.data.instances["transform_it"][0].reshape(4, 4).T.astype(np.float64)
    assert np.allclose(git, np.linalg.inv(M).T, rtol=0, atol=1e-6)


def test_vertex_and_material_defaults(solrt, tmp_path):
    """No NORMAL / COLOR_0 / TEXCOORD_0: normal (0,1,0,1), colour (1,1,1,1),
    uv 0 (src/scene/mod.rs:182-193); no indices: consecutive triangles; no
    material: a default material (factors 1, emissive 0) is appended."""
    p = tmp_path / "d.gltf"
    p.write_text(json.dumps(_triangle_doc([{"mesh": 0}])))
    g = solrt.load_scene(str(p))
    v = g.data.vertices
    assert (v["normal"] == np.array([0, 1, 0, 1], np.float32)).all()
    assert (v["color"] == 1.0).all() and (v["uv"] == 0.0).all() and (v["pos"][:, 3] == 1.0).all()
    assert list(g.data.indices) == [0, 1, 2]
    assert len(g.data.materials) == 1 and g.data.sections["material_index"][0] == 0
    m = g.data.materials[0]
    assert (m["base_color"] == 1).all() and m["metallic"] == 1 and m["roughness"] == 1 and (m["emissive"] == 0).all()


def test_normalized_u8_colors(solrt, tmp_path):
    doc = _triangle_doc([{"mesh": 0}])
    pos = base64.b64decode(doc["buffers"][0]["uri"].split(",")[1])
    col = bytes([255, 0, 51, 255, 0, 255, 102, 128, 10, 20, 30, 40])
    blob = pos + col
    doc["bufferViews"].append({"buffer": 0, "byteOffset": len(pos), "byteLength": len(col)})
    doc["accessors"].append({"bufferView": 1, "componentType": 5121, "normalized": True, "count": 3,
                             "type": "VEC4"})
    doc["meshes"][0]["primitives"][0]["attributes"]["COLOR_0"] = 1
    doc["buffers"] = [{"byteLength": len(blob),
                       "uri": "data:application/octet-stream;base64," + base64.b64encode(blob).decode()}]
    p = tmp_path / "c.gltf"
    p.write_text(json.dumps(doc))
    g = solrt.load_scene(str(p))
    want = (np.frombuffer(col, np.uint8).reshape(3, 4) / 255.0).astype(np.float32)
    assert np.array_equal(g.data.vertices["color"], want)


def test_errors(solrt, tmp_path):
    with pytest.raises(solrt.SolrtError):
        solrt.load_scene(str(tmp_path / "missing.gltf"))
    bad = tmp_path / "bad.gltf"
    bad.write_text("{\"asset\": {\"version\": \"2.0\"}, \"nodes\": [")
    with pytest.raises(solrt.SolrtError, match="malformed"):
        solrt.load_scene(str(bad))
    doc = _triangle_doc([{"mesh": 0}])
    doc["accessors"][0]["count"] = 4                      # reads past the buffer view
    over = tmp_path / "over.gltf"
    over.write_text(json.dumps(doc))
    with pytest.raises(solrt.SolrtError, match="past"):
        solrt.load_scene(str(over))
    doc = _triangle_doc([{"mesh": 0}])
    doc["meshes"][0]["primitives"][0]["mode"] = 1         # lines
    lines = tmp_path / "lines.gltf"
    lines.write_text(json.dumps(doc))
    with pytest.raises(solrt.SolrtError, match="triangle"):
        solrt.load_scene(str(lines))


# ---------------------------------------------------------------------------
# the reference's own models, read independently with numpy
# ---------------------------------------------------------------------------

def _np_read(path):
    doc = json.load(open(path))
    bufs = []
    for b in doc["buffers"]:
        u = b["uri"]
        bufs.append(base64.b64decode(u.split(",", 1)[1]) if u.startswith("data:")
                    else open(os.path.join(os.path.dirname(path), u), "rb").read())
    ncomp = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}
    ctype = {5126: "<f4", 5123: "<u2", 5125: "<u4", 5121: "u1"}

    def acc(i):
        a = doc["accessors"][i]
        bv = doc["bufferViews"][a["bufferView"]]
        dt = np.dtype(ctype[a["componentType"]])
        n = ncomp[a["type"]]
        off = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = bv.get("byteStride", dt.itemsize * n)
        raw = np.frombuffer(bufs[bv["buffer"]], np.uint8)
        rows = [np.frombuffer(raw[off + k * stride: off + k * stride + dt.itemsize * n].tobytes(), dt)
                for k in range(a["count"])]
        return np.array(rows).reshape(a["count"], n)
    return doc, acc


@pytest.mark.parametrize("name", ["cornell.gltf", "tunnel.gltf"])
def test_reference_models(solrt, name):
    path = os.path.join(REF_MODELS, name)
    if not os.path.exists(path):
        pytest.skip("reference models not present")
    doc, acc = _np_read(path)
    g = solrt.load_scene(path)
    d = g.data
    k = 0
    for mi, mesh in enumerate(doc["meshes"]):
        for prim in mesh["primitives"]:
            s = d.sections[k]
            pos = acc(prim["attributes"]["POSITION"])
            v = d.vertices[s["vertex_offset"]:s["vertex_offset"] + s["vertex_count"]]
            assert np.array_equal(v["pos"][:, :3], pos.astype(np.float32))
            if "NORMAL" in prim["attributes"]:
                assert np.array_equal(v["normal"][:, :3], acc(prim["attributes"]["NORMAL"]).astype(np.float32))
            if "COLOR_0" in prim["attributes"]:
                c = acc(prim["attributes"]["COLOR_0"])
                c = c / {np.dtype("u1"): 255.0, np.dtype("<u2"): 65535.0}.get(c.dtype, 1.0)
                assert np.allclose(v["color"][:, :c.shape[1]], c, rtol=0, atol=1e-7)
            idx = acc(prim["indices"]).reshape(-1)
            assert np.array_equal(d.indices[s["index_offset"]:s["index_offset"] + s["index_count"]], idx)
            assert s["material_index"] == prim["material"]
            k += 1
    assert k == len(d.sections)
    for m, gm in zip(d.materials, doc["materials"]):
        pbr = gm.get("pbrMetallicRoughness", {})
        assert np.array_equal(m["base_color"], np.float32(pbr.get("baseColorFactor", [1, 1, 1, 1])))
        assert m["metallic"] == np.float32(pbr.get("metallicFactor", 1.0))
        assert m["roughness"] == np.float32(pbr.get("roughnessFactor", 1.0))
        assert np.array_equal(m["emissive"], np.float32(gm.get("emissiveFactor", [0, 0, 0])))
    cam_node = next(n for n in doc["nodes"] if "camera" in n)
    c = g.camera(16 / 9)
    assert np.array_equal(np.array(c.view), np.float32(cam_node["matrix"]))
    yfov = doc["cameras"][0]["perspective"]["yfov"]
    ref = solrt.camera_from_view(cam_node["matrix"], yfov, 16 / 9, doc["cameras"][0]["perspective"]["znear"],
                                 doc["cameras"][0]["perspective"].get("zfar", 100.0))
    assert np.array_equal(np.array(c.projection), np.array(ref.projection))
    if name == "cornell.gltf":
        assert d.tri_count == 32 and len(d.materials) == 8


def _png16(path, px16, filters):
    """Writes a 16-bit RGBA PNG with the given per-row filter types."""
    import zlib
    h, w, _ = px16.shape
    raw = px16.astype(">u2").tobytes()
    stride = w * 8
    rows = []
    prev = bytes(stride)
    for y in range(h):
        line = raw[y * stride:(y + 1) * stride]
        f = filters[y % len(filters)]
        out = bytearray(stride)
        for x in range(stride):
            a = line[x - 8] if x >= 8 else 0
            b = prev[x]
            c = prev[x - 8] if x >= 8 else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[x] = (line[x] - pred) & 0xFF
        rows.append(bytes([f]) + bytes(out))
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 16, 6, 0, 0, 0)) +
                 chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


def test_read_png_8_and_16_bit(solrt, tmp_path):
    io = solrt.imageio
    x = np.random.default_rng(4).integers(0, 256, (9, 11, 4), dtype=np.uint8)
    io.write_png(str(tmp_path / "a.png"), x)
    assert np.array_equal(io.read_png(str(tmp_path / "a.png")), x)
    px = np.random.default_rng(5).integers(0, 65536, (7, 5, 4), dtype=np.uint32)
    _png16(str(tmp_path / "b.png"), px, filters=[0, 1, 2, 3, 4])
    want = ((px + 128) // 257).astype(np.uint8)
    assert np.array_equal(io.read_png(str(tmp_path / "b.png")), want)


def test_reference_blue_noise_texture(solrt):
    path = reference_path("assets", "textures", "HDR_RGBA_0.png")
    if not os.path.exists(path):
        pytest.skip("reference textures not present")
    from importlib import import_module
    render = import_module("sol-rs_gb300.render")
    t = render.load_blue_noise(path)
    assert t.shape == (256, 256, 4) and t.dtype == np.uint8
    assert abs(float(t.mean()) - 127.5) < 2.0          # uniform blue noise
    raw = solrt.imageio.read_png(path)
    assert np.array_equal(t, raw[::-1])               # Texture2d::new flips rows
