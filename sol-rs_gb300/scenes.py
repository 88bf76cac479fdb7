"""Synthetic scenes of the benchmark configurations, as plain arrays.

A SceneData holds exactly what SceneDescription::from_meshes consumes in the
reference (src/ray/mod.rs:59-156): ModelVertex array (64 B each,
src/scene/mesh.rs:9-14), u32 indices, primitive sections (vertex range, index
range, material; src/scene/mod.rs:37-44), MaterialInfo array (48 B,
src/scene/mod.rs:21-29) and optional per-section instances (transform,
transform_it; src/ray/mod.rs:18-24). The same arrays feed the CUDA library
and the CPU oracle.

All randomness comes from numpy's PCG64 Generator with the configuration's
seed. Vertex normals are per-face for walls, boxes and the soup (vertices
are not shared between faces) and radial for the tunnel.
"""
import math

import numpy as np

VERTEX_DTYPE = np.dtype([("pos", "<f4", 4), ("color", "<f4", 4), ("normal", "<f4", 4), ("uv", "<f4", 4)])
MATERIAL_DTYPE = np.dtype([("base_color", "<f4", 4), ("emissive", "<f4", 3), ("padding0", "<f4"),
                           ("metallic", "<f4"), ("roughness", "<f4"), ("padding1", "<f4"), ("padding2", "<f4")])
SECTION_DTYPE = np.dtype([("vertex_offset", "<u4"), ("vertex_count", "<u4"), ("index_offset", "<u4"),
                          ("index_count", "<u4"), ("material_index", "<u4"), ("reserved", "<u4")])
INSTANCE_DTYPE = np.dtype([("id", "<u4"), ("texture_offset", "<u4"), ("padding", "<f4", 2),
                           ("transform", "<f4", 16), ("transform_it", "<f4", 16)])
assert VERTEX_DTYPE.itemsize == 64 and MATERIAL_DTYPE.itemsize == 48 and INSTANCE_DTYPE.itemsize == 144


class SceneData:
    def __init__(self, vertices, indices, sections, materials, instances=None, camera=None, name=""):
        self.vertices = np.ascontiguousarray(vertices, dtype=VERTEX_DTYPE)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32)
        self.sections = np.ascontiguousarray(sections, dtype=SECTION_DTYPE)
        self.materials = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
        self.instances = None if instances is None else np.ascontiguousarray(instances, dtype=INSTANCE_DTYPE)
        self.camera = camera or {}
        self.name = name

    @property
    def tri_count(self):
        return int(self.sections["index_count"].sum() // 3) if len(self.sections) else 0

    def nbytes(self):
        n = self.vertices.nbytes + self.indices.nbytes + self.sections.nbytes + self.materials.nbytes
        return n + (self.instances.nbytes if self.instances is not None else 0)


def material(base=(1, 1, 1), emissive=(0, 0, 0), metallic=0.0, roughness=1.0):
    m = np.zeros(1, MATERIAL_DTYPE)
    m["base_color"][0] = (base[0], base[1], base[2], 1.0)
    m["emissive"][0] = emissive
    m["metallic"][0] = metallic
    m["roughness"][0] = roughness
    return m[0]


class _Builder:
    """Accumulates sections of unshared-vertex triangles."""

    def __init__(self):
        self.verts, self.idx, self.secs, self.mats = [], [], [], []
        self.nv = 0
        self.ni = 0

    def add_material(self, m):
        self.mats.append(m)
        return len(self.mats) - 1

    def add_section(self, positions, normals, colors, indices, mat):
        nv = len(positions)
        v = np.zeros(nv, VERTEX_DTYPE)
        v["pos"][:, :3] = positions
        v["pos"][:, 3] = 1.0
        v["normal"][:, :3] = normals
        v["normal"][:, 3] = 1.0
        v["color"][:, :3] = colors
        v["color"][:, 3] = 1.0
        s = np.zeros(1, SECTION_DTYPE)
        s["vertex_offset"], s["vertex_count"] = self.nv, nv
        s["index_offset"], s["index_count"] = self.ni, len(indices)
        s["material_index"] = mat
        self.verts.append(v)
        self.idx.append(np.asarray(indices, np.uint32))
        self.secs.append(s)
        self.nv += nv
        self.ni += len(indices)

    def add_quads(self, quads, mat, color=(1.0, 1.0, 1.0)):
        """quads: (Q, 4, 3) corner positions in order around the quad."""
        quads = np.asarray(quads, np.float32).reshape(-1, 4, 3)
        n = np.cross(quads[:, 1] - quads[:, 0], quads[:, 2] - quads[:, 0])
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        pos = quads.reshape(-1, 3)
        nrm = np.repeat(n, 4, axis=0)
        col = np.tile(np.asarray(color, np.float32), (len(pos), 1))
        base = np.arange(len(quads), dtype=np.uint32)[:, None] * 4
        tri = np.concatenate([base + np.array([0, 1, 2], np.uint32), base + np.array([0, 2, 3], np.uint32)], axis=1)
        self.add_section(pos, nrm, col, tri.reshape(-1), mat)

    def build(self, camera=None, name=""):
        return SceneData(np.concatenate(self.verts) if self.verts else np.zeros(0, VERTEX_DTYPE),
                         np.concatenate(self.idx) if self.idx else np.zeros(0, np.uint32),
                         np.concatenate(self.secs) if self.secs else np.zeros(0, SECTION_DTYPE),
                         np.array(self.mats, MATERIAL_DTYPE), None, camera, name)


def _box_quads(cx, cz, w, d, h, angle_deg):
    """Four sides and the top of a box on the floor (no bottom face: the
    reference's cornell.gltf boxes have 10 triangles, accessors 15 and 18)."""
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    corners = []
    for dx, dz in ((-w / 2, -d / 2), (w / 2, -d / 2), (w / 2, d / 2), (-w / 2, d / 2)):
        corners.append((cx + ca * dx - sa * dz, cz + sa * dx + ca * dz))
    q = []
    for i in range(4):
        (x0, z0), (x1, z1) = corners[i], corners[(i + 1) % 4]
        q.append([(x0, 0, z0), (x1, 0, z1), (x1, h, z1), (x0, h, z0)])
    q.append([(x, h, z) for x, z in corners[::-1]])
    return np.array(q, np.float32)


CORNELL_CAMERA = dict(eye=(0.5, 0.5, -1.4), center=(0.5, 0.5, 0.5), up=(0.0, -1.0, 0.0), vfov=40.0)


def cornell(white=(0.73, 0.73, 0.73), red=(0.65, 0.05, 0.05), green=(0.12, 0.45, 0.15),
            light=(17.0, 12.0, 4.0), short_angle=15.0, tall_angle=-18.0, short_pos=(0.66, 0.35),
            tall_pos=(0.34, 0.64), builder=None):
    """Procedural Cornell box in [0,1]^3: floor, ceiling, back, left (red,
    x=0), right (green, x=1), a 0.25 x 0.25 ceiling light, a 0.3-tall box
    rotated 15 deg and a 0.6-tall box rotated -18 deg. 32 triangles."""
    b = builder or _Builder()
    m_light = b.add_material(material(emissive=light))
    m_white = b.add_material(material(base=white))
    m_red = b.add_material(material(base=red))
    m_green = b.add_material(material(base=green))
    lo, hi = 0.375, 0.625
    b.add_quads([[(lo, 0.999, lo), (hi, 0.999, lo), (hi, 0.999, hi), (lo, 0.999, hi)]], m_light)
    b.add_quads([[(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)]], m_white)          # floor
    b.add_quads([[(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)]], m_white)          # ceiling
    b.add_quads([[(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]], m_white)          # back
    b.add_quads([[(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)]], m_red)            # left
    b.add_quads([[(1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)]], m_green)          # right
    b.add_quads(_box_quads(short_pos[0], short_pos[1], 0.3, 0.3, 0.3, short_angle), m_white)
    b.add_quads(_box_quads(tall_pos[0], tall_pos[1], 0.3, 0.3, 0.6, tall_angle), m_white)
    if builder is None:
        return b.build(dict(CORNELL_CAMERA), "cornell")
    return b


def soup(n_tris, seed=2, lo=0.0, hi=1.0, sigma=0.005, builder=None):
    """Triangle soup: centroids uniform in [lo,hi]^3, each vertex = centroid +
    N(0, sigma^2) per axis, per-triangle albedo uniform in [0.2, 0.8]^3 stored
    as vertex colour under a white material."""
    rng = np.random.default_rng(seed)
    cen = rng.uniform(lo, hi, size=(n_tris, 3)).astype(np.float32)
    off = rng.normal(0.0, sigma, size=(n_tris, 3, 3)).astype(np.float32)
    pos = (cen[:, None, :] + off).astype(np.float32)
    alb = rng.uniform(0.2, 0.8, size=(n_tris, 3)).astype(np.float32)
    n = np.cross(pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0, 1, 0], np.float32)).astype(np.float32)
    b = builder or _Builder()
    m = b.add_material(material(base=(1.0, 1.0, 1.0)))
    b.add_section(pos.reshape(-1, 3), np.repeat(n, 3, axis=0), np.repeat(alb, 3, axis=0),
                  np.arange(3 * n_tris, dtype=np.uint32), m)
    if builder is None:
        cam = dict(eye=(0.5 * (lo + hi), 0.5 * (lo + hi), lo - 1.2 * (hi - lo)), center=(0.5 * (lo + hi),) * 3,
                   up=(0.0, -1.0, 0.0), vfov=45.0)
        return b.build(cam, "soup%d" % n_tris)
    return b


def rotation(axis, deg):
    """3x3 rotation about a unit axis (Rodrigues), FP64."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    t = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * (K @ K)


def instance_of(M, ident):
    """SceneInstance of a 4x4 row-major FP64 transform: transform and
    inverse-transpose rounded to FP32, stored column-major (glam layout)."""
    inst = np.zeros((), INSTANCE_DTYPE)
    inst["id"] = ident
    inst["transform"] = M.astype(np.float32).T.reshape(-1)
    inst["transform_it"] = np.linalg.inv(M.astype(np.float32).astype(np.float64)).T.astype(np.float32).T.reshape(-1)
    return inst


def instanced_soups(n_side=4, tris_each=16384, seed=5, angle=0.0):
    """n_side^3 sections, each a triangle soup of `tris_each` triangles in the
    unit cube of its own object space, placed by its instance in one cell of
    an n_side^3 grid over [0, 1]^3 (scaled by 1 / n_side, turned by a random
    rotation about its centre plus `angle` degrees about y): the per-section
    instances of SceneDescription::from_meshes (src/ray/mod.rs:59-156)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    insts = []
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                soup(tris_each, seed=seed * 1000 + k, builder=b)
                R = rotation(rng.normal(size=3), rng.uniform(0, 360)) @ rotation((0, 1, 0), angle)
                c = (np.array([ix, iy, iz], np.float64) + 0.5) / n_side
                M = np.eye(4)
                M[:3, :3] = R / n_side
                M[:3, 3] = c - (R / n_side) @ np.full(3, 0.5)
                insts.append(instance_of(M, k))
                k += 1
    cam = dict(eye=(0.5, 0.5, -1.2), center=(0.5, 0.5, 0.5), up=(0.0, -1.0, 0.0), vfov=45.0)
    d = b.build(cam, "instances%dx%d" % (n_side ** 3, tris_each))
    d.instances = np.array(insts, INSTANCE_DTYPE)
    return d


def _value_noise(u, v, nu, nv, rng):
    """Smooth value noise on a periodic-in-u lattice of nu x nv cells,
    values uniform in [-1, 1], smoothstep interpolation. u, v in cell units."""
    lat = rng.uniform(-1.0, 1.0, size=(nv + 2, nu)).astype(np.float64)
    iu = np.floor(u).astype(np.int64)
    iv = np.floor(v).astype(np.int64)
    fu = u - iu
    fv = v - iv
    su = fu * fu * (3 - 2 * fu)
    sv = fv * fv * (3 - 2 * fv)
    i0, i1 = iu % nu, (iu + 1) % nu
    j0, j1 = np.clip(iv, 0, nv + 1), np.clip(iv + 1, 0, nv + 1)
    a = lat[j0, i0] * (1 - su) + lat[j0, i1] * su
    b = lat[j1, i0] * (1 - su) + lat[j1, i1] * su
    return a * (1 - sv) + b * sv


TUNNEL_CAMERA = dict(eye=(0.0, 0.0, 2.0), center=(0.0, 0.0, 12.0), up=(0.0, -1.0, 0.0), vfov=60.0)


def tunnel(n_ang=2048, n_ax=1024, radius=1.0, length=200.0, amp=0.02, emissive_frac=0.02, emission=5.0, seed=3):
    """Tessellated cylinder along +z (n_ang x n_ax quads, 2 triangles each),
    vertex radius 1 + amp * value_noise, radial normals pointing inward, a
    fraction of quads emissive. Open at both ends."""
    rng = np.random.default_rng(seed)
    ang = np.arange(n_ang, dtype=np.float64) * (2 * math.pi / n_ang)
    zs = np.arange(n_ax + 1, dtype=np.float64) * (length / n_ax)
    A, Z = np.meshgrid(ang, zs)                       # (n_ax+1, n_ang)
    noise = _value_noise(A / (2 * math.pi) * 64.0, Z / length * 256.0, 64, 256, rng)
    r = radius * (1.0 + amp * noise)
    pos = np.stack([r * np.cos(A), r * np.sin(A), Z], axis=-1).reshape(-1, 3).astype(np.float32)
    nrm = np.stack([-np.cos(A), -np.sin(A), np.zeros_like(A)], axis=-1).reshape(-1, 3).astype(np.float32)
    col = np.ones_like(pos)
    j, i = np.meshgrid(np.arange(n_ax, dtype=np.uint32), np.arange(n_ang, dtype=np.uint32), indexing="ij")
    v00 = j * n_ang + i
    v01 = j * n_ang + (i + 1) % n_ang
    v10 = (j + 1) * n_ang + i
    v11 = (j + 1) * n_ang + (i + 1) % n_ang
    tris = np.stack([np.stack([v00, v10, v11], -1), np.stack([v00, v11, v01], -1)], axis=2)  # (n_ax, n_ang, 2, 3)
    emis = rng.random((n_ax, n_ang)) < emissive_frac
    b = _Builder()
    m_wall = b.add_material(material(base=(0.73, 0.73, 0.73)))
    m_light = b.add_material(material(base=(1, 1, 1), emissive=(emission, emission, emission)))
    wall_idx = tris[~emis].reshape(-1)
    light_idx = tris[emis].reshape(-1)
    v = np.zeros(len(pos), VERTEX_DTYPE)
    v["pos"][:, :3] = pos
    v["pos"][:, 3] = 1.0
    v["normal"][:, :3] = nrm
    v["normal"][:, 3] = 1.0
    v["color"][:, :3] = col
    v["color"][:, 3] = 1.0
    secs = np.zeros(2, SECTION_DTYPE)
    secs["vertex_offset"] = 0
    secs["vertex_count"] = len(pos)
    secs["index_offset"] = [0, len(wall_idx)]
    secs["index_count"] = [len(wall_idx), len(light_idx)]
    secs["material_index"] = [m_wall, m_light]
    return SceneData(v, np.concatenate([wall_idx, light_idx]), secs, np.array(b.mats, MATERIAL_DTYPE), None,
                     dict(TUNNEL_CAMERA), "tunnel%dx%d" % (n_ang, n_ax))


def mixed_scene(i, seed_base=4, min_tris=1000, max_tris=500000):
    """One scene of the batched workload: a randomised Cornell box with a
    triangle soup of log-uniform size inside it, plus its job parameters."""
    rng = np.random.default_rng(seed_base + i)
    n = int(round(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))))
    white = tuple(rng.uniform(0.6, 0.8, 3))
    red = (rng.uniform(0.5, 0.8), rng.uniform(0.02, 0.1), rng.uniform(0.02, 0.1))
    green = (rng.uniform(0.05, 0.2), rng.uniform(0.3, 0.6), rng.uniform(0.05, 0.2))
    b = cornell(white=white, red=red, green=green, short_angle=rng.uniform(-30, 30), tall_angle=rng.uniform(-30, 30),
                builder=_Builder())
    soup(n, seed=seed_base + i, lo=0.15, hi=0.85, sigma=0.005, builder=b)
    res = int(rng.choice([128, 256, 512, 1024]))
    spp = int(rng.integers(4, 65))
    data = b.build(dict(CORNELL_CAMERA), "mixed%d" % i)
    return data, dict(width=res, height=res, spp=spp, max_bounces=5, seed=seed_base + i)


def probe_rays(data, camera, width, height, n, seed=7, tmin=1e-3, tmax=1e4):
    """Ray set of the hit-record studies: every pixel-centre camera ray of a
    width x height image of `camera` (row-major, first), then seeded rays
    from uniform points of the scene's bounding box in uniform directions,
    n rays in all. Returns a structured array (origin, tmin, dir, tmax);
    camera directions are normalize(P^-1 (x, y, 1, 1)) through the view
    inverse, computed in FP64 and rounded to FP32."""
    ray_dtype = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
    n_cam = min(n, width * height)
    rays = np.zeros(n, ray_dtype)
    V = np.array(camera.view_inverse, np.float64).reshape(4, 4).T
    P = np.array(camera.projection_inverse, np.float64).reshape(4, 4).T
    ys, xs = np.mgrid[0:height, 0:width]
    d = np.stack([(xs + 0.5) / width * 2 - 1, (ys + 0.5) / height * 2 - 1, np.ones(xs.shape), np.ones(xs.shape)], -1)
    t = d.reshape(-1, 4)[:n_cam] @ P.T
    t = t[:, :3] / np.linalg.norm(t[:, :3], axis=1, keepdims=True)
    rays["origin"][:n_cam] = V[:3, 3].astype(np.float32)
    rays["dir"][:n_cam] = (t @ V[:3, :3].T).astype(np.float32)
    rng = np.random.default_rng(seed)
    pos = data.vertices["pos"][:, :3]
    lo, hi = pos.min(0).astype(np.float64), pos.max(0).astype(np.float64)
    m = n - n_cam
    rays["origin"][n_cam:] = (lo + rng.random((m, 3)) * (hi - lo)).astype(np.float32)
    dd = rng.normal(size=(m, 3))
    rays["dir"][n_cam:] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    rays["tmin"] = tmin
    rays["tmax"] = tmax
    return rays


def near_edge(hits):
    """Hits within about one float ulp of a triangle edge: a barycentric
    (u, v or 1 - u - v) below 2^-23. `hits` is a (t, prim, u, v) array."""
    h = np.asarray(hits)
    u = h["u"].astype(np.float64)
    v = h["v"].astype(np.float64)
    hit = h["prim"] != 0xFFFFFFFF
    return hit & (np.minimum(np.minimum(u, v), 1.0 - u - v) < 2.0 ** -23)


def write_gltf(data, path, view=None, yfov=None, znear=0.01, zfar=100.0, node_transforms=None,
               index_type="u32", external_bin=False):
    """Writes a SceneData as glTF 2.0 that load_scene reads back
    (src/scene/mod.rs:138-295 / solrt_gltf_load): one mesh and one node per
    section, positions / normals / COLOR_0 / TEXCOORD_0 as float accessors,
    indices as u16 or u32, the materials' factors, and optionally a
    perspective camera node whose matrix is `view` (column-major) with
    `yfov` in the reference's unit (degrees, passed through Camera::from_view).

    node_transforms: optional per-section dict of glTF node properties
    ("matrix" or "translation"/"rotation"/"scale"); the vertices are written
    as stored, so the loaded instance transform is the node's.
    Path suffix .glb writes a binary container; external_bin writes the
    buffer beside a .gltf instead of a base64 data URI.
    """
    import base64
    import json
    import os
    import struct

    blob = bytearray()
    views, accessors = [], []

    def add(arr, ctype, atype, target=None, minmax=False):
        arr = np.ascontiguousarray(arr)
        while len(blob) % 4:
            blob.append(0)
        off = len(blob)
        blob.extend(arr.tobytes())
        bv = {"buffer": 0, "byteOffset": off, "byteLength": arr.nbytes}
        if target:
            bv["target"] = target
        views.append(bv)
        acc = {"bufferView": len(views) - 1, "componentType": ctype, "count": int(arr.shape[0]), "type": atype}
        if minmax and arr.shape[0]:
            acc["min"] = [float(x) for x in arr.min(axis=0)]
            acc["max"] = [float(x) for x in arr.max(axis=0)]
        accessors.append(acc)
        return len(accessors) - 1

    meshes, nodes = [], []
    for si, s in enumerate(data.sections):
        v = data.vertices[int(s["vertex_offset"]):int(s["vertex_offset"] + s["vertex_count"])]
        idx = data.indices[int(s["index_offset"]):int(s["index_offset"] + s["index_count"])]
        attrs = {
            "POSITION": add(v["pos"][:, :3].astype("<f4"), 5126, "VEC3", 34962, minmax=True),
            "NORMAL": add(v["normal"][:, :3].astype("<f4"), 5126, "VEC3", 34962),
            "COLOR_0": add(v["color"].astype("<f4"), 5126, "VEC4", 34962),
            "TEXCOORD_0": add(v["uv"][:, :2].astype("<f4"), 5126, "VEC2", 34962),
        }
        if index_type == "u16":
            ia = add(idx.astype("<u2"), 5123, "SCALAR", 34963)
        else:
            ia = add(idx.astype("<u4"), 5125, "SCALAR", 34963)
        meshes.append({"primitives": [{"attributes": attrs, "indices": ia, "material": int(s["material_index"]),
                                       "mode": 4}]})
        node = {"mesh": si}
        if node_transforms is not None and node_transforms[si]:
            node.update(node_transforms[si])
        nodes.append(node)
    mats = []
    for m in data.materials:
        mats.append({"pbrMetallicRoughness": {"baseColorFactor": [float(x) for x in m["base_color"]],
                                              "metallicFactor": float(m["metallic"]),
                                              "roughnessFactor": float(m["roughness"])},
                     "emissiveFactor": [float(x) for x in m["emissive"]]})
    doc = {"asset": {"version": "2.0", "generator": "sol-rs_gb300 scenes.write_gltf"},
           "scene": 0, "scenes": [{"nodes": list(range(len(nodes)))}],
           "nodes": nodes, "meshes": meshes, "materials": mats, "accessors": accessors, "bufferViews": views}
    if view is not None:
        doc["cameras"] = [{"type": "perspective",
                           "perspective": {"yfov": float(yfov), "znear": float(znear), "zfar": float(zfar),
                                           "aspectRatio": 1.0}}]
        nodes.append({"camera": 0, "matrix": [float(x) for x in np.asarray(view, np.float64).reshape(16)]})
        doc["scenes"][0]["nodes"].append(len(nodes) - 1)
    while len(blob) % 4:
        blob.append(0)
    if str(path).endswith(".glb"):
        doc["buffers"] = [{"byteLength": len(blob)}]
        js = json.dumps(doc).encode()
        js += b" " * ((4 - len(js) % 4) % 4)
        total = 12 + 8 + len(js) + 8 + len(blob)
        with open(path, "wb") as f:
            f.write(struct.pack("<4sII", b"glTF", 2, total))
            f.write(struct.pack("<II", len(js), 0x4E4F534A) + js)
            f.write(struct.pack("<II", len(blob), 0x004E4942) + bytes(blob))
        return
    if external_bin:
        bin_name = os.path.splitext(os.path.basename(str(path)))[0] + ".bin"
        with open(os.path.join(os.path.dirname(str(path)), bin_name), "wb") as f:
            f.write(bytes(blob))
        doc["buffers"] = [{"byteLength": len(blob), "uri": bin_name}]
    else:
        doc["buffers"] = [{"byteLength": len(blob),
                           "uri": "data:application/octet-stream;base64," + base64.b64encode(bytes(blob)).decode()}]
    with open(path, "w") as f:
        json.dump(doc, f)
