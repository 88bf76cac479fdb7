"""Shared test inputs: seeded rays (random, camera, adversarial) and scenes."""
import importlib

import numpy as np

solrt = importlib.import_module("sol-rs_gb300")
S = solrt.scenes


def reference_path(*parts):
    """A file of the reference checkout (located by the recipe that reads it,
    oracle/ref_glsl/build_ref.py); tests skip where it is absent."""
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "ref_glsl")
    if here not in sys.path:
        sys.path.insert(0, here)
    import build_ref
    return os.path.join(build_ref.reference_root(), *parts)


def random_rays(n, lo, hi, seed, tmin=1e-4, tmax=1e4):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, solrt.RAY_DTYPE)
    r["origin"] = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    r["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def edge_rays(data, n, seed, eye=None):
    """Rays aimed exactly at triangle vertices and at points on shared edges
    (midpoints and random fractions), from random origins: the cases where a
    non-watertight test leaks between neighbouring triangles."""
    rng = np.random.default_rng(seed)
    v = data.vertices["pos"][:, :3].astype(np.float32)
    idx = data.indices.reshape(-1, 3)
    sec = data.sections
    # global vertex ids per triangle (sections are relative to vertex_offset)
    tv = []
    for s in sec:
        t = data.indices[s["index_offset"]:s["index_offset"] + s["index_count"]].reshape(-1, 3) + s["vertex_offset"]
        tv.append(t)
    tv = np.concatenate(tv)
    pick = rng.integers(0, len(tv), n)
    a = v[tv[pick, 0]]
    b = v[tv[pick, 1]]
    c = v[tv[pick, 2]]
    kind = rng.integers(0, 4, n)
    f = rng.random(n).astype(np.float32)[:, None]
    target = np.where(kind[:, None] == 0, a, np.where(kind[:, None] == 1, (a + b) * np.float32(0.5),
                                                       np.where(kind[:, None] == 2, a + (b - a) * f, b + (c - b) * f)))
    lo, hi = v.min(0), v.max(0)
    ext = hi - lo
    if eye is None:
        org = (lo - 0.5 * ext + rng.random((n, 3)) * 2.0 * ext).astype(np.float32)
    else:
        org = np.tile(np.asarray(eye, np.float32), (n, 1))
    d = (target - org).astype(np.float32)
    r = np.zeros(n, solrt.RAY_DTYPE)
    r["origin"] = org
    r["dir"] = d
    r["tmin"] = 1e-6
    r["tmax"] = 1e4
    return r


def axis_rays(lo, hi, n, seed):
    """Rays with one or two zero direction components."""
    rng = np.random.default_rng(seed)
    r = np.zeros(n, solrt.RAY_DTYPE)
    r["origin"] = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    zero = rng.integers(0, 6, n)
    for k in range(3):
        d[zero == k, k] = 0.0
    d[zero == 3, 0] = 0.0
    d[zero == 3, 1] = 0.0
    d[zero == 4, 1] = 0.0
    d[zero == 4, 2] = 0.0
    r["dir"] = d
    r["tmin"] = 0.0
    r["tmax"] = 1e4
    return r


def hits_equal(a, b):
    return np.array_equal(a.view(np.uint32).reshape(-1, 4), b.view(np.uint32).reshape(-1, 4))


def hit_mismatch(a, b):
    return np.nonzero(np.any(a.view(np.uint32).reshape(-1, 4) != b.view(np.uint32).reshape(-1, 4), axis=1))[0]


def camera_of(data, aspect):
    c = data.camera
    return solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], aspect)


def single_triangle():
    b = S._Builder()
    m = b.add_material(S.material(base=(0.5, 0.5, 0.5)))
    b.add_section(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 0, 1]] * 3, np.float32),
                  np.ones((3, 3), np.float32), np.array([0, 1, 2], np.uint32), m)
    return b.build(dict(eye=(0.3, 0.3, -2), center=(0.3, 0.3, 0), up=(0, -1, 0), vfov=40.0), "tri1")


def empty_scene():
    b = S._Builder()
    b.add_material(S.material())
    return b.build(dict(S.CORNELL_CAMERA), "empty")


def transformed_cornell():
    """Cornell box with a non-identity instance transform per section
    (rotation about y + translation), as glTF node transforms produce."""
    d = S.cornell()
    th = np.radians(30.0)
    T = np.array([[np.cos(th), 0, np.sin(th), 0.1], [0, 1, 0, -0.2], [-np.sin(th), 0, np.cos(th), 0.3], [0, 0, 0, 1]],
                 np.float64)
    Tit = np.linalg.inv(T).T
    inst = np.zeros(len(d.sections), S.INSTANCE_DTYPE)
    inst["id"] = np.arange(len(d.sections))
    inst["transform"] = T.T.reshape(-1).astype(np.float32)      # column-major
    inst["transform_it"] = Tit.T.reshape(-1).astype(np.float32)
    d.instances = inst
    return d


def bvh_args(solrt_mod, name):
    """SceneDescription keyword arguments of a BVH name: bvh_kind's names,
    plus "bvh8s" / "bvh4s" for the wide kinds with the SAH collapse,
    "bvh2s" for the binary tree restructured by treelets and "bvh2ts" for
    the two-level kind with every BLAS restructured so."""
    if name in ("bvh8s", "bvh4s", "bvh2s", "bvh2ts"):
        return dict(bvh=bvh_kind(solrt_mod, name[:-1]), sah=True)
    return dict(bvh=bvh_kind(solrt_mod, name))


def bvh_kind(solrt_mod, name):
    """"bvh2" / "bvh2q" / "bvh2t" / "bvh4" / "bvh8" / "bvh8f" -> solrt BVH kind."""
    return {"bvh2": solrt_mod.BVH2, "bvh2q": solrt_mod.BVH2_Q16, "bvh2t": solrt_mod.BVH2_TWO_LEVEL,
            "bvh4": solrt_mod.BVH4_Q8, "bvh8": solrt_mod.BVH8_Q8, "bvh8f": solrt_mod.BVH8_F32}[name]
