"""Generates tests/golden/glsl_sampling.json, ref_pathtrace_cornell.npz and
ref_ao_debug_cornell.npz from the reference's own shaders.

Builds oracle/_ref/libref_glsl.so (the reference's assets/glsl/sampling.glsl
and postprocess.glsl compiled as C++ by oracle/ref_glsl/build_ref.py) and
records, with float bit patterns, the outputs of:
  tea, nextRand sequences, nextRand2, buildOrthonormalBasis,
  fresnelDielectric, sampleGGXDistribution,
  sampleCosineWeightedHemisphere and gammaCorrect
on seeded inputs. Run in a checkout next to the reference:

    python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_glsl"))

import build_ref  # noqa: E402


def fbits(x):
    return struct.unpack("<I", struct.pack("<f", float(x)))[0]


def main():
    lib = ctypes.CDLL(build_ref.build())
    f3 = ctypes.c_float * 3
    lib.ref_tea.restype = ctypes.c_uint32
    lib.ref_tea.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    lib.ref_next_rand.restype = ctypes.c_float
    lib.ref_next_rand.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    lib.ref_fresnel.restype = ctypes.c_float
    rng = np.random.default_rng(20261203)

    out = {"source": "reference assets/glsl/sampling.glsl + postprocess.glsl compiled as C++",
           "float_encoding": "IEEE-754 binary32 bit patterns"}

    # tea on (pixel, frame) style pairs and random pairs
    pairs = [(0, 0), (1, 0), (0, 1), (65535, 7), (0xffffffff, 0xffffffff)]
    pairs += [(int(a), int(b)) for a, b in zip(rng.integers(0, 2**32, 59, dtype=np.uint64),
                                               rng.integers(0, 2**32, 59, dtype=np.uint64))]
    pairs += [(x + y * 256, f) for x, y, f in [(3, 5, 0), (255, 255, 12), (17, 200, 1000)]]
    out["tea"] = [[a, b, lib.ref_tea(a, b)] for a, b in pairs]

    # nextRand sequences from TEA seeds
    seqs = []
    for seed in [0, 1, lib.ref_tea(0, 0), lib.ref_tea(123, 4), 0xdeadbeef, 0xffffffff]:
        st = ctypes.c_uint32(seed)
        vals = []
        for _ in range(48):
            r = lib.ref_next_rand(ctypes.byref(st))
            vals.append([fbits(r), st.value])
        seqs.append({"seed": seed, "steps": vals})
    out["next_rand"] = seqs

    # nextRand2: order of the two draws
    st = ctypes.c_uint32(lib.ref_tea(7, 9))
    o2 = (ctypes.c_float * 2)()
    lib.ref_next_rand2(ctypes.byref(st), o2)
    out["next_rand2"] = {"seed": lib.ref_tea(7, 9), "out": [fbits(o2[0]), fbits(o2[1])], "state": st.value}

    def rand_unit(n):
        v = rng.normal(size=(n, 3)).astype(np.float32)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        return v.astype(np.float32)

    normals = np.concatenate([rand_unit(60), np.array(
        [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, -1, 0], [0.6, 0, -0.8]], np.float32)])

    onb = []
    for n in normals:
        u, v = f3(), f3()
        lib.ref_onb(f3(*n), u, v)
        onb.append([[fbits(c) for c in n], [fbits(c) for c in u], [fbits(c) for c in v]])
    out["onb"] = onb

    fres = []
    for i, m in zip(rand_unit(64), rand_unit(64)):
        for eta in (np.float32(1.0) / np.float32(1.5), np.float32(1.5)):
            r = lib.ref_fresnel(f3(*i), f3(*m), ctypes.c_float(eta))
            fres.append([[fbits(c) for c in i], [fbits(c) for c in m], fbits(eta), fbits(r)])
    out["fresnel"] = fres

    ggx, cosw = [], []
    xis = rng.random((len(normals), 2)).astype(np.float32)
    alphas = np.concatenate([[0.0, 1.0, 0.8002925], rng.random(len(normals) - 3)]).astype(np.float32) ** 2
    for n, xi, a2 in zip(normals, xis, alphas):
        o = f3()
        lib.ref_sample_ggx(f3(*n), ctypes.c_float(xi[0]), ctypes.c_float(xi[1]), ctypes.c_float(a2), o)
        ggx.append([[fbits(c) for c in n], fbits(xi[0]), fbits(xi[1]), fbits(a2), [fbits(c) for c in o]])
        lib.ref_sample_cosine(f3(*n), ctypes.c_float(xi[0]), ctypes.c_float(xi[1]), o)
        cosw.append([[fbits(c) for c in n], fbits(xi[0]), fbits(xi[1]), [fbits(c) for c in o]])
    out["sample_ggx"] = ggx
    out["sample_cosine"] = cosw

    gam = []
    for c in np.concatenate([[0.0, 1.0, 0.5, 1e-6, 2.0], rng.random(59) * 1.2]).astype(np.float32):
        o = f3()
        lib.ref_gamma(f3(c, c, c), ctypes.c_float(2.2), o)
        gam.append([fbits(c), fbits(o[0])])
    out["gamma"] = gam

    # postprocess.glsl tonemaps (Hable's filmic curve, Narkowicz's ACES fit)
    lib.ref_tonemap_uncharted2.argtypes = [f3, f3]
    lib.ref_tonemap_aces.argtypes = [f3, f3]
    tm = {"uncharted2": [], "aces": []}
    xs = np.concatenate([[0.0, 1e-6, 0.5, 1.0, 2.0, 11.2, 100.0], rng.random(57) * 4.0]).astype(np.float32)
    for c in xs:
        for name, fn in (("uncharted2", lib.ref_tonemap_uncharted2), ("aces", lib.ref_tonemap_aces)):
            o = f3()
            fn(f3(c, c, c), o)
            tm[name].append([fbits(c), fbits(o[0])])
    out["tonemap"] = tm

    path = os.path.join(HERE, "glsl_sampling.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path)
    pathtrace_fixture()


def pathtrace_fixture():
    """tests/golden/ref_pathtrace_cornell.npz: the reference's pathtrace.rgen /
    .rchit / .rmiss (compiled as C++, traceRayEXT answered by the oracle's
    watertight closest hit) on the procedural Cornell box, 32 x 24 pixels,
    sky on, two launches (frames 0 and 1) accumulated: the RGBA32F
    accumulation image and the RGBA8 image after each launch."""
    sys.path.insert(0, ROOT)
    import importlib
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    d = solrt.scenes.cornell()
    w, h = 32, 24
    c = d.camera
    cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], w / h)
    o = oracle.OracleScene(d)
    acc = None
    out = {}
    for f in range(2):
        acc, rgba8 = oracle.ref_path_render(o, cam, w, h, frame=f, sky=True, accum=acc)
        out["accum%d" % f] = acc.copy()
        out["rgba8_%d" % f] = rgba8.copy()
    path = os.path.join(HERE, "ref_pathtrace_cornell.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)
    # the sibling pipelines: ao.rgen / .rchit / .rmiss (frames 0 and 1, a seeded
    # stand-in for the blue-noise texture) and debug.rgen / .rchit / .rmiss
    noise = np.random.default_rng(20261204).integers(0, 256, (64, 64, 4), dtype=np.uint8)
    out = {"noise": noise}
    acc = None
    for f in range(2):
        acc = oracle.ref_ao_render(o, cam, w, h, noise, frame=f, accum=acc)
        out["ao%d" % f] = acc.copy()
    out["debug_rgba8"] = oracle.ref_debug_render(o, cam, w, h)
    path = os.path.join(HERE, "ref_ao_debug_cornell.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
