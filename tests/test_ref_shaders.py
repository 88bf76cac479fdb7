"""The oracle's pipelines against the reference's own shaders:
pathtrace.rgen / .rchit / .rmiss, ao.* and debug.* (with sampling.glsl,
postprocess.glsl and payload.glsl), rewritten to C++ by
oracle/ref_glsl/build_ref.py and run as ray-tracing pipelines on CPU
threads, traceRayEXT answered by the oracle's watertight closest hit and
sin / cos by the evaluation the oracle and the device share (GLSL leaves
both to the implementation).

The reference material model, its per-pixel TEA / PCG stream, 8 samples, 32
bounces and mix accumulation map to MATERIAL_REF, RNG_REF_STREAM, spp 8,
max_bounces 32 and ACCUM_REF_MIX: the images must be equal bit for bit.
The pipelines are built when the reference checkout (or sources generated
from it) is present; the committed fixtures ref_pathtrace_cornell.npz and
ref_ao_debug_cornell.npz, made by the same pipelines
(tests/golden/make_golden.py), are checked everywhere."""
import os

import numpy as np
import pytest

from helpers import S, camera_of, reference_path, solrt, transformed_cornell

HERE = os.path.dirname(os.path.abspath(__file__))


def _oracle_frames(oracle, o, cam, w, h, sky, frames):
    acc = None
    for f in range(frames):
        p = solrt.render_params(w, h, spp=8, max_bounces=32, frame=f, material_mode=solrt.MATERIAL_REF,
                                rng_mode=solrt.RNG_REF_STREAM, accum_mode=solrt.ACCUM_REF_MIX,
                                miss_mode=solrt.MISS_REF_SKY if sky else solrt.MISS_BLACK)
        acc, rgba8, _ = o.render(cam, p, accum=acc)
    return acc, rgba8


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference shaders not available (no checkout, no generated sources)")
    return oracle


@pytest.mark.parametrize("name,sky", [("cornell", False), ("cornell", True), ("soup", True)])
def test_reference_shaders_equal_oracle(ref, name, sky):
    d = S.cornell() if name == "cornell" else S.soup(20000, seed=3)
    w, h = 48, 40
    cam = camera_of(d, w / h)
    o = ref.OracleScene(d)
    acc = None
    for f in range(2):
        acc, r8 = ref.ref_path_render(o, cam, w, h, frame=f, sky=sky, accum=acc)
    oa, o8 = _oracle_frames(ref, o, cam, w, h, sky, 2)
    assert np.array_equal(acc.view(np.uint32), oa.view(np.uint32))
    assert np.array_equal(r8, o8)
    assert acc[..., :3].mean() > 0


def test_reference_shaders_transformed_sections(ref):
    """Sections with transforms: like the reference, shading interpolates
    object-space vertex data and then applies the section's transform_it /
    transform (pathtrace.rchit:80-90), so the images are equal too."""
    d = transformed_cornell()
    w, h = 48, 40
    cam = camera_of(d, w / h)
    o = ref.OracleScene(d)
    for sky in (False, True):
        acc = None
        for f in range(2):
            acc, r8 = ref.ref_path_render(o, cam, w, h, frame=f, sky=sky, accum=acc)
        oa, o8 = _oracle_frames(ref, o, cam, w, h, sky, 2)
        assert np.array_equal(acc.view(np.uint32), oa.view(np.uint32)), sky
        assert np.array_equal(r8, o8), sky


REF_MODELS = reference_path("assets", "models")


@pytest.mark.parametrize("model,sky", [("cornell.gltf", False), ("tunnel.gltf", True)])
def test_reference_shaders_on_reference_models(ref, model, sky):
    """The reference's own scenes (node transforms, u16 / u32 indices,
    COLOR_0) read by the glTF loader, rendered by the reference's shaders and
    by the oracle: equal bit for bit."""
    path = os.path.join(REF_MODELS, model)
    if not os.path.exists(path):
        pytest.skip("reference models not present")
    g = solrt.load_scene(path)
    w, h = 40, 30
    cam = g.camera(w / h)
    if cam is None:  # the tunnel has none: the example's default camera (5-pathtrace.rs:128-135)
        cam = solrt.camera_look_at((0.0, 0.0, -2.0), (0.0, 0.0, 0.0), (0.0, -1.0, 0.0), 45.0, w / h)
    o = ref.OracleScene(g.data)
    acc = None
    for f in range(2):
        acc, r8 = ref.ref_path_render(o, cam, w, h, frame=f, sky=sky, accum=acc)
    oa, o8 = _oracle_frames(ref, o, cam, w, h, sky, 2)
    assert np.array_equal(acc.view(np.uint32), oa.view(np.uint32))
    assert np.array_equal(r8, o8)
    assert acc[..., :3].mean() > 0


def test_oracle_equals_reference_pipeline_fixture(oracle):
    """The committed image of the reference pipeline (Cornell box, 32 x 24,
    sky, frames 0 and 1) against the oracle, bit for bit."""
    fx = np.load(os.path.join(HERE, "golden", "ref_pathtrace_cornell.npz"))
    d = S.cornell()
    w, h = 32, 24
    cam = camera_of(d, w / h)
    o = oracle.OracleScene(d)
    acc = None
    for f in range(2):
        p = solrt.render_params(w, h, spp=8, max_bounces=32, frame=f, material_mode=solrt.MATERIAL_REF,
                                rng_mode=solrt.RNG_REF_STREAM, miss_mode=solrt.MISS_REF_SKY)
        acc, rgba8, _ = o.render(cam, p, accum=acc)
        assert np.array_equal(acc.view(np.uint32), fx["accum%d" % f].view(np.uint32)), f
        assert np.array_equal(rgba8, fx["rgba8_%d" % f]), f


def blue_noise_fixture():
    """The seeded 64 x 64 RGBA8 stand-in of textures/HDR_RGBA_0.png that
    tests/golden/make_golden.py used."""
    return np.random.default_rng(20261204).integers(0, 256, (64, 64, 4), dtype=np.uint8)


@pytest.mark.parametrize("name", ["cornell", "transformed", "soup"])
def test_reference_ao_and_debug_shaders_equal_oracle(ref, name):
    """ao.rgen / .rchit / .rmiss (4 samples, 4 hits, blue-noise directions,
    RGBA32F target of 4-ray-ao.rs) and debug.rgen / .rchit / .rmiss (RGBA8
    target of 3-ray-debug.rs) against the oracle's AO and debug integrators."""
    d = {"cornell": S.cornell, "transformed": transformed_cornell, "soup": lambda: S.soup(20000, seed=3)}[name]()
    w, h = 48, 40
    cam = camera_of(d, w / h)
    o = ref.OracleScene(d)
    noise = blue_noise_fixture()
    ra = oa = None
    for f in range(3):
        ra = ref.ref_ao_render(o, cam, w, h, noise, frame=f, accum=ra)
        p = solrt.render_params(w, h, spp=4, max_bounces=4, frame=f, integrator=solrt.INTEGRATOR_AO)
        oa, _, _ = o.render(cam, p, accum=oa, blue_noise=noise)
        assert np.array_equal(ra.view(np.uint32), oa.view(np.uint32)), f
    r8 = ref.ref_debug_render(o, cam, w, h)
    _, d8, _ = o.render(cam, solrt.render_params(w, h, spp=1, max_bounces=1, integrator=solrt.INTEGRATOR_DEBUG))
    assert np.array_equal(r8[..., :3], d8[..., :3])


def test_oracle_equals_reference_ao_debug_fixture(oracle):
    fx = np.load(os.path.join(HERE, "golden", "ref_ao_debug_cornell.npz"))
    d = S.cornell()
    w, h = 32, 24
    cam = camera_of(d, w / h)
    o = oracle.OracleScene(d)
    acc = None
    for f in range(2):
        p = solrt.render_params(w, h, spp=4, max_bounces=4, frame=f, integrator=solrt.INTEGRATOR_AO)
        acc, _, _ = o.render(cam, p, accum=acc, blue_noise=fx["noise"])
        assert np.array_equal(acc.view(np.uint32), fx["ao%d" % f].view(np.uint32)), f
    _, d8, _ = o.render(cam, solrt.render_params(w, h, spp=1, max_bounces=1, integrator=solrt.INTEGRATOR_DEBUG))
    assert np.array_equal(d8[..., :3], fx["debug_rgba8"][..., :3])
