"""The oracle's path against the reference's own shaders: pathtrace.rgen,
pathtrace.rchit and pathtrace.rmiss (with sampling.glsl, postprocess.glsl
and payload.glsl), rewritten to C++ by oracle/ref_glsl/build_ref.py and run
as a ray-tracing pipeline on CPU threads, traceRayEXT answered by the
oracle's watertight closest hit and sin / cos by the evaluation the oracle
and the device share (GLSL leaves both to the implementation).

The reference material model, its per-pixel TEA / PCG stream, 8 samples, 32
bounces and mix accumulation map to MATERIAL_REF, RNG_REF_STREAM, spp 8,
max_bounces 32 and ACCUM_REF_MIX: the images must be equal bit for bit.
The pipeline is built when the reference checkout (or sources generated from
it) is present; the committed fixture ref_pathtrace_cornell.npz, made by the
same pipeline (tests/golden/make_golden.py), is checked everywhere."""
import os

import numpy as np
import pytest

from helpers import S, camera_of, solrt, transformed_cornell

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


REF_MODELS = "/root/reference/assets/models"


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
