"""The reference's sibling ray-tracing pipelines over the same traversal:
debug (barycentrics / ray direction, debug.rgen + debug.rchit + debug.rmiss)
and ambient occlusion (ao.rgen + ao.rchit + ao.rmiss with a blue-noise
texture). Both must equal the oracle bit for bit, on both BVH kinds."""
import numpy as np
import pytest

from helpers import S, bvh_kind, camera_of, transformed_cornell

pytestmark = pytest.mark.gpu


def blue_noise(h=64, w=48, seed=17):
    """Seeded stand-in for textures/HDR_RGBA_0.png (RGBA8 texels)."""
    return np.random.default_rng(seed).integers(0, 256, (h, w, 4), dtype=np.uint8)


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
@pytest.mark.parametrize("scene", ["cornell", "transformed", "soup"])
def test_debug_matches_oracle(solrt, oracle, ctx, bvh, scene):
    data = {"cornell": S.cornell, "transformed": transformed_cornell, "soup": lambda: S.soup(20000, seed=3)}[scene]()
    w, h = 48, 40
    kind = bvh_kind(solrt, bvh)
    cam = camera_of(data, w / h)
    sc = solrt.SceneDescription(ctx, data, bvh=kind)
    img = solrt.Image(ctx, w, h)
    p = solrt.render_params(w, h, spp=1, integrator=solrt.INTEGRATOR_DEBUG)
    ctx.reset_stats()
    solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
    ga, g8 = img.read()
    oa, o8, st = oracle.OracleScene(data, two_level=kind == solrt.BVH2_TWO_LEVEL).render(cam, p)
    assert np.array_equal(ga.view(np.uint32), oa.view(np.uint32))
    assert np.array_equal(g8, o8)
    s = ctx.stats()
    assert s.segments == st.segments == w * h and s.error_flags == 0
    hit = np.abs(ga[..., :3].sum(-1) - 1.0) < 1e-5
    assert hit.any()


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
def test_ao_matches_oracle(solrt, oracle, ctx, bvh):
    data = S.cornell()
    w, h = 40, 32
    kind = bvh_kind(solrt, bvh)
    cam = camera_of(data, w / h)
    noise = blue_noise()
    ctx.set_blue_noise(noise)
    sc = solrt.SceneDescription(ctx, data, bvh=kind)
    img = solrt.Image(ctx, w, h)
    o = oracle.OracleScene(data, two_level=kind == solrt.BVH2_TWO_LEVEL)
    acc = np.zeros((h, w, 4), np.float32)
    seg = 0
    ctx.reset_stats()
    for f in range(3):
        p = solrt.render_params(w, h, spp=4, max_bounces=4, frame=f, integrator=solrt.INTEGRATOR_AO)
        solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
        acc, o8, st = o.render(cam, p, accum=acc, blue_noise=noise)
        seg += st.segments
    ga, g8 = img.read()
    assert np.array_equal(ga.view(np.uint32), acc.view(np.uint32))
    assert np.array_equal(g8, o8)
    assert ctx.stats().segments == seg and ctx.stats().error_flags == 0
    assert 0.0 < ga[..., :3].mean() < 1.0


def test_integrator_errors(solrt, ctx):
    data = S.cornell()
    c2 = solrt.Context(0)
    sc = solrt.SceneDescription(c2, data)
    img = solrt.Image(c2, 8, 8)
    cam = camera_of(data, 1.0)
    with pytest.raises(solrt.SolrtError, match="blue_noise"):
        solrt.Renderer(c2).cmd_trace_rays(sc, cam, solrt.render_params(8, 8, spp=4, max_bounces=4,
                                                                       integrator=solrt.INTEGRATOR_AO), img)
    with pytest.raises(solrt.SolrtError, match="integrator"):
        solrt.Renderer(c2).cmd_trace_rays(sc, cam, solrt.render_params(8, 8, integrator=7), img)
    p = solrt.render_params(8, 8, integrator=solrt.INTEGRATOR_DEBUG)
    with pytest.raises(solrt.SolrtError, match="path integrator"):
        solrt.Batch(c2, [(sc, img, cam, p)])
    sc.close()
    img.close()
    c2.close()


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2t", "bvh8"])
def test_gpu_equals_reference_ao_debug_fixture(solrt, ctx, bvh):
    """The device against the committed images of the reference's own
    ao.rgen / .rchit / .rmiss and debug.rgen / .rchit / .rmiss compiled as
    C++ (tests/golden/ref_ao_debug_cornell.npz): bit for bit."""
    import os
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ao_debug_cornell.npz"))
    d = S.cornell()
    w, h = 32, 24
    cam = camera_of(d, w / h)
    ctx.set_blue_noise(fx["noise"])
    sc = solrt.SceneDescription(ctx, d, bvh=bvh_kind(solrt, bvh))
    img = solrt.Image(ctx, w, h)
    r = solrt.Renderer(ctx)
    for f in range(2):
        r.cmd_trace_rays(sc, cam, solrt.render_params(w, h, spp=4, max_bounces=4, frame=f,
                                                      integrator=solrt.INTEGRATOR_AO), img)
        a32, _ = img.read()
        assert np.array_equal(a32.view(np.uint32), fx["ao%d" % f].view(np.uint32)), f
    dbg = solrt.Image(ctx, w, h)
    r.cmd_trace_rays(sc, cam, solrt.render_params(w, h, spp=1, max_bounces=1, integrator=solrt.INTEGRATOR_DEBUG), dbg)
    _, d8 = dbg.read()
    assert np.array_equal(d8[..., :3], fx["debug_rgba8"][..., :3])
