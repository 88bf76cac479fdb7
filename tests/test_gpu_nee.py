"""Next-event estimation (SOLRT_INTEGRATOR_PATH_NEE): the shadow-ray queue
of the wavefront against the oracle's per-pixel restatement of the same
estimator. Images must match bit for bit, as must the counts of path
segments, shadow rays and unoccluded shadow rays; the estimator must
converge to the reference estimator's image (same expectation, less noise),
and the parameter checks must reject what it does not support."""
import numpy as np
import pytest

from helpers import S, bvh_kind, camera_of, transformed_cornell

pytestmark = pytest.mark.gpu


def _case(solrt, name):
    L = solrt.MATERIAL_LAMBERT
    nee = solrt.INTEGRATOR_PATH_NEE
    if name == "cornell":
        return S.cornell(), 48, 40, dict(spp=4, max_bounces=5, material_mode=L, rng_mode=solrt.RNG_PER_SAMPLE,
                                         seed=1, integrator=nee)
    if name == "cornell_ref_stream":
        return S.cornell(), 32, 32, dict(spp=3, max_bounces=8, material_mode=L, rng_mode=solrt.RNG_REF_STREAM,
                                         integrator=nee)
    if name == "transformed":
        return transformed_cornell(), 32, 32, dict(spp=3, max_bounces=4, material_mode=L,
                                                   rng_mode=solrt.RNG_PER_SAMPLE, seed=7, integrator=nee)
    if name == "tunnel_kahan":  # many small emissive triangles: the pick's binary search
        return S.tunnel(n_ang=256, n_ax=128, length=25.0), 48, 28, dict(
            spp=2, max_bounces=6, material_mode=L, rng_mode=solrt.RNG_PER_SAMPLE, seed=3,
            miss_mode=solrt.MISS_REF_SKY, accum_mode=solrt.ACCUM_KAHAN, integrator=nee)
    raise KeyError(name)


def _render_both(solrt, oracle, ctx, data, w, h, kw, frames=2, bvh=None):
    bvh = solrt.BVH2 if bvh is None else bvh
    cam = camera_of(data, w / h)
    sc = solrt.SceneDescription(ctx, data, bvh=bvh)
    mode = kw.get("accum_mode", solrt.ACCUM_REF_MIX)
    img = solrt.Image(ctx, w, h, mode)
    r = solrt.Renderer(ctx)
    o = oracle.OracleScene(data, two_level=bvh == solrt.BVH2_TWO_LEVEL)
    acc = np.zeros((h, w, 4), np.float32)
    ks = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    kc = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    seg = shadow = unocc = 0
    ctx.reset_stats()
    for f in range(frames):
        p = solrt.render_params(w, h, frame=f, **kw)
        r.cmd_trace_rays(sc, cam, p, img)
        acc, _, st = o.render(cam, p, accum=acc, ksum=ks, kcomp=kc)
        seg += st.segments
        shadow += st.shadow_segments
        unocc += st.shadow_unoccluded
    ctx.synchronize()
    ga, _ = img.read()
    return ga, acc, ctx.stats(), (seg, shadow, unocc)


@pytest.mark.parametrize("kernel", ["wavefront", "mega"])
@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
@pytest.mark.parametrize("name", ["cornell", "cornell_ref_stream", "transformed", "tunnel_kahan"])
def test_nee_bit_exact(solrt, oracle, ctx, name, bvh, kernel):
    """The shadow-ray queue of the wavefront, and the per-pixel kernel
    tracing each shadow ray at its vertex, against the oracle."""
    data, w, h, kw = _case(solrt, name)
    kw = dict(kw, kernel=solrt.KERNEL_MEGA if kernel == "mega" else solrt.KERNEL_WAVEFRONT)
    ga, oa, st, (seg, shadow, unocc) = _render_both(solrt, oracle, ctx, data, w, h, kw, bvh=bvh_kind(solrt, bvh))
    diff = np.nonzero(np.any(ga.view(np.uint32) != oa.view(np.uint32), axis=-1))
    assert len(diff[0]) == 0, (len(diff[0]), list(zip(diff[0][:5], diff[1][:5])), ga[diff][:3], oa[diff][:3])
    assert st.segments == seg and st.error_flags == 0
    assert st.shadow_segments == shadow and st.shadow_unoccluded == unocc
    assert shadow > 0 and 0 < unocc <= shadow
    assert np.isfinite(ga).all() and ga[..., :3].mean() > 0


def test_nee_converges_to_the_reference_estimator(solrt, ctx):
    """Same expectation as pathtrace.rchit's estimator with Lambert
    materials, lower noise: the image mean agrees within 1.5 %, and the
    median per-pixel difference between two seeds is several times smaller
    than the plain estimator's at equal spp."""
    d = S.cornell()
    w = h = 64
    cam = camera_of(d, 1.0)
    sc = solrt.SceneDescription(ctx, d)
    r = solrt.Renderer(ctx)

    def render(integ, spp, seed):
        img = solrt.Image(ctx, w, h, solrt.ACCUM_REF_MIX)
        p = solrt.render_params(w, h, spp=spp, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                                rng_mode=solrt.RNG_PER_SAMPLE, seed=seed, integrator=integ)
        r.cmd_trace_rays(sc, cam, p, img)
        ctx.synchronize()
        a = img.read()[0][..., :3].copy()
        img.close()
        return a

    ref = render(solrt.INTEGRATOR_PATH, 8192, 11)
    nee = render(solrt.INTEGRATOR_PATH_NEE, 1024, 12)
    assert abs(nee.mean() - ref.mean()) < 0.015 * ref.mean(), (nee.mean(), ref.mean())
    n1, n2 = render(solrt.INTEGRATOR_PATH_NEE, 256, 21), render(solrt.INTEGRATOR_PATH_NEE, 256, 22)
    p1, p2 = render(solrt.INTEGRATOR_PATH, 256, 21), render(solrt.INTEGRATOR_PATH, 256, 22)
    assert np.median(np.abs(n1 - n2)) < 0.3 * np.median(np.abs(p1 - p2))


def test_nee_scene_without_lights(solrt, oracle, ctx):
    """No emissive triangle: no shadow rays, the sky alone lights the image,
    still equal to the oracle."""
    d = S.soup(20000, seed=2)
    kw = dict(spp=2, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=4,
              miss_mode=solrt.MISS_GRADIENT, integrator=solrt.INTEGRATOR_PATH_NEE)
    ga, oa, st, (seg, shadow, unocc) = _render_both(solrt, oracle, ctx, d, 40, 24, kw, frames=1)
    assert np.array_equal(ga.view(np.uint32), oa.view(np.uint32))
    assert st.segments == seg and st.shadow_segments == 0 == shadow


def test_nee_rejects_unsupported(solrt, ctx):
    d = S.cornell()
    sc = solrt.SceneDescription(ctx, d)
    img = solrt.Image(ctx, 8, 8, solrt.ACCUM_REF_MIX)
    cam = camera_of(d, 1.0)
    r = solrt.Renderer(ctx)
    bad = [dict(material_mode=solrt.MATERIAL_REF),
           dict(material_mode=solrt.MATERIAL_REF, kernel=solrt.KERNEL_MEGA)]
    for kw in bad:
        p = solrt.render_params(8, 8, spp=1, max_bounces=2, integrator=solrt.INTEGRATOR_PATH_NEE, **kw)
        with pytest.raises(solrt.SolrtError):
            r.cmd_trace_rays(sc, cam, p, img)
    srv = solrt.Server(ctx)
    with pytest.raises(solrt.SolrtError):
        srv.submit(sc, cam, solrt.render_params(8, 8, spp=1, integrator=solrt.INTEGRATOR_PATH_NEE,
                                                material_mode=solrt.MATERIAL_REF))
    srv.close()


def test_nee_pass_splitting_invariance(solrt, oracle):
    """Tiny path capacities force many passes (each with its own shadow
    queue per bounce); the image must not change and must equal the
    oracle's."""
    data, w, h, kw = _case(solrt, "cornell")
    kw = dict(kw, spp=5)
    out = []
    for cap in (0, 1000, 4096 + 7):
        c = solrt.Context(0, path_capacity=cap)
        ga, oa, st, (seg, shadow, unocc) = _render_both(solrt, oracle, c, data, w, h, kw, frames=1)
        assert st.shadow_segments == shadow and st.segments == seg
        out.append(ga)
        c.close()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    assert np.array_equal(out[0].view(np.uint32), oa.view(np.uint32))
