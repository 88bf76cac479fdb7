"""Radiance parity on identical RNG streams: the wavefront CUDA renderer
against the oracle's sequential per-pixel evaluation of pathtrace.rgen /
.rchit / .rmiss. The RGBA32F accumulation image must match bit for bit; the
RGBA8 image within 1 (gamma uses powf on the device, the C library's pow on
the host); the count of traced segments must be equal."""
import numpy as np
import pytest

from helpers import S, bvh_kind, camera_of, transformed_cornell

pytestmark = pytest.mark.gpu


def cornell_ref_materials():
    """Cornell box with cornell.gltf-like materials: a mirror tall box
    (metallic 1, roughness 0), glossy walls (roughness 0.89), light 15."""
    d = S.cornell(light=(15.0, 15.0, 15.0))
    d.materials["roughness"] = 0.8945907
    d.materials["metallic"][1] = 0.0
    # tall box is the last section; give it its own mirror material
    mats = list(d.materials)
    mats.append(S.material(base=(0.72, 0.72, 0.72), metallic=0.9999999776, roughness=0.0))
    d.materials = np.array(mats, S.MATERIAL_DTYPE)
    d.sections["material_index"][-1] = len(mats) - 1
    return d


def _case(name):
    A = importlib_solrt()
    if name == "cornell_lambert":
        return S.cornell(), 64, 64, dict(spp=4, max_bounces=5, material_mode=A.MATERIAL_LAMBERT,
                                         rng_mode=A.RNG_PER_SAMPLE, seed=1)
    if name == "cornell_ref_stream":
        return cornell_ref_materials(), 48, 40, dict(spp=3, max_bounces=32, material_mode=A.MATERIAL_REF,
                                                     rng_mode=A.RNG_REF_STREAM)
    if name == "cornell_ref_sky":
        return cornell_ref_materials(), 40, 32, dict(spp=2, max_bounces=8, material_mode=A.MATERIAL_REF,
                                                     rng_mode=A.RNG_PER_SAMPLE, miss_mode=A.MISS_REF_SKY)
    if name == "transformed":
        return transformed_cornell(), 32, 32, dict(spp=2, max_bounces=5, material_mode=A.MATERIAL_REF,
                                                   rng_mode=A.RNG_PER_SAMPLE, seed=7)
    if name == "soup_gradient":
        return S.soup(30000, seed=2), 64, 36, dict(spp=2, max_bounces=4, material_mode=A.MATERIAL_LAMBERT,
                                                   rng_mode=A.RNG_PER_SAMPLE, seed=2, miss_mode=A.MISS_GRADIENT)
    if name == "tunnel_kahan":
        return S.tunnel(n_ang=256, n_ax=128, length=25.0), 64, 36, dict(
            spp=2, max_bounces=8, material_mode=A.MATERIAL_LAMBERT, rng_mode=A.RNG_PER_SAMPLE, seed=3,
            miss_mode=A.MISS_REF_SKY, accum_mode=A.ACCUM_KAHAN)
    raise KeyError(name)


def importlib_solrt():
    import importlib
    return importlib.import_module("sol-rs_gb300")


def _render_both(solrt, oracle, ctx, data, w, h, kw, frames=2, bvh=None, sah=False):
    bvh = solrt.BVH2 if bvh is None else bvh
    cam = camera_of(data, w / h)
    sc = solrt.SceneDescription(ctx, data, bvh=bvh, sah=sah)
    mode = kw.get("accum_mode", solrt.ACCUM_REF_MIX)
    img = solrt.Image(ctx, w, h, mode)
    r = solrt.Renderer(ctx)
    o = oracle.OracleScene(data, two_level=bvh == solrt.BVH2_TWO_LEVEL)
    acc = np.zeros((h, w, 4), np.float32)
    ks = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    kc = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    seg_o = 0
    ctx.reset_stats()
    for f in range(frames):
        p = solrt.render_params(w, h, frame=f, **kw)
        r.cmd_trace_rays(sc, cam, p, img)
        acc, rgba_o, st = o.render(cam, p, accum=acc, ksum=ks, kcomp=kc)
        seg_o += st.segments
    ctx.synchronize()
    ga, g8 = img.read()
    stats = ctx.stats()
    return ga, g8, acc, rgba_o, stats, seg_o


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
@pytest.mark.parametrize("name", ["cornell_lambert", "cornell_ref_stream", "cornell_ref_sky", "transformed",
                                  "soup_gradient", "tunnel_kahan"])
def test_render_bit_exact(solrt, oracle, ctx, name, bvh):
    data, w, h, kw = _case(name)
    kind = bvh_kind(solrt, bvh)
    ga, g8, oa, o8, stats, seg_o = _render_both(solrt, oracle, ctx, data, w, h, kw, bvh=kind)
    diff = np.nonzero(np.any(ga.view(np.uint32) != oa.view(np.uint32), axis=-1))
    assert len(diff[0]) == 0, (len(diff[0]), list(zip(diff[0][:5], diff[1][:5])), ga[diff][:3], oa[diff][:3])
    assert np.max(np.abs(g8.astype(int) - o8.astype(int))) <= 1
    assert stats.segments == seg_o
    assert stats.error_flags == 0
    assert np.isfinite(ga).all() and ga[..., :3].mean() > 0


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8"])
@pytest.mark.parametrize("name", ["cornell_ref_sky", "soup_gradient", "tunnel_kahan", "transformed"])
def test_render_bit_exact_sah_collapse(solrt, oracle, ctx, name, bvh):
    """Wide BVHs collapsed by SAH, and binary BVHs restructured by treelets,
    render the oracle's image too."""
    data, w, h, kw = _case(name)
    ga, g8, oa, o8, stats, seg_o = _render_both(solrt, oracle, ctx, data, w, h, kw, bvh=bvh_kind(solrt, bvh), sah=True)
    assert np.array_equal(ga.view(np.uint32), oa.view(np.uint32))
    assert stats.segments == seg_o and stats.error_flags == 0


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
@pytest.mark.parametrize("name", ["cornell_lambert", "cornell_ref_stream", "soup_gradient", "tunnel_kahan"])
def test_megakernel_equals_wavefront(solrt, oracle, ctx, name, bvh):
    """The per-pixel megakernel (the reference's loop structure) renders the
    same image as the wavefront and as the oracle."""
    data, w, h, kw = _case(name)
    kind = bvh_kind(solrt, bvh)
    ga, g8, oa, o8, stats, seg_o = _render_both(solrt, oracle, ctx, data, w, h, dict(kw, kernel=solrt.api.KERNEL_MEGA),
                                                bvh=kind)
    assert np.array_equal(ga.view(np.uint32), oa.view(np.uint32))
    assert stats.segments == seg_o and stats.error_flags == 0


@pytest.mark.parametrize("name", ["cornell_lambert", "soup_gradient", "tunnel_kahan"])
def test_visit_counters_vs_oracle(solrt, oracle, name):
    """The device counters of node visits and triangle tests (the N_node and
    N_tri of the roofline's algorithmic bytes) against the oracle's CPU
    traversal of the same binary LBVH on the same paths: the warp-organised
    kernel visits what the per-ray loop visits, plus the speculative visits
    of lanes that hold a leaf (and widened boxes), within a few percent."""
    data, w, h, kw = _case(name)
    c = solrt.Context(0, enable_counters=True)
    sc = solrt.SceneDescription(c, data, bvh=solrt.BVH2)
    cam = camera_of(data, w / h)
    mode = kw.get("accum_mode", solrt.ACCUM_REF_MIX)
    img = solrt.Image(c, w, h, mode)
    o = oracle.OracleScene(data)
    acc = np.zeros((h, w, 4), np.float32)
    ks = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    kc = np.zeros((h, w, 4), np.float32) if mode == solrt.ACCUM_KAHAN else None
    seg = nv = nt = 0
    c.reset_stats()
    for f in range(2):
        p = solrt.render_params(w, h, frame=f, **kw)
        solrt.Renderer(c).cmd_trace_rays(sc, cam, p, img)
        acc, _, st = o.render(cam, p, accum=acc, ksum=ks, kcomp=kc)
        seg += st.segments
        nv += st.node_visits
        nt += st.tri_tests
    c.synchronize()
    g = c.stats()
    assert g.segments == seg and g.error_flags == 0
    assert nv > 0 and nt > 0
    assert 0.999 * nv <= g.node_visits <= 1.10 * nv, (g.node_visits, nv)
    assert 0.999 * nt <= g.tri_tests <= 1.10 * nt, (g.tri_tests, nt)
    img.close()
    sc.close()
    c.close()


def test_pass_splitting_invariance(solrt, oracle):
    """A tiny path capacity forces many passes and pixel chunks; the image
    must not change."""
    data, w, h, kw = _case("cornell_lambert")
    kw = dict(kw, spp=5)
    out = []
    for cap in (0, 1000, 4096 + 7):
        c = solrt.Context(0, path_capacity=cap)
        ga, _, oa, _, _, _ = _render_both(solrt, oracle, c, data, w, h, kw, frames=1)
        out.append(ga)
        c.close()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    assert np.array_equal(out[0].view(np.uint32), oa.view(np.uint32))


def test_render_rejects_bad_params(solrt, ctx):
    data = S.cornell()
    sc = solrt.SceneDescription(ctx, data)
    img = solrt.Image(ctx, 16, 16)
    cam = camera_of(data, 1.0)
    r = solrt.Renderer(ctx)
    with pytest.raises(solrt.SolrtError):
        r.cmd_trace_rays(sc, cam, solrt.render_params(32, 16), img)
    with pytest.raises(solrt.SolrtError):
        r.cmd_trace_rays(sc, cam, solrt.render_params(16, 16, spp=0), img)
    with pytest.raises(solrt.SolrtError):
        r.cmd_trace_rays(sc, cam, solrt.render_params(16, 16, max_bounces=5000), img)
    with pytest.raises(solrt.SolrtError):
        r.cmd_trace_rays(sc, cam, solrt.render_params(16, 16, accum_mode=solrt.ACCUM_KAHAN), img)


def test_full_size_soup_properties(solrt, ctx):
    """1M-triangle soup at 1920x1080, 1 spp, depth 4: finite, deterministic
    across runs and pass splits, one primary segment per path."""
    data = S.soup(1_000_000, seed=2)
    sc = solrt.SceneDescription(ctx, data)
    cam = camera_of(data, 1920 / 1080)
    p = solrt.render_params(1920, 1080, spp=1, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=2, miss_mode=solrt.MISS_GRADIENT)
    r = solrt.Renderer(ctx)
    imgs = []
    for _ in range(2):
        img = solrt.Image(ctx, 1920, 1080)
        ctx.reset_stats()
        r.cmd_trace_rays(sc, cam, p, img)
        ctx.synchronize()
        imgs.append(img.read()[0])
        st = ctx.stats()
        assert st.paths == 1920 * 1080
        assert 1920 * 1080 <= st.segments <= 5 * 1920 * 1080
    assert np.array_equal(imgs[0], imgs[1])
    assert np.isfinite(imgs[0]).all()


@pytest.mark.parametrize("accum", ["mix", "kahan"])
def test_checkpoint_resume(solrt, ctx, accum):
    """Four frames rendered straight through equal two frames, a snapshot of
    the accumulation state restored into a fresh image, then frames 2 and 3
    (bit for bit, both accumulation modes)."""
    data = S.cornell()
    w, h = 32, 24
    mode = solrt.ACCUM_KAHAN if accum == "kahan" else solrt.ACCUM_REF_MIX
    cam = camera_of(data, w / h)
    sc = solrt.SceneDescription(ctx, data)
    r = solrt.Renderer(ctx)

    def params(f):
        return solrt.render_params(w, h, spp=2, max_bounces=4, frame=f, material_mode=solrt.MATERIAL_LAMBERT,
                                   rng_mode=solrt.RNG_PER_SAMPLE, seed=4, accum_mode=mode)
    straight = solrt.Image(ctx, w, h, mode)
    for f in range(4):
        r.cmd_trace_rays(sc, cam, params(f), straight)
    a_ref, b_ref = straight.read()
    first = solrt.Image(ctx, w, h, mode)
    for f in range(2):
        r.cmd_trace_rays(sc, cam, params(f), first)
    snap = first.snapshot()
    resumed = solrt.Image(ctx, w, h, mode)
    resumed.restore(snap)
    for f in range(2, 4):
        r.cmd_trace_rays(sc, cam, params(f), resumed)
    a, b = resumed.read()
    assert np.array_equal(a.view(np.uint32), a_ref.view(np.uint32))
    assert np.array_equal(b, b_ref)


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2t", "bvh8"])
def test_gpu_equals_reference_pipeline_fixture(solrt, ctx, bvh):
    """The device against the committed image of the reference's own
    pathtrace.rgen / .rchit / .rmiss compiled as C++ (tests/golden/
    ref_pathtrace_cornell.npz): Cornell box, 32 x 24, sky, REF materials,
    the reference's per-pixel stream, 8 spp, 32 bounces, two launches
    accumulated; bit for bit."""
    import os
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_pathtrace_cornell.npz"))
    d = S.cornell()
    w, h = 32, 24
    cam = camera_of(d, w / h)
    sc = solrt.SceneDescription(ctx, d, bvh=bvh_kind(solrt, bvh))
    img = solrt.Image(ctx, w, h)
    r = solrt.Renderer(ctx)
    for f in range(2):
        p = solrt.render_params(w, h, spp=8, max_bounces=32, frame=f, material_mode=solrt.MATERIAL_REF,
                                rng_mode=solrt.RNG_REF_STREAM, miss_mode=solrt.MISS_REF_SKY)
        r.cmd_trace_rays(sc, cam, p, img)
        a32, a8 = img.read()
        assert np.array_equal(a32.view(np.uint32), fx["accum%d" % f].view(np.uint32)), f
        assert np.max(np.abs(a8.astype(int) - fx["rgba8_%d" % f].astype(int))) <= 1, f
