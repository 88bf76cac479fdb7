"""Rendering scenes read from glTF: a Cornell box written as .glb with
translation-rotation-scale node transforms and a camera node renders bit for
bit like the oracle on the same loaded arrays, and a glTF of the plain
Cornell box renders exactly like the directly built scene."""
import numpy as np
import pytest

from helpers import S, bvh_kind, camera_of

pytestmark = pytest.mark.gpu


def _transformed_glb(solrt, path):
    d = S.cornell(light=(15.0, 15.0, 15.0))
    th = np.radians(20.0)
    nodes = []
    for i in range(len(d.sections)):
        if i % 2:
            nodes.append({"translation": [0.02 * i, -0.01, 0.03], "rotation": [0.0, np.sin(th / 2), 0.0, np.cos(th / 2)],
                          "scale": [1.0, 1.0 + 0.01 * i, 1.0]})
        else:
            nodes.append({})
    view = np.array(solrt.camera_look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, -1, 0), 40.0, 1.0).view)
    S.write_gltf(d, str(path), view=view, yfov=40.0, znear=0.1, zfar=100.0, node_transforms=nodes)
    return solrt.load_scene(str(path))


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
def test_gltf_render_matches_oracle(solrt, oracle, ctx, tmp_path, bvh):
    g = _transformed_glb(solrt, tmp_path / "cornell.glb")
    w, h = 40, 32
    cam = g.camera(w / h)
    kind = bvh_kind(solrt, bvh)
    sc = solrt.SceneDescription(ctx, g.data, bvh=kind)
    img = solrt.Image(ctx, w, h)
    p = solrt.render_params(w, h, spp=3, max_bounces=6, material_mode=solrt.MATERIAL_REF,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=11, miss_mode=solrt.MISS_REF_SKY)
    ctx.reset_stats()
    solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
    ga, _ = img.read()
    oa, _, st = oracle.OracleScene(g.data, two_level=kind == solrt.BVH2_TWO_LEVEL).render(cam, p)
    assert np.array_equal(ga.view(np.uint32), oa.view(np.uint32))
    assert ctx.stats().segments == st.segments and ctx.stats().error_flags == 0
    assert ga[..., :3].mean() > 0


def test_gltf_equals_direct_scene(solrt, ctx, tmp_path):
    d = S.cornell()
    S.write_gltf(d, str(tmp_path / "plain.gltf"), index_type="u16")
    g = solrt.load_scene(str(tmp_path / "plain.gltf"))
    w, h = 32, 32
    cam = camera_of(d, 1.0)
    p = solrt.render_params(w, h, spp=2, max_bounces=5, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=3)
    out = []
    for data in (d, g.data):
        sc = solrt.SceneDescription(ctx, data)
        img = solrt.Image(ctx, w, h)
        solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
        out.append(img.read()[0])
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


@pytest.mark.parametrize("integrator", ["path", "ao", "debug"])
def test_render_cli_on_gltf(solrt, ctx, tmp_path, integrator):
    """The headless example command on a written .glb: its PNG equals the
    RGBA8 image of the same launches made through the Python API."""
    import importlib
    render = importlib.import_module("sol-rs_gb300.render")
    g = _transformed_glb(solrt, tmp_path / "cornell.glb")
    out = tmp_path / "out.png"
    args = ["--model", str(tmp_path / "cornell.glb"), "--width", "32", "--height", "24", "--frames", "2",
            "--integrator", integrator, "--out", str(out)]
    if integrator == "path":
        args += ["--sky", "--bounces", "6"]
    assert render.main(args) == 0
    png = solrt.imageio.read_png(str(out))
    cam = g.camera(32 / 24)
    if integrator == "ao":
        ctx.set_blue_noise(render.load_blue_noise(None))
    sc = solrt.SceneDescription(ctx, g.data)
    img = solrt.Image(ctx, 32, 24)
    integ = {"path": solrt.INTEGRATOR_PATH, "ao": solrt.INTEGRATOR_AO, "debug": solrt.INTEGRATOR_DEBUG}[integrator]
    spp, bounces = {"path": (8, 6), "ao": (4, 4), "debug": (1, 1)}[integrator]
    for f in range(1 if integrator == "debug" else 2):
        p = solrt.render_params(32, 24, spp=spp, max_bounces=bounces, frame=f, integrator=integ,
                                miss_mode=solrt.MISS_REF_SKY if integrator == "path" else solrt.MISS_BLACK)
        solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
    _, rgba8 = img.read()
    if integrator == "debug":
        rgba8 = rgba8.copy()
        rgba8[..., 3] = 0
        png = png.copy()
        png[..., 3] = 0
    assert np.array_equal(png, rgba8)
