"""Per-frame instance transforms (blas_transform(s) + tlas_regenerate,
src/ray/mod.rs:162-181): a dynamic scene moved on the device renders and
traces exactly like a scene created from scratch with the same instances,
whether the BVH is rebuilt (identical nodes) or refitted (different boxes,
same closest hits), and like the oracle."""
import numpy as np
import pytest

from helpers import S, bvh_args, camera_of, hits_equal, random_rays

pytestmark = pytest.mark.gpu


def _rot_y(deg, t=(0, 0, 0), s=(1, 1, 1)):
    a = np.radians(deg)
    M = np.eye(4)
    M[:3, :3] = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]) * np.asarray(s)[None, :]
    M[:3, 3] = t
    return M


def _frames(nsec):
    out = []
    for f in range(3):
        out.append([_rot_y(7.0 * f + 3 * i, (0.01 * f, -0.02 * (i % 3), 0.015 * i), (1.0, 1.0 + 0.05 * f, 1.0))
                    if (i + f) % 2 else np.eye(4) for i in range(nsec)])
    return out


def _with_instances(solrt, data, transforms):
    d = S.SceneData(data.vertices, data.indices, data.sections, data.materials,
                    np.array([solrt.instance_from_transform(t, i) for i, t in enumerate(transforms)]),
                    data.camera, data.name)
    return d


def _render(solrt, ctx, sc, cam, w, h, p):
    img = solrt.Image(ctx, w, h)
    solrt.Renderer(ctx).cmd_trace_rays(sc, cam, p, img)
    return img.read()[0]


@pytest.mark.parametrize("integ", ["path", "nee"])
@pytest.mark.parametrize("mode", ["rebuild", "refit"])
@pytest.mark.parametrize("bvh", ["bvh2", "bvh2s", "bvh2q", "bvh2t", "bvh2ts", "bvh4", "bvh8", "bvh8f"])
def test_regenerate_matches_fresh_scene(solrt, oracle, ctx, bvh, mode, integ):
    """nee: the light tree of next-event estimation is rebuilt from the moved
    vertices, as a fresh scene builds it (the light section moves too).
    bvh2s / bvh2ts: the treelet restructuring (of the whole tree, or of each
    BLAS) gives a rebuilt dynamic scene the fresh scene's bytes too."""
    args = bvh_args(solrt, bvh)
    kind = args["bvh"]
    regen = solrt.REGEN_REBUILD if mode == "rebuild" else solrt.REGEN_REFIT
    base = S.cornell()
    w, h = 32, 32
    cam = camera_of(base, 1.0)
    p = solrt.render_params(w, h, spp=2, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=9,
                            integrator=solrt.INTEGRATOR_PATH_NEE if integ == "nee" else solrt.INTEGRATOR_PATH)
    dyn = solrt.SceneDescription(ctx, base, dynamic=True, **args)
    rays = random_rays(4000, -0.2, 1.2, seed=21)
    for f, transforms in enumerate(_frames(len(base.sections))):
        dyn.blas_transforms(transforms)
        dyn.tlas_regenerate(regen)
        moved = _with_instances(solrt, base, transforms)
        fresh = solrt.SceneDescription(ctx, moved, **args)
        a = _render(solrt, ctx, dyn, cam, w, h, p)
        b = _render(solrt, ctx, fresh, cam, w, h, p)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f
        assert hits_equal(dyn.trace_rays(rays), fresh.trace_rays(rays))
        if mode == "rebuild":
            na, ta = dyn.bvh_export()
            nb, tb = fresh.bvh_export()
            assert np.array_equal(na, nb) and np.array_equal(ta, tb)
        if f == 2:
            oa, _, _ = oracle.OracleScene(moved, two_level=kind == solrt.BVH2_TWO_LEVEL).render(cam, p)
            assert np.array_equal(a.view(np.uint32), oa.view(np.uint32))
        fresh.close()
    assert ctx.stats().error_flags == 0


def test_refit_soup_tracks_motion(solrt, ctx):
    """A 20k-triangle section rotated by 25 degrees: the refitted BVH (boxes
    grow, topology stays) still finds exactly the fresh scene's hits."""
    base = S.soup(20000, seed=5)
    dyn = solrt.SceneDescription(ctx, base, dynamic=True)
    T = _rot_y(25.0, (0.5, 0.0, 0.5)) @ _rot_y(0.0, (-0.5, 0.0, -0.5))
    dyn.blas_transforms([T])
    dyn.tlas_regenerate(solrt.REGEN_REFIT)
    fresh = solrt.SceneDescription(ctx, _with_instances(solrt, base, [T]))
    rays = random_rays(20000, -0.3, 1.3, seed=22)
    assert hits_equal(dyn.trace_rays(rays), fresh.trace_rays(rays))


def test_static_scene_rejects_instances(solrt, ctx):
    sc = solrt.SceneDescription(ctx, S.cornell())
    with pytest.raises(solrt.SolrtError, match="DYNAMIC"):
        sc.set_instances(np.zeros(len(S.cornell().sections), S.INSTANCE_DTYPE))
    dyn = solrt.SceneDescription(ctx, S.cornell(), dynamic=True)
    with pytest.raises(solrt.SolrtError, match="section count"):
        dyn.set_instances(np.zeros(3, S.INSTANCE_DTYPE))
