"""CPU checks of the oracle itself: its LBVH against brute force, the
watertight test on adversarial rays, LBVH invariants and render
properties (no GPU)."""
import numpy as np
import pytest

from helpers import S, axis_rays, edge_rays, empty_scene, hits_equal, random_rays, single_triangle, solrt


@pytest.fixture(scope="module")
def cornell(oracle):
    return oracle.OracleScene(S.cornell())


@pytest.fixture(scope="module")
def soup(oracle):
    return oracle.OracleScene(S.soup(30000, seed=2))


def test_bvh_matches_brute_force_cornell(cornell):
    rays = random_rays(20000, 0.02, 0.98, seed=1)
    a, _ = cornell.trace(rays, brute=True)
    b, _ = cornell.trace(rays)
    assert hits_equal(a, b)
    assert (a["prim"] != solrt.NO_HIT).mean() > 0.7


def test_bvh_matches_brute_force_soup_edges(soup):
    rays = np.concatenate([random_rays(5000, 0.0, 1.0, seed=2), edge_rays(soup.data, 5000, seed=3),
                           axis_rays(0.0, 1.0, 3000, seed=4)])
    a, fba = soup.trace(rays, brute=True)
    b, fbb = soup.trace(rays)
    assert hits_equal(a, b)


def test_bvh_matches_brute_force_in_plane_rays(oracle):
    """Rays with a zero direction component lying exactly in box planes (the
    tunnel's angle-0 vertices have y = 0): 0 * inf in the slab test must not
    cull the box."""
    d = S.tunnel(n_ang=256, n_ax=128, length=25.0)
    o = oracle.OracleScene(d)
    rays = np.concatenate([edge_rays(d, 6000, seed=33, eye=(0.0, 0.0, 2.0)), axis_rays(-1.0, 1.0, 4000, seed=34)])
    a, _ = o.trace(rays, brute=True)
    b, _ = o.trace(rays)
    assert hits_equal(a, b)


def test_watertight_no_leak_on_shared_edges(oracle):
    """A closed cube (12 triangles, shared edges and vertices): every ray from
    inside must hit it, including rays through edges and vertices."""
    d = S.cornell()
    # close the box: add the front face (z = 0)
    b = S._Builder()
    m = b.add_material(S.material())
    b.add_quads([[(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)], [(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)],
                 [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)],
                 [(1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)], [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)]], m)
    cube = oracle.OracleScene(b.build())
    rng = np.random.default_rng(5)
    n = 4000
    rays = np.zeros(n, solrt.RAY_DTYPE)
    rays["origin"] = rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32)
    corners = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    tgt = corners[rng.integers(0, 8, n)]
    half = rng.integers(0, 2, n).astype(bool)
    # half the rays aim at edge midpoints between two corners sharing two coordinates
    tgt2 = tgt.copy()
    ax = rng.integers(0, 3, n)
    tgt2[np.arange(n), ax] = 0.5
    tgt = np.where(half[:, None], tgt2, tgt)
    rays["dir"] = (tgt - rays["origin"]).astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = 1e4
    h, _ = cube.trace(rays, brute=True)
    assert (h["prim"] != solrt.NO_HIT).all()
    h2, _ = cube.trace(rays)
    assert hits_equal(h, h2)


def test_lbvh_invariants(soup):
    child, boxes, order, morton = soup.bvh()
    n = soup.tri_count
    assert np.all(np.diff(morton.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(order), np.arange(n))
    leaves = child[child >= 0x80000000] & 0x7FFFFFFF
    assert np.array_equal(np.sort(leaves), np.arange(n))
    internal = child[child < 0x80000000]
    assert np.array_equal(np.sort(internal), np.arange(1, n - 1))
    # every internal child box lies within its parent box
    for i in range(0, n - 1, 97):
        for c in child[i]:
            if c < 0x80000000:
                assert np.all(boxes[c, :3] >= boxes[i, :3]) and np.all(boxes[c, 3:] <= boxes[i, 3:])


def test_empty_and_single_triangle(oracle):
    e = oracle.OracleScene(empty_scene())
    rays = random_rays(100, -1, 1, seed=6)
    h, _ = e.trace(rays)
    assert (h["prim"] == solrt.NO_HIT).all() and np.all(h["t"] == rays["tmax"])
    t = oracle.OracleScene(single_triangle())
    rays = np.zeros(3, solrt.RAY_DTYPE)
    rays["origin"] = [[0.2, 0.2, -1], [0.9, 0.9, -1], [0.2, 0.2, 1]]
    rays["dir"] = [[0, 0, 1], [0, 0, 1], [0, 0, 1]]
    rays["tmax"] = 1e4
    h, _ = t.trace(rays)
    assert h["prim"][0] == 0 and h["t"][0] == 1.0
    assert abs(h["u"][0] - 0.2) < 1e-6 and abs(h["v"][0] - 0.2) < 1e-6
    assert h["prim"][1] == solrt.NO_HIT and h["prim"][2] == solrt.NO_HIT


def test_tmin_tmax_respected(cornell):
    rays = random_rays(2000, 0.1, 0.9, seed=7)
    h, _ = cornell.trace(rays)
    hit = h["prim"] != solrt.NO_HIT
    rays2 = rays.copy()
    rays2["tmax"] = np.where(hit, h["t"] * 0.999, rays["tmax"])
    h2, _ = cornell.trace(rays2)
    assert np.all(h2["prim"][hit] != h["prim"][hit]) or np.all(h2["t"][hit] <= rays2["tmax"][hit])
    rays3 = rays.copy()
    rays3["tmin"] = np.where(hit, h["t"], 0)
    h3, _ = cornell.trace(rays3)
    assert np.all(h3["t"][hit & (h3["prim"] != solrt.NO_HIT)] > h["t"][hit & (h3["prim"] != solrt.NO_HIT)])


def test_camera_product_matches_oracle(oracle, solrt):
    for eye, ctr, up, fov, asp in [((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, -1, 0), 40.0, 1.0),
                                   ((10, 10, 10), (0, 0, 0), (0, -1, 0), 35.0, 16 / 9),
                                   ((0, 0, 2), (0, 0, 12), (0, -1, 0), 60.0, 2560 / 1440)]:
        a = solrt.camera_look_at(eye, ctr, up, fov, asp)
        b = oracle.camera_look_at(eye, ctr, up, fov, asp)
        for f in ("view", "view_inverse", "projection", "projection_inverse"):
            assert list(getattr(a, f)) == list(getattr(b, f))
    # glam look_at_rh / perspective_rh conventions
    c = solrt.camera_look_at((0, 0, 5), (0, 0, 0), (0, 1, 0), 90.0, 1.0, 0.1, 100.0)
    V = np.array(c.view, np.float64).reshape(4, 4).T
    assert np.allclose(V @ [0, 0, 0, 1], [0, 0, -5, 1])
    P = np.array(c.projection, np.float64).reshape(4, 4).T
    assert abs(P[0, 0] - 1.0) < 1e-6 and P[3, 2] == -1.0 and abs(P[2, 2] - 100.0 / (0.1 - 100.0)) < 1e-6


def _params(w, h, spp, **kw):
    base = dict(max_bounces=5, material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=1)
    base.update(kw)
    return solrt.render_params(w, h, spp=spp, **base)


def test_render_progressive_mix_equals_mean(oracle, solrt):
    """Two launches of 4 spp mixed with alpha 1 and 1/2 equal the mean of
    the two launches (pathtrace.rgen:89-92)."""
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    a0, _, _ = sc.render(cam, _params(32, 32, 4, frame=0))
    f0 = a0.copy()
    acc = a0.copy()
    sc.render(cam, _params(32, 32, 4, frame=1), accum=acc)
    a1, _, _ = sc.render(cam, _params(32, 32, 4, frame=1, accum_start_frame=1))
    assert np.allclose(acc[..., :3], 0.5 * (f0[..., :3] + a1[..., :3]), rtol=1e-5, atol=1e-6)


def test_render_kahan_equals_mix_mean(oracle, solrt):
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    a, _, _ = sc.render(cam, _params(32, 32, 8))
    k, _, _ = sc.render(cam, _params(32, 32, 8, accum_mode=solrt.ACCUM_KAHAN))
    assert np.allclose(a, k, rtol=1e-5, atol=1e-6)


def test_render_fp32_vs_fp64_close(oracle, solrt):
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    a32, _, s32 = sc.render(cam, _params(32, 32, 16))
    a64, _, s64 = sc.render(cam, _params(32, 32, 16), precision=64)
    rmse = float(np.sqrt(np.mean((a32[..., :3] - a64[..., :3]) ** 2)))
    assert rmse < 0.05
    assert abs(int(s32.segments) - int(s64.segments)) < 0.01 * s32.segments


def test_ref_stream_matches_sequential_samples(oracle, solrt):
    """REF_STREAM: sample s+1 continues the RNG where sample s stopped; the
    per-sample radiance export and the accumulated image agree."""
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    p = _params(16, 16, 4, rng_mode=solrt.RNG_REF_STREAM, material_mode=solrt.MATERIAL_REF)
    samples = sc.render_samples(cam, p)
    acc, _, _ = sc.render(cam, p)
    s = np.zeros((256, 3), np.float32)
    for k in range(4):
        s = s + samples[:, k, :3]
    mean = np.float32(1.0 / 4) * s
    assert np.array_equal(mean.reshape(16, 16, 3), acc[..., :3])


def test_debug_integrator_properties(oracle, solrt):
    """debug.rgen/.rchit/.rmiss: hits give barycentrics that sum to 1 and
    agree with the ray-file trace of the same pixel-centre rays; misses give
    the ray direction."""
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    p = _params(24, 24, 1, integrator=solrt.INTEGRATOR_DEBUG)
    acc, rgba8, st = sc.render(cam, p)
    assert st.segments == 24 * 24
    assert (acc[..., 3] == 0).all() and (rgba8[..., 3] == 0).all()
    bary = acc[..., :3]
    hit = np.abs(bary.sum(-1) - 1.0) < 1e-6
    assert hit.mean() > 0.9                       # the box fills the view
    assert (bary[hit] >= -1e-6).all()
    e = oracle.OracleScene(empty_scene())
    acc_e, _, _ = e.render(cam, p)
    dirs = acc_e[..., :3]
    assert np.allclose(np.linalg.norm(dirs, axis=-1), 1.0, atol=1e-5)


def test_ao_integrator_properties(oracle, solrt):
    """ao.rgen: an empty scene is fully open (1.0); inside the closed-top
    Cornell box occlusion darkens every pixel that sees a wall; the running
    mix of two frames equals their mean."""
    noise = np.random.default_rng(3).integers(0, 256, (32, 32, 4), dtype=np.uint8)
    d = S.cornell()
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    p0 = _params(16, 16, 4, max_bounces=4, integrator=solrt.INTEGRATOR_AO)
    e, _, _ = oracle.OracleScene(empty_scene()).render(cam, p0, blue_noise=noise)
    assert (e[..., :3] == 1.0).all()
    sc = oracle.OracleScene(d)
    a0, _, st = sc.render(cam, p0, blue_noise=noise)
    assert 0.0 < a0[..., :3].mean() < 1.0 and st.paths == 16 * 16 * 4
    acc = a0.copy()
    sc.render(cam, _params(16, 16, 4, max_bounces=4, frame=1, integrator=solrt.INTEGRATOR_AO), accum=acc,
              blue_noise=noise)
    a1, _, _ = sc.render(cam, _params(16, 16, 4, max_bounces=4, frame=1, accum_start_frame=1,
                                      integrator=solrt.INTEGRATOR_AO), blue_noise=noise)
    assert np.allclose(acc[..., :3], 0.5 * (a0[..., :3] + a1[..., :3]), rtol=1e-5, atol=1e-6)
    with pytest.raises(ValueError):
        sc.render(cam, p0)                        # no texture


def test_two_level_oracle(oracle):
    """Two-level mode: with identity instances every ray meets the same
    triangle at the same t as in the flattened scene (object space = world
    space); with transformed sections the same triangles are hit, at t
    within rounding of the flattened ones."""
    from helpers import transformed_cornell
    d = S.cornell()
    rays = np.concatenate([random_rays(20000, 0.01, 0.99, seed=81), edge_rays(d, 5000, seed=82)])
    flat, _ = oracle.OracleScene(d).trace(rays, brute=True)
    two, _ = oracle.OracleScene(d, two_level=True).trace(rays, brute=True)
    assert hits_equal(flat, two)
    d = transformed_cornell()
    o = oracle.OracleScene(d)
    tw, _ = o.world()
    lo, hi = tw[..., 0, :3].reshape(-1, 3).min(0), tw[..., 0, :3].reshape(-1, 3).max(0)
    rays = random_rays(20000, 0.0, 1.0, seed=83)
    rays["origin"] = (lo + (hi - lo) * rays["origin"]).astype(np.float32)
    flat, _ = o.trace(rays, brute=True)
    two, _ = oracle.OracleScene(d, two_level=True).trace(rays, brute=True)
    same = flat["prim"] == two["prim"]
    assert same.mean() > 0.995
    hit = same & (flat["prim"] != solrt.NO_HIT)
    assert np.allclose(flat["t"][hit], two["t"][hit], rtol=1e-4, atol=1e-5)


def test_nee_estimator_converges(oracle, solrt):
    """The oracle's next-event estimator (SOLRT_INTEGRATOR_PATH_NEE) has the
    expectation of pathtrace.rchit's estimator with Lambert materials: image
    means within 2 %, and far less noise at equal spp (median per-pixel
    difference between two seeds)."""
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    ref, _, s_ref = sc.render(cam, _params(32, 32, 2048, max_bounces=4, seed=1))
    nee, _, s_nee = sc.render(cam, _params(32, 32, 256, max_bounces=4, seed=2,
                                           integrator=solrt.INTEGRATOR_PATH_NEE))
    assert s_ref.shadow_segments == 0 and s_nee.shadow_segments > 0
    assert 0 < s_nee.shadow_unoccluded <= s_nee.shadow_segments
    assert abs(nee[..., :3].mean() - ref[..., :3].mean()) < 0.02 * ref[..., :3].mean()
    n2, _, _ = sc.render(cam, _params(32, 32, 256, max_bounces=4, seed=3, integrator=solrt.INTEGRATOR_PATH_NEE))
    n3, _, _ = sc.render(cam, _params(32, 32, 256, max_bounces=4, seed=4, integrator=solrt.INTEGRATOR_PATH_NEE))
    p2, _, _ = sc.render(cam, _params(32, 32, 256, max_bounces=4, seed=3))
    p3, _, _ = sc.render(cam, _params(32, 32, 256, max_bounces=4, seed=4))
    assert np.median(np.abs(n2 - n3)[..., :3]) < 0.3 * np.median(np.abs(p2 - p3)[..., :3])


def test_nee_needs_lambert(oracle, solrt):
    d = S.cornell()
    sc = oracle.OracleScene(d)
    cam = oracle.camera_look_at(d.camera["eye"], d.camera["center"], d.camera["up"], d.camera["vfov"], 1.0)
    with pytest.raises(ValueError):
        sc.render(cam, _params(8, 8, 1, material_mode=solrt.MATERIAL_REF, integrator=solrt.INTEGRATOR_PATH_NEE))
