"""Batched rendering: jobs of different scenes, sizes, spp, bounce limits and
modes share wavefront passes; every job's image must equal (bit for bit)
the image of the same job rendered alone with solrt_render, with and
without CUDA-graph replay, and with a tiny path capacity that forces many
mixed passes. Alone-vs-mixed invariance is the serving property of the
batched path."""
import numpy as np
import pytest

from helpers import S, bvh_kind, camera_of, empty_scene, single_triangle, transformed_cornell

pytestmark = pytest.mark.gpu


def _specs(solrt):
    L, R = solrt.MATERIAL_LAMBERT, solrt.MATERIAL_REF
    PS, RS = solrt.RNG_PER_SAMPLE, solrt.RNG_REF_STREAM
    return [
        (S.cornell(), 48, 40, dict(spp=3, max_bounces=5, material_mode=L, rng_mode=PS, seed=1, job_id=0)),
        (S.cornell(light=(15, 15, 15)), 32, 32, dict(spp=2, max_bounces=32, material_mode=R, rng_mode=RS)),
        (S.soup(20000, seed=2), 64, 36, dict(spp=5, max_bounces=4, material_mode=L, rng_mode=PS, seed=2, job_id=2,
                                             miss_mode=solrt.MISS_GRADIENT)),
        (S.tunnel(n_ang=128, n_ax=64, length=20.0), 40, 24, dict(spp=2, max_bounces=8, material_mode=L, rng_mode=PS,
                                                                 seed=3, job_id=3, miss_mode=solrt.MISS_REF_SKY,
                                                                 accum_mode=solrt.ACCUM_KAHAN)),
        (transformed_cornell(), 24, 24, dict(spp=7, max_bounces=3, material_mode=R, rng_mode=PS, seed=5, job_id=4,
                                             miss_mode=solrt.MISS_REF_SKY)),
        (single_triangle(), 16, 16, dict(spp=1, max_bounces=2, material_mode=L, rng_mode=PS, seed=6, job_id=5)),
        (empty_scene(), 8, 8, dict(spp=2, max_bounces=1, material_mode=L, rng_mode=PS, seed=7, job_id=6,
                                   miss_mode=solrt.MISS_GRADIENT)),
        # next-event estimation jobs share passes (and shadow queues) with the rest
        (S.cornell(), 32, 24, dict(spp=3, max_bounces=4, material_mode=L, rng_mode=PS, seed=8, job_id=7,
                                   integrator=solrt.INTEGRATOR_PATH_NEE)),
        (S.tunnel(n_ang=128, n_ax=64, length=20.0), 24, 16, dict(spp=2, max_bounces=6, material_mode=L,
                                                                 rng_mode=RS, miss_mode=solrt.MISS_REF_SKY,
                                                                 accum_mode=solrt.ACCUM_KAHAN,
                                                                 integrator=solrt.INTEGRATOR_PATH_NEE)),
    ]


def _make(solrt, ctx, bvh, frame=0):
    out = []
    for data, w, h, kw in _specs(solrt):
        sc = solrt.SceneDescription(ctx, data, bvh=bvh)
        img = solrt.Image(ctx, w, h, kw.get("accum_mode", solrt.ACCUM_REF_MIX))
        out.append((sc, img, camera_of(data, w / h), solrt.render_params(w, h, frame=frame, **kw)))
    return out


def _alone(solrt, ctx, jobs, frames=1):
    res = []
    r = solrt.Renderer(ctx)
    for sc, img, cam, p in jobs:
        solo = solrt.Image(ctx, p.width, p.height, p.accum_mode)
        for f in range(frames):
            q = solrt.RenderParams.from_buffer_copy(p)
            q.frame = f
            r.cmd_trace_rays(sc, cam, q, solo)
        ctx.synchronize()
        res.append(solo.read())
    return res


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
def test_batch_equals_alone(solrt, ctx, bvh, graph):
    kind = bvh_kind(solrt, bvh)
    jobs = _make(solrt, ctx, kind)
    batch = solrt.Batch(ctx, jobs, graph=graph)
    ctx.reset_stats()
    batch.launch()
    ctx.synchronize()
    assert ctx.stats().error_flags == 0
    if graph:   # second frame through the same plan (graph replay)
        upd = []
        for sc, img, cam, p in jobs:
            q = solrt.RenderParams.from_buffer_copy(p)
            q.frame = 1
            upd.append((sc, img, cam, q))
        batch.update(upd)
        batch.launch()
        ctx.synchronize()
    alone = _alone(solrt, ctx, jobs, frames=2 if graph else 1)
    for (sc, img, cam, p), (a32, a8) in zip(jobs, alone):
        b32, b8 = img.read()
        assert np.array_equal(b32.view(np.uint32), a32.view(np.uint32))
        assert np.array_equal(b8, a8)
    batch.close()


def test_batch_many_passes(solrt):
    """Capacity of 2000 paths: every pass mixes partial jobs; images still
    equal the unconstrained batch."""
    big = solrt.Context(0)
    small = solrt.Context(0, path_capacity=2000)
    res = []
    for c in (big, small):
        jobs = _make(solrt, c, solrt.BVH2)
        b = solrt.Batch(c, jobs)
        b.launch()
        c.synchronize()
        info = b.info()
        res.append(([img.read()[0] for _, img, _, _ in jobs], info))
        b.close()
    assert res[1][1]["passes"] > res[0][1]["passes"] >= 1
    for x, y in zip(res[0][0], res[1][0]):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    big.close()
    small.close()


def test_batch_matches_oracle(solrt, oracle, ctx):
    jobs = _make(solrt, ctx, solrt.BVH2)
    b = solrt.Batch(ctx, jobs)
    b.launch()
    ctx.synchronize()
    for (data, w, h, kw), (sc, img, cam, p) in [x for i, x in enumerate(zip(_specs(solrt), jobs)) if i in (0, 1, 2, 7)]:
        want, _, _ = oracle.OracleScene(data).render(cam, p)
        got, _ = img.read()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_batch_rejects_mixed_bvh_kinds(solrt, ctx):
    d = S.cornell()
    a = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2)
    b = solrt.SceneDescription(ctx, d, bvh=solrt.BVH8_Q8)
    ia, ib = solrt.Image(ctx, 8, 8), solrt.Image(ctx, 8, 8)
    cam = camera_of(d, 1.0)
    p = solrt.render_params(8, 8)
    with pytest.raises(solrt.SolrtError):
        solrt.Batch(ctx, [(a, ia, cam, p), (b, ib, cam, p)])


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
def test_autotune_keeps_images(solrt, bvh):
    """solrt_batch_autotune times every extend block size x shared stack
    depth and three pass sizes; the batch re-planned with the winner renders
    the same images as the default configuration, and the winner stays on
    the context."""
    kind = bvh_kind(solrt, bvh)
    c = solrt.Context(0, path_capacity=1 << 18)
    jobs = _make(solrt, c, kind)
    b = solrt.Batch(c, jobs, graph=True)
    b.launch()
    c.synchronize()
    want = [img.read()[0].copy() for _, img, _, _ in jobs]
    r = b.autotune()
    for _, img, _, _ in jobs:   # KAHAN images summed every tuning launch
        img.clear()
    assert r["candidates"] >= (5 if bvh in ("bvh8", "bvh8f") else 8)   # 8-wide: no shared stack
    assert r["block_size"] in (64, 128, 256) and r["smem_stack"] in (16, 32)
    assert r["best_ms"] > 0 and r["best_ms"] <= r["initial_ms"] * 1.05
    assert c.get_tune() == {k: r[k] for k in ("block_size", "smem_stack", "pass_paths")}
    b.launch()
    c.synchronize()
    for (_, img, _, _), w in zip(jobs, want):
        assert np.array_equal(img.read()[0].view(np.uint32), w.view(np.uint32))
    assert c.stats().error_flags == 0
    b.close()
    c.close()


def test_every_tune_config_renders_the_same(solrt):
    c = solrt.Context(0, path_capacity=1 << 18)
    jobs = _make(solrt, c, solrt.BVH2)
    ref = None
    for blk in (64, 128, 256):
        for sm in (16, 32):
            for pp in (0, 5000):
                c.set_tune(blk, sm, pp)
                for _, img, _, _ in jobs:
                    img.clear()
                b = solrt.Batch(c, jobs)
                b.launch()
                c.synchronize()
                got = [img.read()[0].copy() for _, img, _, _ in jobs]
                if ref is None:
                    ref = got
                for x, y in zip(ref, got):
                    assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (blk, sm, pp)
                b.close()
    with pytest.raises(solrt.SolrtError):
        c.set_tune(96, 32, 0)
    with pytest.raises(solrt.SolrtError):
        c.set_tune(128, 8, 0)
    with pytest.raises(solrt.SolrtError):
        c.set_tune(128, 32, 1 << 20)
    c.close()


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2t", "bvh8"])
def test_persistent_batch_equals_alone(solrt, ctx, bvh):
    """SOLRT_BATCH_PERSISTENT: all jobs in one persistent per-pixel launch
    (warps take pixels from a device work counter, each thread traces its
    pixel's samples to the end) render every job's image bit for bit as
    solrt_render of that job alone; two launches accumulate two frames."""
    kind = bvh_kind(solrt, bvh)
    jobs = [j for j, (_, _, _, kw) in zip(_make(solrt, ctx, kind), _specs(solrt))
            if kw.get("integrator", solrt.INTEGRATOR_PATH) == solrt.INTEGRATOR_PATH]
    batch = solrt.Batch(ctx, jobs, persistent=True)
    ctx.reset_stats()
    batch.launch()
    upd = []
    for sc, img, cam, p in jobs:
        q = solrt.RenderParams.from_buffer_copy(p)
        q.frame = 1
        upd.append((sc, img, cam, q))
    batch.update(upd)
    batch.launch()
    ctx.synchronize()
    st = ctx.stats()
    assert st.error_flags == 0 and st.launches <= 2 * 2
    got = [img.read() for _, img, _, _ in jobs]
    want = _alone(solrt, ctx, jobs, frames=2)
    for (a32, a8), (b32, b8) in zip(got, want):
        assert np.array_equal(a32.view(np.uint32), b32.view(np.uint32))
        assert np.array_equal(a8, b8)
    batch.close()


@pytest.mark.parametrize("bvh", ["bvh2", "bvh2t", "bvh8"])
def test_persistent_batch_with_nee_equals_alone(solrt, ctx, bvh):
    """A persistent per-pixel batch holding next-event-estimation jobs (each
    thread traces a vertex's shadow ray at once) renders every job as
    solrt_render of that job alone, with the same shadow-ray counts."""
    kind = bvh_kind(solrt, bvh)
    jobs = _make(solrt, ctx, kind)
    batch = solrt.Batch(ctx, jobs, persistent=True)
    ctx.reset_stats()
    batch.launch()
    ctx.synchronize()
    st = ctx.stats()
    assert st.error_flags == 0 and st.shadow_segments > 0
    got = [img.read() for _, img, _, _ in jobs]
    batch.close()
    ctx.reset_stats()
    want = _alone(solrt, ctx, jobs, frames=1)
    st2 = ctx.stats()
    assert (st.segments, st.shadow_segments, st.shadow_unoccluded) == (st2.segments, st2.shadow_segments,
                                                                         st2.shadow_unoccluded)
    for (a32, a8), (b32, b8) in zip(got, want):
        assert np.array_equal(a32.view(np.uint32), b32.view(np.uint32))
        assert np.array_equal(a8, b8)


def _plain_jobs(solrt, ctx, kind):
    return [j for j, (_, _, _, kw) in zip(_make(solrt, ctx, kind), _specs(solrt))
            if kw.get("integrator", solrt.INTEGRATOR_PATH) == solrt.INTEGRATOR_PATH]


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("bvh", ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
def test_cooperative_batch_equals_alone(solrt, ctx, bvh, graph):
    """SOLRT_BATCH_COOPERATIVE: every wavefront pass of the batch as phases
    of one cooperative launch (grid-wide barriers between generate, extend,
    shade, the shadow-ray phases of next-event estimation and accumulate)
    renders each job bit for bit as solrt_render of that job alone, over two
    frames, with and without a CUDA graph; one kernel launch per step."""
    kind = bvh_kind(solrt, bvh)
    jobs = _make(solrt, ctx, kind)   # next-event-estimation jobs included
    batch = solrt.Batch(ctx, jobs, graph=graph, cooperative=True)
    ctx.reset_stats()
    batch.launch()
    ctx.synchronize()
    st = ctx.stats()
    assert st.error_flags == 0 and st.launches == 1
    upd = []
    for sc, img, cam, p in jobs:
        q = solrt.RenderParams.from_buffer_copy(p)
        q.frame = 1
        upd.append((sc, img, cam, q))
    batch.update(upd)
    batch.launch()
    ctx.synchronize()
    assert ctx.stats().error_flags == 0
    got = [img.read() for _, img, _, _ in jobs]
    want = _alone(solrt, ctx, jobs, frames=2)
    for (a32, a8), (b32, b8) in zip(got, want):
        assert np.array_equal(a32.view(np.uint32), b32.view(np.uint32))
        assert np.array_equal(a8, b8)
    batch.close()


def test_cooperative_many_passes_and_counts(solrt):
    """A capacity of 2000 paths makes dozens of mixed passes inside the one
    launch; images and segment / path / shadow-ray counts equal the
    per-stage launches'."""
    res = []
    for coop in (False, True):
        c = solrt.Context(0, path_capacity=2000)
        jobs = _make(solrt, c, solrt.BVH2)
        b = solrt.Batch(c, jobs, cooperative=coop)
        c.reset_stats()
        b.launch()
        c.synchronize()
        st = c.stats()
        assert st.error_flags == 0
        res.append(([img.read()[0].copy() for _, img, _, _ in jobs], b.info(), st.segments, st.paths,
                    st.shadow_segments, st.shadow_unoccluded))
        b.close()
        c.close()
    assert res[0][1]["passes"] > 10 and res[0][1] == res[1][1]
    assert res[0][2:] == res[1][2:] and res[0][4] > 0
    for x, y in zip(res[0][0], res[1][0]):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_cooperative_batch_refusals(solrt, ctx):
    plain = _plain_jobs(solrt, ctx, solrt.BVH2)
    with pytest.raises(solrt.SolrtError):
        solrt.Batch(ctx, plain, persistent=True, cooperative=True)


def test_grid_barrier_wait_is_bounded(solrt, ctx):
    """The cooperative launch's barrier wait gives up after its budget: a
    grid whose block 0 never arrives ends with SOLRT_EFLAG_TIMEOUT raised by
    the waiting blocks (no hang, no fault), and the context keeps working."""
    import time
    flags = np.zeros(1, np.uint32)
    t0 = time.time()
    ctx.debug_unit(8, 0, fin=np.array([0.05], np.float32), out_u=flags)
    assert flags[0] & solrt.api.EFLAG_TIMEOUT
    assert time.time() - t0 < 30.0
    jobs = _plain_jobs(solrt, ctx, solrt.BVH2)[:1]
    b = solrt.Batch(ctx, jobs, cooperative=True)
    b.launch()
    ctx.synchronize()
    assert ctx.stats().error_flags == 0
    b.close()


def test_autotune_cache_miss_then_hit(solrt, tmp_path):
    """solrt_batch_autotune_cached: the first call times the candidates and
    stores the winner under the batch's key; a new batch of the same shape
    (other cameras) finds it, re-plans with it without timing, and renders
    the same images as the tuned batch."""
    path = str(tmp_path / "tune.jsonl")
    c = solrt.Context(0, path_capacity=1 << 18)
    jobs = _plain_jobs(solrt, c, solrt.BVH2)
    b = solrt.Batch(c, jobs, graph=True)
    r1 = b.autotune_cached(path)
    assert not r1["cache_hit"] and r1["candidates"] >= 8
    key = b.tune_key()
    assert key.startswith("gpu=") and "|kind=0|" in key
    assert solrt.api.tune_cache_lookup(path, key)["block_size"] == r1["block_size"]
    for _, img, _, _ in jobs:
        img.clear()
    b.launch()
    c.synchronize()
    want = [img.read()[0].copy() for _, img, _, _ in jobs]
    b.close()
    c.set_tune(128, 32, 0)
    b2 = solrt.Batch(c, jobs, graph=True)
    assert b2.tune_key() == key
    r2 = b2.autotune_cached(path)
    assert r2["cache_hit"] and r2["candidates"] == 0
    assert c.get_tune() == {k: r1[k] for k in ("block_size", "smem_stack", "pass_paths")}
    for _, img, _, _ in jobs:
        img.clear()
    b2.launch()
    c.synchronize()
    for (_, img, _, _), w in zip(jobs, want):
        assert img.read()[0].view(np.uint32).tobytes() == w.view(np.uint32).tobytes()
    b2.close()
    c.close()


def test_cooperative_autotune_tunes_the_pass_size_only(solrt):
    """A cooperative batch has one launch shape: the autotuner times only
    the pass sizes (at most 3 candidates besides the start) and the
    re-planned batch renders the same images."""
    c = solrt.Context(0, path_capacity=1 << 18)
    jobs = _plain_jobs(solrt, c, solrt.BVH2)
    b = solrt.Batch(c, jobs, graph=True, cooperative=True)
    b.launch()
    c.synchronize()
    want = [img.read()[0].copy() for _, img, _, _ in jobs]
    r = b.autotune()
    assert 1 <= r["candidates"] <= 4
    assert (r["block_size"], r["smem_stack"]) == (128, 32)
    for _, img, _, _ in jobs:
        img.clear()
    b.launch()
    c.synchronize()
    for (_, img, _, _), w in zip(jobs, want):
        assert np.array_equal(img.read()[0].view(np.uint32), w.view(np.uint32))
    b.close()
    c.close()
