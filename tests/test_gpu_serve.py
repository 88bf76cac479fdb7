"""Serving: jobs submitted while others run are admitted at tick
boundaries, advance together, and each result equals the same job rendered
alone (continuous batching must not change images). Admission by memory
budget, LRU eviction of completed results and the bounded wait are
exercised with small budgets."""
import time

import numpy as np
import pytest

from helpers import S, camera_of

pytestmark = pytest.mark.gpu


def _scenes(solrt, ctx):
    return [solrt.SceneDescription(ctx, S.cornell()), solrt.SceneDescription(ctx, S.soup(20000, seed=2)),
            solrt.SceneDescription(ctx, S.tunnel(n_ang=128, n_ax=64, length=20.0))]


def _job(solrt, i):
    rng = np.random.default_rng(100 + i)
    w = int(rng.choice([16, 24, 40]))
    h = int(rng.choice([16, 32]))
    kw = dict(spp=int(rng.integers(1, 9)), max_bounces=int(rng.integers(1, 6)), seed=7 + i, job_id=i,
              material_mode=solrt.MATERIAL_LAMBERT if i % 2 else solrt.MATERIAL_REF,
              rng_mode=solrt.RNG_PER_SAMPLE if i % 3 else solrt.RNG_REF_STREAM,
              miss_mode=int(i % 3), accum_mode=solrt.ACCUM_KAHAN if i % 4 == 1 else solrt.ACCUM_REF_MIX,
              integrator=solrt.INTEGRATOR_PATH_NEE if i % 4 == 3 else solrt.INTEGRATOR_PATH)
    return int(rng.integers(0, 3)), solrt.render_params(w, h, **kw)


@pytest.mark.parametrize("ticks", ["fixed", "adaptive"])
@pytest.mark.parametrize("policy", [0, 1])
def test_served_results_equal_alone(solrt, policy, ticks):
    ctx = solrt.Context(0)
    scenes = _scenes(solrt, ctx)
    datas = [S.cornell(), S.soup(20000, seed=2), S.tunnel(n_ang=128, n_ax=64, length=20.0)]
    # small ticks: jobs span many ticks and overlap (adaptive: ticks of about
    # 1 ms of device time, resized after every tick)
    if ticks == "fixed":
        srv = solrt.Server(ctx, tick_paths=3000, policy=policy)
    else:
        srv = solrt.Server(ctx, tick_paths=0, tick_ms=1, policy=policy)
    tickets = []
    for i in range(24):
        si, p = _job(solrt, i)
        cam = camera_of(datas[si], p.width / p.height)
        tickets.append((srv.submit(scenes[si], cam, p), si, cam, p))
        if i % 6 == 5:
            time.sleep(0.01)   # arrivals while ticks run
    results = []
    for t, si, cam, p in tickets:
        r = srv.wait(t, 60000)
        assert r.status == 0 and r.spp_done == p.spp and r.latency_ns >= r.queue_ns
        results.append(srv.read(t, r))
    st = srv.stats()
    assert st.completed == 24 and st.ticks > 1 and st.queue_depth == 0 and st.active == 0
    srv.close()
    # alone, on a fresh context
    ctx2 = solrt.Context(0)
    scenes2 = _scenes(solrt, ctx2)
    r = solrt.Renderer(ctx2)
    for (t, si, cam, p), (a32, a8) in zip(tickets, results):
        img = solrt.Image(ctx2, p.width, p.height, p.accum_mode)
        r.cmd_trace_rays(scenes2[si], cam, p, img)
        b32, b8 = img.read()
        assert np.array_equal(a32.view(np.uint32), b32.view(np.uint32)), t
        assert np.array_equal(a8, b8)
        img.close()


def test_budget_admission_and_eviction(solrt):
    ctx = solrt.Context(0)
    sc = solrt.SceneDescription(ctx, S.cornell())
    cam = camera_of(S.cornell(), 1.0)
    scene_bytes = sc.device_bytes()
    img_bytes = 32 * 32 * 40
    # room for the scene and two 32x32 images: later jobs wait or evict old results
    srv = solrt.Server(ctx, memory_budget=scene_bytes + 2 * img_bytes + 100)
    p = solrt.render_params(32, 32, spp=4, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=1)
    tickets = [srv.submit(sc, cam, p) for _ in range(6)]
    r = srv.wait(tickets[-1], 60000)   # results of earlier jobs may already be evicted
    assert r.status == 0
    st = srv.stats()
    assert st.completed == 6 and st.evicted >= 3
    assert st.bytes_in_use <= scene_bytes + 2 * img_bytes + 100
    # the oldest results were evicted
    s, _ = srv.poll(tickets[0])
    assert s == 7   # SOLRT_ERR_NOT_FOUND
    # a job bigger than the whole budget fails instead of waiting forever
    big = solrt.render_params(256, 256, spp=1)
    t = srv.submit(sc, cam, big)
    with pytest.raises(solrt.SolrtError) as e:
        srv.wait(t, 20000)
    assert e.value.status == 8   # SOLRT_ERR_BUDGET
    srv.close()


def test_wait_is_bounded(solrt):
    ctx = solrt.Context(0)
    sc = solrt.SceneDescription(ctx, S.soup(20000, seed=3))
    cam = camera_of(S.soup(20000, seed=3), 1.0)
    srv = solrt.Server(ctx, tick_paths=1000)
    p = solrt.render_params(64, 64, spp=64, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                            rng_mode=solrt.RNG_PER_SAMPLE, seed=3)
    t = srv.submit(sc, cam, p)
    with pytest.raises(solrt.SolrtError) as e:
        srv.wait(t, 0)
    assert e.value.status == 4   # SOLRT_ERR_TIMEOUT
    r = srv.wait(t, 60000)
    assert r.status == 0
    srv.close()


def test_shortest_first_finishes_small_jobs_first(solrt):
    """Under SERVE_SHORTEST_FIRST a small job submitted after a large one,
    while the large one is running, completes first."""
    ctx = solrt.Context(0)
    scenes = _scenes(solrt, ctx)
    d = S.cornell()
    srv = solrt.Server(ctx, tick_paths=20000, policy=solrt.api.SERVE_SHORTEST_FIRST)
    big = solrt.render_params(128, 128, spp=64, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                              rng_mode=solrt.RNG_PER_SAMPLE, seed=1)
    small = solrt.render_params(16, 16, spp=2, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                                rng_mode=solrt.RNG_PER_SAMPLE, seed=2, job_id=1)
    tb = srv.submit(scenes[0], camera_of(d, 1.0), big)
    time.sleep(0.002)
    ts = srv.submit(scenes[0], camera_of(d, 1.0), small)
    rs = srv.wait(ts, 60000)
    rb = srv.wait(tb, 60000)
    assert rs.status == 0 and rb.status == 0
    assert rs.latency_ns < rb.latency_ns
    srv.close()
    with pytest.raises(solrt.SolrtError):
        solrt.Server(ctx, policy=7)


@pytest.mark.parametrize("policy", [0, 1])
def test_job_larger_than_a_tick_completes(solrt, policy):
    """A job with more pixels than one tick holds still runs (one sample per
    tick) under both policies, next to small jobs, and renders as alone."""
    ctx = solrt.Context(0)
    d = S.cornell()
    sc = solrt.SceneDescription(ctx, d)
    srv = solrt.Server(ctx, tick_paths=256, policy=policy)
    big = solrt.render_params(32, 32, spp=3, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                              rng_mode=solrt.RNG_PER_SAMPLE, seed=5)
    small = solrt.render_params(8, 8, spp=2, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                                rng_mode=solrt.RNG_PER_SAMPLE, seed=6, job_id=1)
    cam = camera_of(d, 1.0)
    tb = srv.submit(sc, cam, big)
    ts = srv.submit(sc, cam, small)
    rb = srv.wait(tb, 60000)
    rs = srv.wait(ts, 60000)
    assert rb.status == 0 and rb.spp_done == 3 and rs.status == 0
    got = srv.read(tb, rb)[0]
    srv.close()
    img = solrt.Image(ctx, 32, 32)
    solrt.Renderer(ctx).cmd_trace_rays(sc, cam, big, img)
    assert np.array_equal(img.read()[0].view(np.uint32), got.view(np.uint32))


def _wait_status(srv, ticket, timeout_s=60.0):
    """Polls until the job leaves the queued / running states; returns the status."""
    t0 = time.time()
    while time.time() - t0 < timeout_s:
        s, _ = srv.poll(ticket)
        if s != solrt_mod().ERR_NOT_READY:
            return s
        time.sleep(0.002)
    return None


def solrt_mod():
    import importlib
    return importlib.import_module("sol-rs_gb300").api


def test_cancel_queued_and_running(solrt):
    """A cancelled running job leaves after its tick and a cancelled queued
    job at once; both report SOLRT_ERR_CANCELLED; the other jobs finish with
    the images they have alone."""
    ctx = solrt.Context(0)
    scenes = _scenes(solrt, ctx)
    d = S.cornell()
    # tiny ticks: the long job is still running when it is cancelled
    srv = solrt.Server(ctx, tick_paths=2000, memory_budget=16 << 20)
    long_p = solrt.render_params(512, 512, spp=256, max_bounces=4, material_mode=solrt.MATERIAL_LAMBERT,
                                 rng_mode=solrt.RNG_PER_SAMPLE, seed=3)
    keep = [solrt.render_params(24, 24, spp=4, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                                rng_mode=solrt.RNG_PER_SAMPLE, seed=10 + i, job_id=i) for i in range(3)]
    cam = camera_of(d, 1.0)
    t_long = srv.submit(scenes[0], cam, long_p)
    t_keep = [srv.submit(scenes[0], cam, p) for p in keep]
    t_queued = srv.submit(scenes[0], cam, long_p)      # does not fit the budget next to the first
    t0 = time.time()
    while srv.poll(t_long)[1].spp_done == 0 and time.time() - t0 < 30:   # running: one sample per tick
        time.sleep(0.001)
    assert srv.poll(t_long)[0] == solrt.api.ERR_NOT_READY
    assert srv.cancel(t_queued) == 0
    assert srv.poll(t_queued)[0] == solrt.api.ERR_CANCELLED
    assert srv.cancel(t_long) == 0
    st = _wait_status(srv, t_long)
    assert st == solrt.api.ERR_CANCELLED
    results = [srv.read(t, srv.wait(t, 60000)) for t in t_keep]
    done = srv.submit(scenes[0], cam, keep[0])
    srv.wait(done, 60000)
    assert srv.cancel(done) == solrt.api.ERR_INVALID      # already finished
    # the completion queue holds every finished ticket once, cancelled ones
    # included, and is empty once fetched
    fin = srv.finished(max_tickets=2)
    assert sorted(fin) == sorted([t_long, t_queued, done] + t_keep) and len(set(fin)) == len(fin)
    assert fin.index(t_queued) < fin.index(t_long)       # cancelled first while queued
    assert srv.finished() == []
    assert srv.release(t_long) == 0
    srv.close()
    r = solrt.Renderer(ctx)
    for p, (a32, _) in zip(keep, results):
        img = solrt.Image(ctx, p.width, p.height)
        r.cmd_trace_rays(scenes[0], cam, p, img)
        assert np.array_equal(img.read()[0].view(np.uint32), a32.view(np.uint32))
        img.close()


def test_injected_allocation_failure(solrt):
    """Host-side fault injection: the first admission fails as an image
    allocation failure would; the job reports SOLRT_ERR_OOM and the server
    goes on serving the others."""
    ctx = solrt.Context(0)
    scenes = _scenes(solrt, ctx)
    d = S.cornell()
    srv = solrt.Server(ctx, inject_alloc_failures=1)
    cam = camera_of(d, 1.0)
    ps = [solrt.render_params(16, 16, spp=2, max_bounces=3, material_mode=solrt.MATERIAL_LAMBERT,
                              rng_mode=solrt.RNG_PER_SAMPLE, seed=20 + i, job_id=i) for i in range(3)]
    tickets = [srv.submit(scenes[0], cam, p) for p in ps]
    assert _wait_status(srv, tickets[0]) == solrt.api.ERR_OOM
    for t in tickets[1:]:
        r = srv.wait(t, 60000)
        assert r.status == 0
    assert srv.stats().completed == 2
    srv.close()


def _host_estimate(oracle, data, cam, p):
    """The stopping rule's estimate recomputed on the host from the oracle's
    per-sample radiance (FP64 sums): sqrt(mean over pixels of the variance
    of the pixel mean summed over RGB / 3)."""
    o = oracle.OracleScene(data)
    x = o.render_samples(cam, p).astype(np.float64)[..., :3]      # pixels, samples, rgb
    n = x.shape[1]
    var = (np.sum(x * x, axis=(1, 2)) - np.sum(x.sum(1) ** 2, axis=1) / n) / (n - 1) / n
    return float(np.sqrt(np.mean(np.maximum(var, 0.0)) / 3.0))


@pytest.mark.parametrize("accum", ["mix", "kahan"])
def test_stopping_rule(solrt, oracle, accum):
    """With a loose bound every job stops once its estimated RMSE against
    its converged image is below it: fewer samples than asked, the estimate
    matches the host's recomputation from the oracle's samples, and the
    image equals solrt_render of the same job with spp = the samples taken.
    With a bound no image reaches, every job runs all of its samples."""
    ctx = solrt.Context(0)
    data = S.cornell()
    sc = solrt.SceneDescription(ctx, data)
    mode = solrt.ACCUM_KAHAN if accum == "kahan" else solrt.ACCUM_REF_MIX
    jobs = []
    for i, (w, h) in enumerate([(32, 32)] * 3):
        p = solrt.render_params(w, h, spp=64, max_bounces=4, seed=11 + i, job_id=i, accum_mode=mode,
                                material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE)
        jobs.append((camera_of(data, w / h), p))
    # (on this machine the estimate falls from about 0.44 after 4 samples to 0.12
    # after 64, so a 0.2 bound stops the jobs midway)
    for bound, early in ((0.2, True), (1e-9, False)):
        # ticks of 4 samples per job while all three run: estimates after 4,
        # 8, ... samples
        srv = solrt.Server(ctx, tick_paths=3 * 32 * 32 * 4, stop_rmse=bound, stop_min_spp=4)
        tickets = [srv.submit(sc, cam, p) for cam, p in jobs]
        res = [srv.wait(t, 60000) for t in tickets]
        imgs = [srv.read(t, r) for t, r in zip(tickets, res)]
        st = srv.stats()
        srv.close()
        r_ = solrt.Renderer(ctx)
        for (cam, p), r, (a32, _) in zip(jobs, res, imgs):
            assert r.status == 0
            assert r.rmse_estimate > 0
            if early:
                assert r.stopped_early == 1 and 4 <= r.spp_done < p.spp and r.rmse_estimate <= bound
            else:
                assert r.stopped_early == 0 and r.spp_done == p.spp and r.rmse_estimate > bound
            q = solrt.RenderParams.from_buffer_copy(p)
            q.spp = r.spp_done
            if not early:   # the last estimate was taken before the last tick's samples
                q.spp = r.spp_done - 4
            want = _host_estimate(oracle, data, cam, q)
            assert abs(r.rmse_estimate - want) <= 1e-3 * want, (r.rmse_estimate, want)
            q.spp = r.spp_done
            img = solrt.Image(ctx, p.width, p.height, mode)
            r_.cmd_trace_rays(sc, cam, q, img)
            b32, _ = img.read()
            img.close()
            assert np.array_equal(a32.view(np.uint32), b32.view(np.uint32))
        assert st.stopped_early == (len(jobs) if early else 0)
    sc.close()
    ctx.close()
