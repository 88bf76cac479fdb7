"""Benchmark of the 5-pathtrace hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload soup]
                    [--bvh bvh8] [--impl solrt|reference]

A step is one render launch of the workload (all samples of one frame)
through the C ABI. Default workload: the 1M-triangle soup at 1920x1080,
64 spp, max depth 4, gradient sky, Lambertian, per-sample PCG streams
(seed 2). Metric: Mrays/s = ray segments traced (primary + bounce, counted on
the device) / device time.

  value     device-timed throughput, scene + BVH resident in HBM
  e2e       the same metric through solrt_render + solrt_image_read with the
            image read back into pinned host memory every step (wall clock)
  roofline  the extend (traversal) kernel: algorithmic bytes per segment
            (32 ray + 16 hit + node bytes x nodes visited + 48 x triangles
            tested, visit counts from a counting pass) / its event-timed
            duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (scalar C++ port of the reference shaders
            with its LBVH), all host cores, on a bounded band of rows at 1 spp

--impl reference times that CPU port alone (the reference itself is Rust +
Vulkan RT and cannot run here) on the same metric and config.
Multi-GPU: replicas (each rank renders the full workload; weak scaling).
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s at RMSE≤1e-3 vs FP64 oracle, batched vs plain on 1 GB300; p99 job latency"
UNIT = "Mrays/s"

NODE_BYTES = {0: 64, 1: 80, 2: 64, 3: 224, 4: 32, 5: 64}
# What ncu measured of the BVH2 extend kernel on the full-size workloads.
# dram_bytes_per_segment: dram__bytes_read.sum + dram__bytes_write.sum over
# all extend launches of one full wavefront pass, divided by the segments
# the pass traced (profiles/extend_dram_soup1M_tunnel4M.md). limiter: the
# counters of one `ncu --set full` launch (profiles/extend_soup1M_bvh2_full.md,
# profiles/extend_soup1M_treelet_full.md, profiles/extend_tunnel_640x360_full.md).
# Keys: (workload, "lbvh" or "treelet" BVH2).
EXTEND_CAPTURES = {
    ("soup", "lbvh"): {"dram_bytes_per_segment": 62.4, "dram_source": "profiles/extend_dram_soup1M_tunnel4M.md",
             "limiter": {"l1tex_lsu_wavefronts_pct": 83.8, "l1tex_throughput_pct": 87.8, "issue_active_pct": 60.7,
                         "threads_per_instruction": 14.27, "warps_active_pct": 48.0, "l2_hit_pct": 96.7,
                         "dram_throughput_pct": 1.4, "source": "profiles/extend_soup1M_bvh2_full.md"}},
    ("soup", "treelet"): {"dram_bytes_per_segment": 62.2, "dram_source": "profiles/extend_dram_soup1M_tunnel4M.md",
                          "limiter": {"l1tex_lsu_wavefronts_pct": 85.2, "l1tex_throughput_pct": 87.9,
                                      "issue_active_pct": 66.1, "threads_per_instruction": 14.83,
                                      "warps_active_pct": 48.7, "l2_hit_pct": 94.2,
                                      "source": "profiles/extend_soup1M_treelet_full.md"}},
    ("tunnel", "treelet"): {"dram_bytes_per_segment": 78.0, "dram_source": "profiles/extend_dram_soup1M_tunnel4M.md",
                            "limiter": {"l1tex_lsu_wavefronts_pct": 70.0, "l1tex_throughput_pct": 75.1,
                                        "issue_active_pct": 65.2, "threads_per_instruction": 14.55,
                                        "warps_active_pct": 46.7, "l2_hit_pct": 90.1,
                                        "source": "profiles/extend_tunnel_640x360_full.md (treelet BVH2, bounce level 1)"}},
    ("tunnel", "lbvh"): {"dram_bytes_per_segment": 78.8, "dram_source": "profiles/extend_dram_soup1M_tunnel4M.md",
               "limiter": {"l1tex_lsu_wavefronts_pct": 71.9, "l1tex_throughput_pct": 77.7, "issue_active_pct": 65.0,
                           "threads_per_instruction": 14.52, "warps_active_pct": 46.9, "l2_hit_pct": 91.7,
                           "source": "profiles/extend_tunnel_640x360_full.md (bounce level 1)"}},
}


def workload(name):
    solrt = importlib.import_module("sol-rs_gb300")
    S = solrt.scenes
    if name == "soup":
        data = S.soup(1_000_000, seed=2)
        kw = dict(width=1920, height=1080, spp=64, max_bounces=4, miss_mode=solrt.MISS_GRADIENT,
                  material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=2,
                  accum_mode=solrt.ACCUM_REF_MIX)
        cfg = {"workload": "triangle soup 1M tris, 1920x1080, 64 spp, max depth 4, gradient sky, Lambert",
               "tris": 1_000_000, "width": 1920, "height": 1080, "spp": 64, "max_depth": 4}
    elif name == "cornell":
        data = S.cornell()
        kw = dict(width=256, height=256, spp=16, max_bounces=5, miss_mode=solrt.MISS_BLACK,
                  material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=1,
                  accum_mode=solrt.ACCUM_REF_MIX)
        cfg = {"workload": "procedural Cornell box 32 tris, 256x256, 16 spp, max depth 5, Lambert",
               "tris": 32, "width": 256, "height": 256, "spp": 16, "max_depth": 5}
    elif name == "tunnel":
        data = S.tunnel()
        kw = dict(width=2560, height=1440, spp=128, max_bounces=8, miss_mode=solrt.MISS_REF_SKY,
                  material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=3,
                  accum_mode=solrt.ACCUM_KAHAN)
        cfg = {"workload": "procedural tunnel 2048x1024 segments (4.19M tris), 2560x1440, 128 spp, max depth 8, "
                           "Kahan accumulation, sky", "tris": data.tri_count, "width": 2560, "height": 1440,
               "spp": 128, "max_depth": 8}
    elif name == "instances":
        data = S.instanced_soups(4, 16384, seed=5)
        kw = dict(width=1920, height=1080, spp=64, max_bounces=4, miss_mode=solrt.MISS_GRADIENT,
                  material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=5,
                  accum_mode=solrt.ACCUM_REF_MIX)
        cfg = {"workload": "64 instanced sections of 16384-triangle soups (1.05M tris) in a 4^3 grid, 1920x1080, "
                           "64 spp, max depth 4, gradient sky, Lambert", "tris": data.tri_count, "width": 1920,
               "height": 1080, "spp": 64, "max_depth": 4}
    else:
        raise SystemExit("unknown workload %s" % name)
    return data, kw, cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id):
        self.device_id = device_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.device_id], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def l2_copy_gbs(local):
    """Device copy bandwidth of a 32 MB buffer pair that stays in the 129 MB
    L2 (read + write bytes over CUDA-event time, best of 20): the denominator
    of the roofline of scenes that live in L2."""
    import torch
    dev = torch.device("cuda", local)
    a = torch.empty(8 << 20, dtype=torch.float32, device=dev).fill_(1.0)
    b = torch.empty_like(a)
    best = 0.0
    for _ in range(3):
        b.copy_(a)
    for _ in range(20):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        best = max(best, 2 * a.numel() * 4 / (ms / 1e3) / 1e9)
    return best


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(data, kw, cam, budget_s=10.0, threads=0):
    """Oracle FP32 render (its LBVH, all host cores) of the full image at as
    many samples per pixel as fit in about budget_s (at most the workload's
    spp), sized from a timed band of rows at 1 spp: Mrays/s of that render."""
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    o = oracle.OracleScene(data)
    h = kw["height"]
    rows = max(1, h // 16)
    r0 = h // 2 - rows // 2
    t0 = time.perf_counter()
    o.render(cam, solrt.render_params(**dict(kw, spp=1)), rows=(r0, r0 + rows), threads=threads)
    est = (time.perf_counter() - t0) * h / rows          # seconds for the full image at 1 spp
    spp = max(1, min(kw["spp"], int(budget_s / max(est, 1e-6))))
    t0 = time.perf_counter()
    _, _, st = o.render(cam, solrt.render_params(**dict(kw, spp=spp)), threads=threads)
    dt = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    sample = "full %dx%d image at %d of the workload's %d spp, FP32 oracle with its LBVH" % (
        kw["width"], h, spp, kw["spp"])
    return {"value": st.segments / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
            "segments": int(st.segments), "seconds": round(dt, 3)}


def precision_study(local, data, kw, cam, main_mrays, main_info, main_nodes, main_tris, n_rays=1 << 22,
                    kinds=None, render=True, main_sah=False, capacity=0):
    """The 16-bit quantised binary BVH, the 8-bit quantised 4- and 8-wide BVHs
    and the FP32 8-wide BVH next to the FP32 binary BVH on the same scene:
    hit records of 4M rays (every pixel-centre camera ray of the frame, then
    seeded rays from inside the scene's bounds) traced on the device by each
    kind and compared bit for bit with the oracle's CPU LBVH traversal on all
    host cores (the checker), node bytes, visits per segment, Mrays/s of one
    frame and the FP64 fallback count of each."""
    import torch
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    S = solrt.scenes
    W, H = kw["width"], kw["height"]
    rays = S.probe_rays(data, cam, W, H, n_rays, seed=7)
    t0 = time.perf_counter()
    o = oracle.OracleScene(data)
    want, want_fb = o.trace(rays)
    o.close()
    oracle_s = time.perf_counter() - t0
    want_u = want.view(np.uint32).reshape(-1, 4)
    edge = S.near_edge(want)
    dev = torch.device("cuda", local)
    rays_d = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    out = {"rays_compared": n_rays, "leaf_max": 1}
    vs = {"rays": n_rays, "hits": int((want["prim"] != 0xFFFFFFFF).sum()), "near_edge_hits": int(edge.sum()),
          "mismatches": {}, "near_edge_mismatches": {}, "oracle_fp64_fallbacks": int(want_fb),
          "oracle": "CPU LBVH traversal (FP32 watertight test, FP64 edge fallback, lower index wins ties) on %d "
                    "threads, %.1f s" % (os.cpu_count() or 1, oracle_s),
          "rays_desc": "%d pixel-centre camera rays of the %dx%d frame + %d seeded rays from inside the scene "
                       "bounds" % (min(n_rays, W * H), W, H, max(0, n_rays - W * H))}
    all_kinds = (("bvh2_fp32", solrt.BVH2, False), ("bvh2_treelet", solrt.BVH2, True), ("bvh2_q16", solrt.BVH2_Q16, False),
                 ("bvh4_q8", solrt.BVH4_Q8, False), ("bvh8_q8", solrt.BVH8_Q8, False),
                 ("bvh8_q8_sah", solrt.BVH8_Q8, True), ("bvh8_fp32", solrt.BVH8_F32, False))
    with solrt.Context(local, enable_timing=True, path_capacity=capacity) as ctx, \
            solrt.Context(local, enable_counters=True) as cctx:
        for name, kind, sah in all_kinds:
            if kinds is not None and name not in kinds:
                continue
            sc = solrt.SceneDescription(ctx, data, bvh=kind, leaf_max=0 if kind in (solrt.BVH2, solrt.BVH2_Q16) else 1,
                                        sah=sah)
            info = sc.bvh_info()
            depth = int(info.depth)
            h = torch.zeros((n_rays, 4), dtype=torch.float32, device=dev)
            ctx.reset_stats()
            sc.trace_rays_device(rays_d.data_ptr(), n_rays, h.data_ptr())
            ctx.synchronize()
            fb_trace = ctx.stats().fp64_fallbacks
            got = h.cpu().numpy().view(np.uint32)
            bad = np.any(got != want_u, axis=1)
            vs["mismatches"][name] = int(bad.sum())
            vs["near_edge_mismatches"][name] = int((bad & edge).sum())
            del h
            mr = nodes = tris = None
            if main_info is not None and kind == main_info.kind and sah == main_sah and main_mrays is not None:
                mr, nodes, tris = main_mrays, main_nodes, main_tris
            elif render:
                img = solrt.Image(ctx, W, H, kw["accum_mode"])
                r = solrt.Renderer(ctx)
                r.cmd_trace_rays(sc, cam, solrt.render_params(**kw), img)
                ctx.synchronize()
                ctx.reset_stats()
                r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(kw, frame=1)), img)
                ctx.synchronize()
                st = ctx.stats()
                mr = st.segments / (st.render_ms / 1000.0) / 1e6 if st.render_ms > 0 else None
                img.close()
                csc = solrt.SceneDescription(cctx, data, bvh=kind, leaf_max=0 if kind in (solrt.BVH2, solrt.BVH2_Q16) else 1,
                                             sah=sah)
                cimg = solrt.Image(cctx, W, H, kw["accum_mode"])
                cctx.reset_stats()
                solrt.Renderer(cctx).cmd_trace_rays(csc, cam, solrt.render_params(**dict(kw, spp=min(4, kw["spp"]))),
                                                    cimg)
                cctx.synchronize()
                cs = cctx.stats()
                nodes = cs.node_visits / max(cs.segments, 1)
                tris = cs.tri_tests / max(cs.segments, 1)
                cimg.close()
                csc.close()
            nb = NODE_BYTES[info.kind]
            out[name] = {"mrays_per_s": round(mr, 1) if mr else None, "node_bytes": int(info.node_bytes),
                         "node_count": int(info.node_count), "bytes_per_node": nb,
                         "nodes_per_segment": round(nodes, 2) if nodes is not None else None,
                         "tris_per_segment": round(tris, 2) if tris is not None else None,
                         "node_bytes_per_segment": round(nb * nodes, 1) if nodes is not None else None,
                         "fp64_fallbacks_in_compared_rays": int(fb_trace), "build_ms": round(info.build_ms, 3),
                         "depth": depth}
            sc.close()
    out["hit_ids_vs_oracle"] = vs
    return out


def rmse_vs_fp64(local, data, kw, cam, bvh, rows, frames=1, sah=False):
    """RMSE of the device RGBA32F image (after `frames` accumulated frames)
    against the FP64 oracle on identical RNG streams, over image rows
    [rows[0], rows[1]) (the oracle is the checker). Also compares the same
    rows with the FP32 oracle bit for bit."""
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    W, H = kw["width"], kw["height"]
    with solrt.Context(local) as ctx:
        sc = solrt.SceneDescription(ctx, data, bvh=bvh, sah=sah, keep_data=False)
        img = solrt.Image(ctx, W, H, kw["accum_mode"])
        r = solrt.Renderer(ctx)
        for f in range(frames):
            r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(kw, frame=f)), img)
        acc, _ = img.read()
        img.close()
        sc.close()
    t0 = time.perf_counter()
    o = oracle.OracleScene(data)
    kahan = kw["accum_mode"] == solrt.ACCUM_KAHAN
    out = {}
    for prec in (64, 32):
        a = np.zeros((H, W, 4), np.float32)
        ks = np.zeros((H, W, 4), np.float32) if kahan else None
        kc = np.zeros((H, W, 4), np.float32) if kahan else None
        for f in range(frames):
            a, _, _ = o.render(cam, solrt.render_params(**dict(kw, frame=f)), accum=a, ksum=ks, kcomp=kc, rows=rows,
                               precision=prec)
        out[prec] = a[rows[0]:rows[1]]
    o.close()
    g = acc[rows[0]:rows[1]]
    d = g[..., :3].astype(np.float64) - out[64][..., :3].astype(np.float64)
    v = float(np.sqrt(np.mean(d * d)))
    return {"rmse": v, "bound": 1e-3, "within_bound": v <= 1e-3, "rows": list(rows), "width": W,
            "spp": kw["spp"] * frames, "frames": frames,
            "bit_exact_vs_fp32_oracle": bool(np.array_equal(g.view(np.uint32), out[32].view(np.uint32))),
            "oracle_seconds": round(time.perf_counter() - t0, 2),
            "how": "device RGBA32F after %d frame(s) vs FP64 oracle, identical RNG streams, rows %d-%d of %d"
                   % (frames, rows[0], rows[1] - 1, H)}


def parity_cornell(local):
    """The plain small configuration at its stated size (procedural Cornell
    box, 256x256, 16 spp, depth 5, Lambert, seed 1) rendered whole: bit for
    bit against the FP32 oracle, equal segment counts, RMSE against the FP64
    oracle over the whole image, device Mrays/s."""
    import torch
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    data, kw, cfg = workload("cornell")
    W, H = kw["width"], kw["height"]
    c = data.camera
    cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], W / H)
    with solrt.Context(local) as ctx:
        sc = solrt.SceneDescription(ctx, data)
        img = solrt.Image(ctx, W, H)
        r = solrt.Renderer(ctx)
        p = solrt.render_params(**kw)
        for _ in range(3):
            r.cmd_trace_rays(sc, cam, p, img)
        ext = torch.cuda.ExternalStream(ctx.stream())
        ctx.synchronize()
        ctx.reset_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(10):
            r.cmd_trace_rays(sc, cam, p, img)
        e1.record(ext)
        ctx.synchronize()
        mrays = ctx.stats().segments / (e0.elapsed_time(e1) / 1000.0) / 1e6
        img2 = solrt.Image(ctx, W, H)
        ctx.reset_stats()
        r.cmd_trace_rays(sc, cam, p, img2)
        ctx.synchronize()
        seg = ctx.stats().segments
        acc, _ = img2.read()
        img.close()
        img2.close()
        sc.close()
    t0 = time.perf_counter()
    o = oracle.OracleScene(data)
    a32, _, st = o.render(cam, p)
    a64, _, _ = o.render(cam, p, precision=64)
    o.close()
    d = acc[..., :3].astype(np.float64) - a64[..., :3].astype(np.float64)
    v = float(np.sqrt(np.mean(d * d)))
    return {"workload": cfg["workload"], "device_mrays_s": round(mrays, 1),
            "bit_exact_vs_fp32_oracle": bool(np.array_equal(acc.view(np.uint32), a32.view(np.uint32))),
            "segments": int(seg), "oracle_segments": int(st.segments),
            "rmse_vs_fp64": {"rmse": v, "bound": 1e-3, "within_bound": v <= 1e-3, "rows": [0, H], "spp": kw["spp"],
                             "how": "whole image, one frame, identical RNG streams"},
            "oracle_seconds": round(time.perf_counter() - t0, 2)}


def parity_tunnel(local, n_rays=1 << 22, capacity=0):
    """The procedural tunnel at its stated size (4.19M triangles, 2560x1440,
    128 spp, depth 8, Kahan sums): RMSE against the FP64 oracle over two
    central rows after four frames (512 spp), and the hit records of 4M probe
    rays of the BVH2 and the BVH8-q8 (SAH collapse) against the oracle's
    traversal, with Mrays/s of one frame for each."""
    solrt = importlib.import_module("sol-rs_gb300")
    data, kw, cfg = workload("tunnel")
    W, H = kw["width"], kw["height"]
    c = data.camera
    cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], W / H)
    out = {"workload": cfg["workload"]}
    out["rmse_vs_fp64"] = rmse_vs_fp64(local, data, kw, cam, solrt.BVH2, (H // 2 - 1, H // 2 + 1), frames=4)
    ps = precision_study(local, data, kw, cam, None, None, None, None, n_rays=n_rays,
                         kinds=("bvh2_fp32", "bvh2_treelet", "bvh8_q8", "bvh8_q8_sah"), capacity=capacity)
    out.update(ps)
    return out


def reference_semantics(local, data, kw, cam, budget_s=3.0, sah=True):
    """The workload's scene and image under the settings the reference's
    shaders fix (pathtrace.rgen:41-45, pathtrace.rchit:90-111,
    pathtrace.rmiss:8-21): 8 samples per launch, at most 32 bounces, the
    reference materials and sky, one RNG stream per pixel, mix accumulation.
    Device Mrays/s over the whole image (CUDA events, one launch = one
    frame), and the reference's own pathtrace.rgen / .rchit / .rmiss compiled
    as C++ (oracle/_ref) on all host cores over a central band of rows of the
    same launch, traceRayEXT answered by the oracle's LBVH closest hit; the
    device rows are compared with the reference pipeline's bit for bit."""
    import torch
    import oracle
    solrt = importlib.import_module("sol-rs_gb300")
    W, H = kw["width"], kw["height"]
    p = solrt.render_params(W, H, spp=8, max_bounces=32, material_mode=solrt.MATERIAL_REF,
                            miss_mode=solrt.MISS_REF_SKY, rng_mode=solrt.RNG_REF_STREAM,
                            accum_mode=solrt.ACCUM_REF_MIX)
    out = {"settings": "8 spp per launch, 32 bounces, reference materials, reference sky, per-pixel RNG stream, "
                       "mix accumulation (the reference shaders' own)"}
    with solrt.Context(local) as ctx:
        sc = solrt.SceneDescription(ctx, data, keep_data=False, sah=sah)  # the BVH of the headline
        img = solrt.Image(ctx, W, H)
        r = solrt.Renderer(ctx)
        for f in range(2):
            r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(_params_dict(p), frame=f)), img)
        ext = torch.cuda.ExternalStream(ctx.stream())
        ctx.synchronize()
        ctx.reset_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for f in range(5):
            r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(_params_dict(p), frame=2 + f)), img)
        e1.record(ext)
        ctx.synchronize()
        gpu = ctx.stats().segments / (e0.elapsed_time(e1) / 1000.0) / 1e6
        img.close()
        img = solrt.Image(ctx, W, H)
        r.cmd_trace_rays(sc, cam, p, img)
        acc, _ = img.read()
        img.close()
        sc.close()
    out["device_mrays_s"] = round(gpu, 1)
    if oracle.ref_lib() is None:
        out["reference_shaders"] = {"unavailable": "oracle/_ref not built (no reference checkout and no generated "
                                                   "sources)"}
        return out
    o = oracle.OracleScene(data)
    st = {}
    t0 = time.perf_counter()
    oracle.ref_path_render(o, cam, W, H, rows=(H // 2 - 1, H // 2 + 1), sky=True, stats=st)
    per_row = (time.perf_counter() - t0) / 2
    rows = int(min(H, max(2, budget_s / max(per_row, 1e-6))))
    r0 = max(0, H // 2 - rows // 2)
    t0 = time.perf_counter()
    ra, _ = oracle.ref_path_render(o, cam, W, H, rows=(r0, r0 + rows), sky=True, stats=st)
    dt = time.perf_counter() - t0
    o.close()
    cpu = st["rays"] / dt / 1e6
    out["reference_shaders"] = {"mrays_s": round(cpu, 3), "cores": os.cpu_count() or 1, "rows": [r0, r0 + rows],
                                "traced": int(st["rays"]), "seconds": round(dt, 2)}
    out["device_over_reference_shaders"] = round(gpu / cpu, 1) if cpu > 0 else None
    out["band_bit_exact_vs_reference_shaders"] = bool(
        np.array_equal(acc[r0:r0 + rows].view(np.uint32), ra[r0:r0 + rows].view(np.uint32)))
    return out


def _params_dict(p):
    return {"width": p.width, "height": p.height, "spp": p.spp, "max_bounces": p.max_bounces, "frame": p.frame,
            "seed": p.seed, "miss_mode": p.miss_mode, "material_mode": p.material_mode,
            "accum_mode": p.accum_mode, "rng_mode": p.rng_mode}


def run_batch(args, world, rank, local, pg, njobs=None, steps=None, emit=True, warmup=None):
    """Batched mixed scenes (256 randomised Cornell boxes with log-uniform
    1k-500k-triangle soups, 128^2..1024^2, 4-64 spp, depth 5): one CUDA-graph
    replay per step vs the same jobs rendered one solrt_render at a time,
    with the plain per-pixel megakernel and with the wavefront."""
    import torch
    solrt = importlib.import_module("sol-rs_gb300")
    S = solrt.scenes
    bvh = {"bvh2": solrt.BVH2, "bvh2q": solrt.BVH2_Q16, "bvh2t": solrt.BVH2_TWO_LEVEL, "bvh4": solrt.BVH4_Q8,
           "bvh8": solrt.BVH8_Q8, "bvh8f": solrt.BVH8_F32}[args.bvh]
    njobs = args.jobs if njobs is None else njobs
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    ctx = solrt.Context(local)  # 32M-path passes (128M measured the same: 2904.5 against 2904.0 Mrays/s)
    jobs, tris, pixels, samples = [], 0, 0, 0
    t0 = time.perf_counter()
    for i in range(njobs):
        data, jp = S.mixed_scene(i)
        sc = solrt.SceneDescription(ctx, data, bvh=bvh, keep_data=False, sah=args.sah)
        tris += data.tri_count
        del data
        w, h = jp["width"], jp["height"]
        img = solrt.Image(ctx, w, h)
        c = S.CORNELL_CAMERA
        cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], 1.0)
        p = solrt.render_params(w, h, spp=jp["spp"], max_bounces=jp["max_bounces"], seed=jp["seed"], job_id=i,
                                material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE,
                                miss_mode=solrt.MISS_BLACK)
        jobs.append((sc, img, cam, p))
        pixels += w * h
        samples += w * h * jp["spp"]
    setup_s = time.perf_counter() - t0
    batch = solrt.Batch(ctx, jobs, graph=True)
    # launch shape and pass size chosen by the autotuner (outside the timed
    # region; it leaves the batch re-planned with its choice)
    t1 = time.perf_counter()
    tune = batch.autotune()
    tune["tune_s"] = round(time.perf_counter() - t1, 2)
    info = batch.info()
    ext = torch.cuda.ExternalStream(ctx.stream())

    def timed(fn, steps):
        ctx.synchronize()
        ctx.reset_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(steps):
            fn()
        e1.record(ext)
        ctx.synchronize()
        torch.cuda.synchronize()
        st = ctx.stats()
        return e0.elapsed_time(e1), st.segments, st.launches

    r = solrt.Renderer(ctx)
    mega_params = []
    for sc, img, cam, p in jobs:
        q = solrt.RenderParams.from_buffer_copy(p)
        q.kernel = solrt.api.KERNEL_MEGA
        mega_params.append(q)

    def plain_wavefront():
        for sc, img, cam, p in jobs:
            r.cmd_trace_rays(sc, cam, p, img)

    def plain_mega():
        for (sc, img, cam, _), q in zip(jobs, mega_params):
            r.cmd_trace_rays(sc, cam, q, img)

    for _ in range(max(1, warmup)):
        batch.launch()
    plain_wavefront()
    plain_mega()
    clocks = ClockSampler(str(local)) if emit else None
    if clocks:
        clocks.start()
        time.sleep(0.3)
    barrier(pg)
    ms_b, seg_b, launches_b = timed(batch.launch, steps)
    ms_w, seg_w, launches_w = timed(plain_wavefront, 1)
    ms_m, seg_m, launches_m = timed(plain_mega, 1)
    # the same jobs in one persistent per-pixel launch (device work counter)
    pbatch = solrt.Batch(ctx, jobs, persistent=True)
    pbatch.launch()
    ms_p, seg_p, launches_p = timed(pbatch.launch, 1)
    pbatch.close()
    # the wavefront passes as phases of one cooperative launch (grid-wide
    # barriers between stages), in a CUDA graph; every launch renders the
    # same frame, so its images must equal the batched ones bit for bit
    coop_error = None
    try:
        check = [img.read()[0].copy() for _, img, _, _ in jobs[:8]]
        cbatch = solrt.Batch(ctx, jobs, graph=True, cooperative=True)
        cbatch.launch()
        ms_c, seg_c, launches_c = timed(cbatch.launch, 1)
        coop_equal = all(np.array_equal(x.view(np.uint32), img.read()[0].view(np.uint32))
                         for x, (_, img, _, _) in zip(check, jobs))
        cbatch.close()
    except Exception as ex:  # the other rows stand without it
        coop_error = str(ex)
        ms_c, seg_c, launches_c, coop_equal = 1.0, 0, 0, None
    clk = clocks.stop() if clocks else None
    ms_b_max = max_over_ranks(pg, ms_b)
    value = sum_over_ranks(pg, float(seg_b)) / (ms_b_max / 1000.0) / 1e6
    plain_v = seg_m / (ms_m / 1000.0) / 1e6
    wave_v = seg_w / (ms_w / 1000.0) / 1e6
    cmp = {"jobs": njobs, "batched": round(value, 3), "plain_megakernel_scene_by_scene": round(plain_v, 3),
           "ratio": round(value / plain_v, 3) if plain_v > 0 else None,
           "wavefront_scene_by_scene": round(wave_v, 3),
           "ratio_vs_wavefront": round(value / wave_v, 3) if wave_v > 0 else None,
           "persistent_one_launch": round(seg_p / (ms_p / 1000.0) / 1e6, 3),
           "cooperative_one_launch": round(seg_c / (ms_c / 1000.0) / 1e6, 3) if coop_error is None else None,
           "cooperative_images_equal_batched": coop_equal,
           "cooperative_error": coop_error,
           "batch_ms": round(ms_b_max / steps, 3), "passes": info["passes"], "items": info["items"],
           "pass_fill": round(info["paths"] / max(1, info["passes"] * ctx.capacity()), 3),
           "launches_per_step": {"batched": int(launches_b // steps), "wavefront_scene_by_scene": int(launches_w),
                                 "megakernel_scene_by_scene": int(launches_m), "persistent_one_launch": int(launches_p),
                                 "cooperative_one_launch": int(launches_c)},
           "tris": int(tris), "pixels": int(pixels), "samples": int(samples), "setup_s": round(setup_s, 1),
           "autotune": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in tune.items()}}
    if rank == 0 and emit:
        out = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": steps,
               "warmup": args.warmup, "ms_per_step": round(ms_b_max / steps, 3), "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": "batched mixed scenes: %d x (randomised Cornell box + log-uniform 1k-500k-tri "
                                      "soup), 128^2..1024^2, 4-64 spp, depth 5, one CUDA-graph replay per step"
                                      % njobs, "jobs": njobs, "tris": tris, "pixels": pixels,
                          "samples": samples, "bvh": args.bvh, "passes": info["passes"], "items": info["items"],
                          "setup_s": round(setup_s, 1),
                          "l2": "inputs larger than L2 (scenes + BVHs + queues > 129 MB)"},
               "batched_vs_plain": cmp,
               "segments_per_step": int(seg_b // steps), "gpu_launches": int(launches_b), "clocks": clk}
        print(json.dumps(out), flush=True)
    batch.close()
    for sc, img, _, _ in jobs:
        img.close()
        sc.close()
    ctx.close()
    return cmp


def run_serve(local, rate, duration, n_scenes=16, seed=5, policy=0, stop_rmse=0.0, drain_s=300.0, sah=False):
    """Served render jobs: Poisson arrivals at `rate` jobs/s for `duration`
    seconds; each job draws a scene from a resident pool of config-4 scenes
    (randomised Cornell box + log-uniform soup), a resolution from
    {128^2, 256^2, 512^2, 1024^2}, spp uniform 1..256, depth 5. With
    stop_rmse > 0 the server's stopping rule ends a job once its estimated
    RMSE against its converged image is at most that. Jobs still unfinished
    drain_s seconds after the last arrival are cancelled and counted.
    Returns p50 / p99 job latency of the completed jobs, the throughput over
    the arrival window and over the whole run, and admission-queue depth."""
    solrt = importlib.import_module("sol-rs_gb300")
    S = solrt.scenes
    ctx = solrt.Context(local)
    pool = [solrt.SceneDescription(ctx, S.mixed_scene(i)[0], keep_data=False, sah=sah) for i in range(n_scenes)]
    c = S.CORNELL_CAMERA
    cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], 1.0)
    rng = np.random.default_rng(seed)
    srv = solrt.Server(ctx, policy=policy, stop_rmse=stop_rmse)
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        res = int(rng.choice([128, 256, 512, 1024]))
        arrivals.append((t, int(rng.integers(0, n_scenes)), res, int(rng.integers(1, 257))))
    ctx.reset_stats()
    pending, lat, qdepth, paths, est, early, spp_frac = {}, [], [], 0, [], 0, []
    t0 = time.perf_counter()
    i = 0
    seg_window = None

    def drain():
        nonlocal early
        for tk in srv.finished():   # the completion queue: only jobs that finished since the last look
            if tk not in pending:
                continue
            st_, r = srv.poll(tk)
            if st_ == 0:
                lat.append(r.latency_ns / 1e6)
                if r.rmse_estimate >= 0:
                    est.append(r.rmse_estimate)
                early += int(r.stopped_early)
                spp_frac.append(r.spp_done / pending[tk][1])
                srv.release(tk)
                del pending[tk]

    while i < len(arrivals) or pending:
        now = time.perf_counter() - t0
        while i < len(arrivals) and arrivals[i][0] <= now:
            _, si, res, spp = arrivals[i]
            p = solrt.render_params(res, res, spp=spp, max_bounces=5, seed=seed + i, job_id=i,
                                    material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE)
            pending[srv.submit(pool[si], cam, p)] = (i, spp)
            paths += res * res * spp
            i += 1
        if seg_window is None and now >= duration:
            seg_window = srv.stats().segments
        qdepth.append(srv.stats().queue_depth)
        drain()
        if now > duration + drain_s:
            break
        time.sleep(0.002)
    wall = time.perf_counter() - t0
    unfinished = len(pending)
    for tk in list(pending):
        srv.cancel(tk)
    st = srv.stats()
    srv.close()
    for sc in pool:
        sc.close()
    seg = ctx.stats().segments
    ctx.close()
    lat = np.array(lat) if lat else np.zeros(1)
    out = {"rate_jobs_per_s": rate, "duration_s": duration, "policy": ["fair", "shortest_first"][policy],
           "jobs": len(arrivals), "completed": int(len(arrivals) - unfinished),
           "unfinished_cancelled": int(unfinished), "drain_cap_s": drain_s,
           "p50_latency_ms": round(float(np.percentile(lat, 50)), 2),
           "p99_latency_ms": round(float(np.percentile(lat, 99)), 2),
           "latency_of": "completed jobs",
           "sustained_mrays_s": round(seg / wall / 1e6, 2),
           "window_mrays_s": round((seg_window if seg_window is not None else seg) / min(wall, duration) / 1e6, 2),
           "wall_s": round(wall, 2),
           "busy_fraction": round(st.busy_ms / 1000.0 / wall, 3),
           "max_queue_depth": int(max(qdepth) if qdepth else 0),
           "mean_queue_depth": round(float(np.mean(qdepth)) if qdepth else 0.0, 2),
           "paths_submitted": int(paths), "ticks": int(st.ticks), "last_tick_paths": int(st.tick_paths),
           "tick_size": "adaptive (about 40 ms of device time each)"}
    if stop_rmse > 0:
        out["stop"] = {"rule": "rmse", "bound": stop_rmse, "stopped_early": int(early),
                       "rmse_estimate_median": round(float(np.median(est)), 5) if est else None,
                       "rmse_estimate_min": round(float(np.min(est)), 5) if est else None,
                       "spp_done_over_spp_median": round(float(np.median(spp_frac)), 3) if spp_frac else None,
                       "how": "per job, after each tick: sqrt(mean over pixels and RGB of the sample variance / "
                              "samples), from per-pixel sums and squared sums on the device"}
    return out


def run_reference(args, world, rank, pg):
    """The reference arm: the CPU port of the reference's path (the oracle:
    pathtrace.rgen / .rchit / .rmiss restated in C++ with its LBVH, pinned bit
    for bit against the reference's own shaders compiled as C++) on all host
    cores, on this workload's exact settings, over a central band of rows at
    the full spp per step. The reference itself (Rust + Vulkan ray tracing)
    cannot run on this machine, and its shaders fix settings (8 spp, 32
    bounces, reference materials and sky) other than the configuration's, so
    the port is the implementation that renders this configuration. This arm
    never loads the CUDA library: the camera comes from the oracle."""
    if rank != 0:
        return 0
    import oracle
    data, kw, cfg = workload(args.workload)
    solrt_api = importlib.import_module("sol-rs_gb300.api")
    W, H = kw["width"], kw["height"]
    c = data.camera
    cam = oracle.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], W / H)
    o = oracle.OracleScene(data)
    p = solrt_api.render_params(**kw)
    # one step = a central band of rows at the full spp, sized to ~1 s
    t0 = time.perf_counter()
    o.render(cam, p, rows=(H // 2, H // 2 + 1))
    per_row = time.perf_counter() - t0
    rows = int(min(H, max(1, 1.0 / max(per_row, 1e-6))))
    r0 = max(0, H // 2 - rows // 2)
    for i in range(args.warmup):
        o.render(cam, solrt_api.render_params(**dict(kw, frame=i)), rows=(r0, r0 + rows))
    seg, tt = 0, 0.0
    for i in range(args.steps):
        t0 = time.perf_counter()
        _, _, st = o.render(cam, solrt_api.render_params(**dict(kw, frame=args.warmup + i)), rows=(r0, r0 + rows))
        tt += time.perf_counter() - t0
        seg += st.segments
    o.close()
    v = seg / tt / 1e6
    cores = os.cpu_count() or 1
    sample = ("%d rows x %d px x %d spp per step (central band of the %dx%d frame, the workload's own settings): "
              "FP32 CPU port of the reference's pathtrace shaders with its LBVH, %d threads" % (
                  rows, W, kw["spp"], W, H, cores))
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * tt / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": run_config(cfg, args, world),
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_config(cfg, args, world):
    """The config object of the JSON line, the same for both arms."""
    return dict(cfg, parallelism="replicas" if world > 1 else "single", bvh=args.bvh + ("+sah" if args.sah else ""),
                l2="inputs larger than L2 (scene + BVH + path queues > 129 MB)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="solrt", choices=["solrt", "reference"])
    ap.add_argument("--workload", default="soup", choices=["soup", "cornell", "tunnel", "instances", "batch", "serve"])
    ap.add_argument("--bvh", default="bvh2", choices=["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"])
    ap.add_argument("--sah", action="store_true", help="(the default) SOLRT_BVH_SAH: binary kinds restructured by "
                                                        "treelets toward the SAH, wide kinds collapsed by SAH")
    ap.add_argument("--lbvh", action="store_true", help="plain LBVH (no SOLRT_BVH_SAH)")
    ap.add_argument("--kernel", default="wavefront", choices=["wavefront", "mega"],
                    help="mega: the plain per-pixel kernel (the reference's loop structure) on the same workload")
    ap.add_argument("--nee", action="store_true",
                    help="next-event estimation (shadow-ray queue); shadow rays are reported apart from the metric")
    ap.add_argument("--jobs", type=int, default=256)
    ap.add_argument("--rate", type=float, default=50.0, help="serve: Poisson arrival rate, jobs/s")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: arrival window, s")
    ap.add_argument("--drain", type=float, default=30.0,
                    help="serve: seconds after the last arrival before unfinished jobs are cancelled")
    ap.add_argument("--steady-rate", type=float, default=8.0,
                    help="serve: arrival rate of the second, below-capacity serving run of the default line")
    ap.add_argument("--steady-duration", type=float, default=30.0, help="serve: arrival window of that run, s")
    ap.add_argument("--no-serve-steady", action="store_true", help="skip the below-capacity serving run")
    ap.add_argument("--stop-rmse", type=float, default=1e-3,
                    help="serve: stopping rule, estimated RMSE against the converged image (0 = run every sample)")
    ap.add_argument("--policy", default="shortest", choices=["fair", "shortest"], help="serve: scheduling policy")
    ap.add_argument("--no-serve", action="store_true", help="skip the short serving run of the default line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the BVH8-q8 vs FP32 BVH2 comparison")
    ap.add_argument("--width", type=int, default=0, help="override the workload's image width (profiling runs)")
    ap.add_argument("--height", type=int, default=0, help="override the workload's image height")
    ap.add_argument("--spp", type=int, default=0, help="override the workload's samples per pixel")
    ap.add_argument("--capacity", type=int, default=128 << 20,
                    help="paths per pass of the single-scene contexts (default 128M: a 64-spp 1080p frame in one "
                         "pass, 19 GB of queues; 0 = the library default, 32M)")
    args = ap.parse_args()
    args.sah = not args.lbvh
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        return run_reference(args, world, rank, pg)
    if args.workload == "batch":
        importlib.import_module("sol-rs_gb300.build").build_lib()
        run_batch(args, world, rank, local, pg)
        return 0
    if args.workload == "serve":
        importlib.import_module("sol-rs_gb300.build").build_lib()
        out = run_serve(local, args.rate, args.duration, policy=1 if args.policy == "shortest" else 0,
                        stop_rmse=args.stop_rmse, drain_s=args.drain, sah=args.sah)
        if rank == 0:
            print(json.dumps({"metric": "p99 job latency (served render jobs)", "value": out["p99_latency_ms"],
                              "unit": "ms", "higher_is_better": False, "n_gpus": world, "serving": out}), flush=True)
        return 0

    import torch
    b = importlib.import_module("sol-rs_gb300.build")
    b.build_lib()
    solrt = importlib.import_module("sol-rs_gb300")
    data, kw, cfg = workload(args.workload)
    if args.kernel == "mega":
        kw["kernel"] = solrt.KERNEL_MEGA
        cfg = dict(cfg, kernel="plain per-pixel megakernel (one thread loops samples and bounces)")
    if args.nee:
        kw["integrator"] = solrt.INTEGRATOR_PATH_NEE
        cfg = dict(cfg, integrator="path tracing + next-event estimation (shadow-ray queue)")
    for key in ("width", "height", "spp"):   # reduced sizes for profiler captures
        if getattr(args, key):
            kw[key] = getattr(args, key)
            cfg = dict(cfg, **{key: getattr(args, key)}, reduced=True)
    bvh = {"bvh2": solrt.BVH2, "bvh2q": solrt.BVH2_Q16, "bvh2t": solrt.BVH2_TWO_LEVEL, "bvh4": solrt.BVH4_Q8,
           "bvh8": solrt.BVH8_Q8, "bvh8f": solrt.BVH8_F32}[args.bvh]
    c = data.camera
    cam = solrt.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], kw["width"] / kw["height"])
    params = solrt.render_params(**kw)
    W, H = kw["width"], kw["height"]

    # visit counts per segment (one counting launch at reduced spp)
    with solrt.Context(local, enable_counters=True, path_capacity=args.capacity) as cctx:
        csc = solrt.SceneDescription(cctx, data, bvh=bvh, sah=args.sah)
        cimg = solrt.Image(cctx, W, H, kw["accum_mode"])
        cctx.reset_stats()
        # (the wavefront kernel counts visits; the megakernel's plain depth-first
        # loop visits the same nodes less the speculative ones)
        solrt.Renderer(cctx).cmd_trace_rays(csc, cam, solrt.render_params(
            **dict(kw, spp=min(4, kw["spp"]), kernel=solrt.KERNEL_WAVEFRONT)), cimg)
        cctx.synchronize()
        cs = cctx.stats()
        nodes_per_seg = cs.node_visits / max(cs.segments, 1)
        tris_per_seg = cs.tri_tests / max(cs.segments, 1)
        fb_per_seg = cs.fp64_fallbacks / max(cs.segments, 1)
        cimg.close()
        csc.close()

    ctx = solrt.Context(local, enable_timing=True, path_capacity=args.capacity)
    ctx_capacity = ctx.capacity()
    spp_per_pass = max(1, min(kw["spp"], ctx_capacity // (W * H)))
    passes_per_step = -(-kw["spp"] // spp_per_pass)
    sc = solrt.SceneDescription(ctx, data, bvh=bvh, sah=args.sah)
    info = sc.bvh_info()
    img = solrt.Image(ctx, W, H, kw["accum_mode"])
    r = solrt.Renderer(ctx)
    ext = torch.cuda.ExternalStream(ctx.stream())
    for i in range(args.warmup):
        r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(kw, frame=i)), img)
    ctx.synchronize()
    ctx.reset_stats()
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    clocks = ClockSampler(uuid or str(local))
    clocks.start()
    time.sleep(0.3)
    barrier(pg)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for i in range(args.steps):
        r.cmd_trace_rays(sc, cam, solrt.render_params(**dict(kw, frame=args.warmup + i)), img)
    e1.record(ext)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier(pg)
    ms = e0.elapsed_time(e1)
    st = ctx.stats()
    clk = clocks.stop()
    ms_max = max_over_ranks(pg, ms)
    seg_total = sum_over_ranks(pg, float(st.segments))
    shadow_total = sum_over_ranks(pg, float(st.shadow_segments))
    value = seg_total / (ms_max / 1000.0) / 1e6

    # end to end: render + read back the accumulation and RGBA8 images into pinned host memory
    e2e = None
    if not args.no_e2e:
        host_acc = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True)
        host_8 = torch.empty((H, W, 4), dtype=torch.uint8, pin_memory=True)
        acc_np, rgba_np = host_acc.numpy(), host_8.numpy()
        ctx.reset_stats()
        barrier(pg)
        t0 = time.perf_counter()
        for i in range(args.steps):
            p = solrt.render_params(**dict(kw, frame=args.warmup + args.steps + i))
            r.cmd_trace_rays(sc, cam, p, img)
            img.read_into(acc_np, rgba_np)
        dt = time.perf_counter() - t0
        barrier(pg)
        est = ctx.stats()
        dt_max = max_over_ranks(pg, dt)
        e2e_seg = sum_over_ranks(pg, float(est.segments))
        e2e = {"value": round(e2e_seg / dt_max / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": 256 + 64, "d2h_bytes_per_step": W * H * 20,
               "path": "solrt_render (camera + params from host) + solrt_image_read into pinned host buffers"}

    # instanced workload: the per-frame cost of moving every instance
    # (solrt_scene_set_instances + solrt_scene_regenerate, host-timed)
    regen = None
    if args.workload == "instances":
        S = solrt.scenes
        moved = S.instanced_soups(4, 16384, seed=5, angle=10.0).instances
        dyn = solrt.SceneDescription(ctx, data, bvh=bvh, keep_data=False, dynamic=True, sah=args.sah)
        regen = {}
        for name, mode in (("rebuild", solrt.REGEN_REBUILD), ("refit", solrt.REGEN_REFIT)):
            ts = []
            for i in range(7):
                dyn.set_instances(moved if i % 2 == 0 else data.instances)
                ctx.synchronize()
                t0 = time.perf_counter()
                dyn.tlas_regenerate(mode)
                ctx.synchronize()
                ts.append((time.perf_counter() - t0) * 1e3)
            regen[name + "_ms"] = round(float(np.median(ts[1:])), 3)
        dyn.close()

    # roofline of the extend kernel
    peak, peak_kind = peaks()
    b_seg = 32 + 16 + NODE_BYTES[info.kind] * nodes_per_seg + 48 * tris_per_seg
    ext_s = st.extend_ms / 1000.0
    if args.kernel == "mega":  # traversal and shading in one launch: the whole render time
        ext_s = ms / 1000.0
    # extend launches also trace the shadow rays of --nee (same bytes per ray assumed)
    achieved = ((st.segments + st.shadow_segments) * b_seg) / ext_s / 1e9 if ext_s > 0 else 0.0
    traffic = dram = None
    cap = EXTEND_CAPTURES.get((args.workload, "treelet" if args.sah else "lbvh"))
    if cap and info.kind == solrt.BVH2 and args.kernel != "mega" and not args.nee and ext_s > 0:
        seg_per_launch = st.segments / max(st.extend_launches, 1)
        traffic = round(cap["dram_bytes_per_segment"] * seg_per_launch)
        dram_gbs = cap["dram_bytes_per_segment"] * st.segments / ext_s / 1e9
        dram = {"bytes_per_segment": cap["dram_bytes_per_segment"], "gbs": round(dram_gbs, 1),
                "frac": round(dram_gbs / peak, 4), "source": cap["dram_source"],
                "how": "ncu DRAM bytes per segment of this workload's extend launches x this run's segments / "
                       "this run's extend time"}
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "frac_note": "achieved counts algorithmic bytes (node, triangle, ray and hit bytes of every visit) "
                             "with no cache reuse; L1 / L2 serve nearly all of them, so frac > 1 is not HBM "
                             "traffic: dram is what reaches HBM, limiter what binds" if cap else None,
                "dram": dram, "limiter": cap["limiter"] if (cap and dram) else None,
                "peak_source": peak_kind + " (MEASURED_PEAKS hbm_gbs)",
                "kernel": "k_megakernel (traversal + shading, whole render time)" if args.kernel == "mega"
                          else "k_extend (BVH traversal)", "bytes_per_segment": round(b_seg, 1),
                "nodes_per_segment": round(nodes_per_seg, 2), "tris_per_segment": round(tris_per_seg, 2),
                "extend_ms_per_launch": round(st.extend_ms / max(st.extend_launches, 1), 4),
                "stage_ms_per_step": {"generate": round(st.generate_ms / args.steps, 3),
                                      "extend": round(st.extend_ms / args.steps, 3),
                                      "shade": round(st.shade_ms / args.steps, 3),
                                      "accumulate_finalize": round(st.accumulate_ms / args.steps, 3)},
                "extend_share_of_step": round(st.extend_ms / ms, 4) if ms > 0 else None}
    if args.workload == "cornell":
        # a 32-triangle scene lives in L1 / L2: the HBM fraction says nothing,
        # so the same achieved bytes are set against the L2 copy bandwidth
        l2 = l2_copy_gbs(local)
        roofline["l2"] = {"peak": round(l2, 1), "unit": "GB/s", "frac": round(achieved / l2, 4) if l2 else None,
                          "peak_source": "measured here: 32 MB device-to-device copy, L2-resident, best of 20"}

    # RMSE of the device image against the FP64 oracle on the same RNG
    # streams, over a central band of rows (the oracle is the checker); the
    # tunnel accumulates four frames (its sun-lit sky makes FP32 and FP64
    # paths that part ways differ by a lot for a few samples)
    rmse = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            frames = 4 if args.workload == "tunnel" else 1
            band = {"soup": 32, "tunnel": 1}.get(args.workload, H // 2)
            rows = (max(0, H // 2 - band), min(H, H // 2 + band))
            rmse = rmse_vs_fp64(local, data, kw, cam, bvh, rows, frames=frames, sah=args.sah)
        except Exception as ex:
            rmse = {"error": str(ex)}
    img.close()
    sc.close()
    ctx.close()
    precision = None
    if rank == 0 and args.workload == "soup" and not args.no_precision:
        try:
            precision = precision_study(local, data, kw, cam, value / max(world, 1), info, nodes_per_seg, tris_per_seg,
                                        main_sah=args.sah, capacity=args.capacity)
        except Exception as ex:
            precision = {"error": str(ex)}
    # parity and convergence of the other single-scene configurations at
    # their stated sizes, and the workload under the reference shaders' own
    # settings next to those shaders on the host cores
    configs = refsem = None
    if rank == 0 and args.workload == "soup" and not args.no_precision:
        configs = {}
        for name, fn in (("cornell", parity_cornell), ("tunnel", parity_tunnel)):
            try:
                configs[name] = fn(local, capacity=args.capacity) if name == "tunnel" else fn(local)
            except Exception as ex:
                configs[name] = {"error": str(ex)}
        try:
            refsem = reference_semantics(local, data, kw, cam, sah=args.sah)
        except Exception as ex:
            refsem = {"error": str(ex)}
    # the other two parts of the headline metric, measured on smaller runs:
    # batched vs plain (first 32 jobs of the mixed-scene workload) and the
    # p99 latency of served jobs
    batched = serving = None
    if args.workload == "soup" and not args.no_serve:
        try:
            batched = run_batch(args, world, rank, local, pg, njobs=args.jobs, steps=1, emit=False, warmup=1)
        except Exception as ex:
            batched = {"error": str(ex)}
        try:
            serving = run_serve(local, args.rate, args.duration, policy=1 if args.policy == "shortest" else 0,
                                stop_rmse=args.stop_rmse, drain_s=args.drain, sah=args.sah)
        except Exception as ex:
            serving = {"error": str(ex)}
        # the same distribution at a rate the GPU keeps up with (about half
        # of what it traces), where p99 is a steady-state latency, not backlog
        if not args.no_serve_steady:
            try:
                serving["below_capacity"] = run_serve(local, args.steady_rate, args.steady_duration,
                                                      policy=1 if args.policy == "shortest" else 0,
                                                      stop_rmse=args.stop_rmse, drain_s=args.drain, seed=6,
                                                      sah=args.sah)
            except Exception as ex:
                serving["below_capacity"] = {"error": str(ex)}
    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            try:
                cpu = cpu_baseline(data, kw, cam)
            except Exception as ex:  # the CPU leg must not hide the GPU number
                cpu = {"error": str(ex)}
        out = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": run_config(cfg, args, world),
               "bvh": {"kind": args.bvh, "build_ms": round(info.build_ms, 3), "node_count": int(info.node_count)},
               "path_capacity": int(ctx_capacity), "passes_per_step": passes_per_step,
               "segments_per_step": int(st.segments // args.steps), "fp64_fallbacks_per_segment": fb_per_seg,
               "gpu_launches": int(st.launches), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "clocks": clk, "rmse_vs_fp64": rmse, "precision_study": precision, "batched_vs_plain": batched,
               "serving": serving, "configs_at_stated_size": configs, "reference_semantics": refsem}
        if regen is not None:
            out["regenerate_ms"] = regen
        if args.nee:
            out["shadow_rays"] = {"per_step": int(st.shadow_segments // args.steps),
                                  "mrays_s": round(shadow_total / (ms_max / 1000.0) / 1e6, 3),
                                  "unoccluded_frac": round(st.shadow_unoccluded / max(st.shadow_segments, 1), 4),
                                  "note": "not in value: the metric counts primary + bounce segments"}
        print(json.dumps(out), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
