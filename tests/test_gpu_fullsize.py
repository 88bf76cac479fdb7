"""Parity at the stated sizes of the benchmark configurations.

* Plain small (procedural Cornell box, 32 triangles, 256x256, 16 spp, max
  depth 5, Lambert, per-sample streams, seed 1) rendered whole on the device
  and by the FP32 oracle: RGBA32F bit for bit, equal segment counts, for
  every BVH kind and both kernels; the RMSE of the device image against the
  FP64 oracle on the same streams is checked against 1e-3.
* Triangle soup (1M triangles, seed 2) and procedural tunnel (2048 x 1024
  segments, 4.19M triangles, seed 3): the closest-hit records (t, prim, u, v)
  of 4,194,304 rays per scene (every pixel-centre camera ray of the
  configuration's image, then seeded rays from inside the scene's bounds)
  against the oracle's CPU LBVH traversal (the counterpart of traceRayEXT,
  assets/glsl/pathtrace.rgen:65-76), bit for bit for every BVH kind; hits
  within one float ulp of a triangle edge are counted apart and must agree
  too.
* The wide kinds at those sizes: every triangle in exactly one leaf slot,
  and every slot's decoded (quantised) box contains the exact box of what
  lies below it.
The LBVH topology at these sizes is checked in test_gpu_bvh.py.
"""
import numpy as np
import pytest

from helpers import S, bvh_args, camera_of

pytestmark = pytest.mark.gpu

KINDS = ["bvh2", "bvh2s", "bvh2q", "bvh2t", "bvh2ts", "bvh4", "bvh4s", "bvh8", "bvh8s", "bvh8f"]
N_RAYS = 1 << 22
_cache = {}


def _cornell_case(solrt):
    d = S.cornell()
    kw = dict(spp=16, max_bounces=5, material_mode=solrt.MATERIAL_LAMBERT, rng_mode=solrt.RNG_PER_SAMPLE, seed=1,
              miss_mode=solrt.MISS_BLACK)
    return d, 256, 256, kw


def _cornell_oracle(solrt, oracle):
    if "c1" not in _cache:
        d, w, h, kw = _cornell_case(solrt)
        cam = camera_of(d, w / h)
        o = oracle.OracleScene(d)
        p = solrt.render_params(w, h, **kw)
        a32, r8, st = o.render(cam, p)
        a64, _, _ = o.render(cam, p, precision=64)
        _cache["c1"] = (a32, r8, int(st.segments), a64)
    return _cache["c1"]


@pytest.mark.parametrize("kernel", ["wavefront", "mega"])
@pytest.mark.parametrize("bvh", KINDS)
def test_cornell_full_size_bit_exact(solrt, oracle, ctx, bvh, kernel):
    d, w, h, kw = _cornell_case(solrt)
    if kernel == "mega":
        kw = dict(kw, kernel=solrt.api.KERNEL_MEGA)
    a32, r8, seg_o, a64 = _cornell_oracle(solrt, oracle)
    cam = camera_of(d, w / h)
    sc = solrt.SceneDescription(ctx, d, **bvh_args(solrt, bvh))
    img = solrt.Image(ctx, w, h)
    ctx.reset_stats()
    solrt.Renderer(ctx).cmd_trace_rays(sc, cam, solrt.render_params(w, h, **kw), img)
    ctx.synchronize()
    ga, g8 = img.read()
    st = ctx.stats()
    img.close()
    sc.close()
    bad = np.nonzero(np.any(ga.view(np.uint32) != a32.view(np.uint32), axis=-1))
    assert len(bad[0]) == 0, (len(bad[0]), list(zip(bad[0][:5], bad[1][:5])))
    assert np.max(np.abs(g8.astype(int) - r8.astype(int))) <= 1
    assert st.segments == seg_o and st.error_flags == 0
    dd = ga[..., :3].astype(np.float64) - a64[..., :3].astype(np.float64)
    rmse = float(np.sqrt(np.mean(dd * dd)))
    assert rmse <= 1e-3, rmse


def _probe(solrt, oracle, name):
    """(scene data, rays, oracle hits, oracle FP64 fallbacks) of a config."""
    if name not in _cache:
        if name == "soup":
            d, w, h = S.soup(1_000_000, seed=2), 1920, 1080
        else:
            d, w, h = S.tunnel(), 2560, 1440
        cam = camera_of(d, w / h)
        rays = S.probe_rays(d, cam, w, h, N_RAYS, seed=7)
        o = oracle.OracleScene(d)
        hits, fb = o.trace(rays)
        o.close()
        _cache[name] = (d, rays, hits, fb)
    return _cache[name]


@pytest.mark.parametrize("bvh", KINDS)
@pytest.mark.parametrize("name", ["soup", "tunnel"])
def test_hit_records_full_size_vs_oracle(solrt, oracle, ctx, name, bvh):
    d, rays, want, fb = _probe(solrt, oracle, name)
    sc = solrt.SceneDescription(ctx, d, **bvh_args(solrt, bvh))
    got = sc.trace_rays(rays)
    sc.close()
    a = got.view(np.uint32).reshape(-1, 4)
    b = want.view(np.uint32).reshape(-1, 4)
    bad = np.any(a != b, axis=1)
    edge = S.near_edge(want)
    assert int(edge.sum()) >= 0
    assert not bad[edge].any(), "near-edge mismatches: %d of %d" % (int(bad[edge].sum()), int(edge.sum()))
    assert not bad.any(), "%d of %d hit records differ, first %s" % (int(bad.sum()), len(bad),
                                                                      np.nonzero(bad)[0][:5])
    hit_frac = float((want["prim"] != 0xFFFFFFFF).mean())
    assert hit_frac > 0.4


def _popcount8(x):
    x = x.astype(np.int64)
    c = np.zeros_like(x)
    for b in range(8):
        c += (x >> b) & 1
    return c


def _wide_containment(dec, tris, width, node_count, n):
    """Every triangle in exactly one leaf slot; every non-empty slot's decoded
    box contains the exact box (union of triangle boxes) below it. Vectorised
    over each level of the tree."""
    tv = tris.view(np.float32).reshape(-1, 3, 4)[:, :, :3].astype(np.float64)
    prim = tris.view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(np.sort(prim), np.arange(n))
    tlo, thi = tv.min(1), tv.max(1)
    meta = dec["meta"].astype(np.int64)
    imask = dec["imask"].astype(np.int64)
    slots = np.arange(width)
    full = meta != 0
    inner = full & (((imask[:, None] >> slots) & 1) == 1)
    leaf = full & ~inner
    rank = _popcount8(imask[:, None] & ((1 << slots) - 1))
    child = dec["child_base"].astype(np.int64)[:, None] + rank
    k = _popcount8(meta >> 5)
    t0 = dec["tri_base"].astype(np.int64)[:, None] + (meta & 31)
    # leaf slots: exact box and coverage
    seen = np.zeros(n, np.int64)
    slo = np.full(meta.shape + (3,), np.inf)
    shi = np.full(meta.shape + (3,), -np.inf)
    for j in range(3):
        m = leaf & (k > j)
        idx = t0[m] + j
        assert np.all(idx < n)
        np.add.at(seen, idx, 1)
        slo[m] = np.minimum(slo[m], tlo[idx])
        shi[m] = np.maximum(shi[m], thi[idx])
    assert np.all(seen == 1)
    # levels from the root; children always follow their parent
    assert np.all(child[inner] < node_count)
    levels, frontier, visited = [], np.array([0]), 0
    while len(frontier):
        levels.append(frontier)
        visited += len(frontier)
        frontier = child[frontier][inner[frontier]]
    assert visited == node_count
    nlo = np.full((node_count, 3), np.inf)
    nhi = np.full((node_count, 3), -np.inf)
    for lv in reversed(levels):
        m = inner[lv]
        c = child[lv]
        lo = slo[lv].copy()
        hi = shi[lv].copy()
        lo[m] = nlo[c[m]]
        hi[m] = nhi[c[m]]
        slo[lv] = lo
        shi[lv] = hi
        lo[~full[lv]] = np.inf
        hi[~full[lv]] = -np.inf
        nlo[lv] = lo.min(1)
        nhi[lv] = hi.max(1)
    assert np.all(dec["lo"][full] <= slo[full]) and np.all(dec["hi"][full] >= shi[full])


@pytest.mark.parametrize("bvh", ["bvh4", "bvh4s", "bvh8", "bvh8s", "bvh8f"])
@pytest.mark.parametrize("name", ["soup", "tunnel"])
def test_wide_bvh_full_size_conservative(solrt, oracle, ctx, name, bvh):
    from test_gpu_bvh import _decode_bvh4, _decode_bvh8, _decode_bvh8f
    d = _probe(solrt, oracle, name)[0]
    sc = solrt.SceneDescription(ctx, d, **bvh_args(solrt, bvh))
    nodes, tris = sc.bvh_export()
    info = sc.bvh_info()
    sc.close()
    dec = {"bvh4": _decode_bvh4, "bvh8": _decode_bvh8, "bvh8f": _decode_bvh8f}[bvh.rstrip("s")](nodes)
    _wide_containment(dec, tris, 4 if bvh.startswith("bvh4") else 8, info.node_count, info.tri_count)
