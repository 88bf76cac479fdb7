"""Hit-record parity: the same ray file traced by the CUDA kernels and by the
oracle's brute force. Triangle index, t and barycentrics must match bit for
bit (watertight test with the same arithmetic, deterministic tie-break)."""
import numpy as np
import pytest

from helpers import (S, axis_rays, bvh_args, edge_rays, empty_scene, hit_mismatch, hits_equal, random_rays,
                     single_triangle, transformed_cornell)

pytestmark = pytest.mark.gpu


def _both(solrt, oracle, ctx, data, rays, bvh):
    sc = solrt.SceneDescription(ctx, data, **bvh)
    g = sc.trace_rays(rays)
    o = oracle.OracleScene(data, two_level=bvh["bvh"] == solrt.BVH2_TWO_LEVEL)
    ref, _ = o.trace(rays, brute=True)
    return g, ref


BVHS = ["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f", "bvh4s", "bvh8s"]


def _kind(solrt, name):
    return bvh_args(solrt, name)


@pytest.mark.parametrize("bvh", BVHS)
def test_cornell_random_and_edges(solrt, oracle, ctx, bvh):
    d = S.cornell()
    rays = np.concatenate([random_rays(30000, 0.01, 0.99, seed=11), edge_rays(d, 20000, seed=12),
                           edge_rays(d, 5000, seed=13, eye=d.camera["eye"]), axis_rays(0.0, 1.0, 5000, seed=14)])
    g, ref = _both(solrt, oracle, ctx, d, rays, _kind(solrt, bvh))
    bad = hit_mismatch(g, ref)
    assert len(bad) == 0, (bad[:10], g[bad[:5]], ref[bad[:5]])


@pytest.mark.parametrize("bvh", BVHS)
def test_soup_random_and_edges(solrt, oracle, ctx, bvh):
    d = S.soup(100000, seed=2)
    rays = np.concatenate([random_rays(20000, -0.2, 1.2, seed=21), edge_rays(d, 20000, seed=22),
                           axis_rays(0.0, 1.0, 4000, seed=23)])
    g, ref = _both(solrt, oracle, ctx, d, rays, _kind(solrt, bvh))
    assert hits_equal(g, ref), hit_mismatch(g, ref)[:10]


@pytest.mark.parametrize("bvh", BVHS)
def test_tunnel_small(solrt, oracle, ctx, bvh):
    d = S.tunnel(n_ang=256, n_ax=128, length=25.0)
    rng = np.random.default_rng(31)
    rays = random_rays(20000, -0.5, 0.5, seed=32)
    rays["origin"][:, 2] = rng.uniform(0, 25, len(rays))
    rays = np.concatenate([rays, edge_rays(d, 10000, seed=33, eye=(0.0, 0.0, 2.0))])
    g, ref = _both(solrt, oracle, ctx, d, rays, _kind(solrt, bvh))
    assert hits_equal(g, ref), hit_mismatch(g, ref)[:10]


@pytest.mark.parametrize("bvh", BVHS)
def test_transformed_sections(solrt, oracle, ctx, bvh):
    d = transformed_cornell()
    o = oracle.OracleScene(d)
    tw, _ = o.world()
    lo, hi = tw[..., 0, :3].reshape(-1, 3).min(0), tw[..., 0, :3].reshape(-1, 3).max(0)
    rays = random_rays(20000, 0.0, 1.0, seed=41)
    rays["origin"] = (lo + (hi - lo) * rays["origin"]).astype(np.float32)
    g, ref = _both(solrt, oracle, ctx, d, rays, _kind(solrt, bvh))
    assert hits_equal(g, ref)


@pytest.mark.parametrize("bvh", BVHS)
def test_empty_and_single(solrt, oracle, ctx, bvh):
    rays = random_rays(1000, -1, 1, seed=51)
    g, ref = _both(solrt, oracle, ctx, empty_scene(), rays, _kind(solrt, bvh))
    assert hits_equal(g, ref)
    assert np.all(g["prim"] == solrt.NO_HIT)
    d = single_triangle()
    rays = random_rays(5000, -0.5, 1.5, seed=52)
    rays = np.concatenate([rays, edge_rays(d, 2000, seed=53)])
    g, ref = _both(solrt, oracle, ctx, d, rays, _kind(solrt, bvh))
    assert hits_equal(g, ref)
    assert (g["prim"] == 0).sum() > 100


def test_zero_rays_and_device_api(solrt, ctx):
    import torch
    d = S.cornell()
    sc = solrt.SceneDescription(ctx, d)
    assert len(sc.trace_rays(np.zeros(0, solrt.RAY_DTYPE))) == 0
    rays = random_rays(4096, 0.05, 0.95, seed=61)
    host = sc.trace_rays(rays)
    dr = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    dh = torch.zeros(len(rays) * 16, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    sc.trace_rays_device(dr.data_ptr(), len(rays), dh.data_ptr())
    ctx.synchronize()
    dev = dh.cpu().numpy().view(solrt.HIT_DTYPE)
    assert hits_equal(host, dev)
    with pytest.raises(solrt.SolrtError) as e:  # refused before any launch
        sc.trace_rays_device(dr.data_ptr(), 1 << 31, dh.data_ptr())
    assert e.value.status == 1


def test_invalid_scene_rejected(solrt, ctx):
    d = S.cornell()
    d.indices[0] = 999
    with pytest.raises(solrt.SolrtError) as e:
        solrt.SceneDescription(ctx, d)
    assert e.value.status == 1
    d = S.cornell()
    d.sections["material_index"][0] = 50
    with pytest.raises(solrt.SolrtError):
        solrt.SceneDescription(ctx, d)
