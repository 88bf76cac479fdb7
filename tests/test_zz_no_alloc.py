"""The allocation-free BVH build (solrt_bvh2_build_noalloc).

Callers such as a real-time frame loop that rebuilds a moving mesh's BVH
every frame (where cudaMalloc / cudaFree could stall the whole device) or a
plugin that only receives device buffers from its host application cannot
allocate. This entry point builds the same BVH2 as the scene API with its
temporary data in a fixed scratch array inside the library. The test calls
it through the C ABI twice in a row on device buffers and compares both
results with the BVH that solrt_scene_create builds for the same triangles:
node array and leaf-ordered triangle stream must be identical bytes (the
build is deterministic). It also checks that a too-large request is
refused. This file is collected last so that a failure here comes after
every other test has run.
"""
import ctypes
import importlib

import numpy as np
import pytest

from helpers import S

pytestmark = pytest.mark.gpu


def _world_arrays(data):
    """World-space vertex positions (float4) and triangle records (uint4) as
    the scene upload builds them for identity instance transforms."""
    vpos, tri = [], []
    vb = 0
    for sec in data.sections:
        v = data.vertices["pos"][sec["vertex_offset"]:sec["vertex_offset"] + sec["vertex_count"], :3]
        p = np.zeros((len(v), 4), np.float32)
        p[:, :3] = v + np.float32(0.0)
        vpos.append(p)
        idx = data.indices[sec["index_offset"]:sec["index_offset"] + sec["index_count"]].reshape(-1, 3)
        t = np.zeros((len(idx), 4), np.uint32)
        t[:, :3] = idx + vb
        t[:, 3] = sec["material_index"]
        tri.append(t)
        vb += sec["vertex_count"]
    return np.concatenate(vpos), np.concatenate(tri)


def _bind(lib):
    fn = lib.solrt_bvh2_build_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    return fn


@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(60000, seed=5),
                                   lambda: S.tunnel(n_ang=128, n_ax=64, length=20.0)])
def test_noalloc_build_matches_scene_build(solrt, ctx, maker):
    import torch
    data = maker()
    sc = solrt.SceneDescription(ctx, data, bvh=solrt.BVH2)
    want_nodes, want_tris = sc.bvh_export()
    vpos, tri = _world_arrays(data)
    n = len(tri)
    assert n <= 65536
    dv = torch.from_numpy(vpos).cuda()
    dt = torch.from_numpy(tri.view(np.int32)).cuda()
    nodes = torch.empty(64 * max(n - 1, 1), dtype=torch.uint8, device="cuda")
    tris = torch.empty(48 * n, dtype=torch.uint8, device="cuda")
    fn = _bind(solrt.lib())
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        nodes.fill_(0xA5 + call)
        tris.fill_(0x5A + call)
        st = fn(dv.data_ptr(), dt.data_ptr(), n, nodes.data_ptr(), nodes.numel(), tris.data_ptr(), tris.numel(),
                stream)
        assert st == 0, solrt.lib().solrt_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(nodes.cpu().numpy(), want_nodes), "call %d: nodes differ" % call
        assert np.array_equal(tris.cpu().numpy(), want_tris), "call %d: triangles differ" % call
    sc.close()


def test_noalloc_single_triangle_on_default_stream(solrt, ctx):
    """One triangle (the single-node layout: a root whose two children are
    the same leaf) queued on the legacy default stream (stream = NULL)."""
    import torch
    data = S.soup(1, seed=9)
    sc = solrt.SceneDescription(ctx, data, bvh=solrt.BVH2)
    want_nodes, want_tris = sc.bvh_export()
    vpos, tri = _world_arrays(data)
    dv = torch.from_numpy(vpos).cuda()
    dt = torch.from_numpy(tri.view(np.int32)).cuda()
    nodes = torch.full((64,), 0xA5, dtype=torch.uint8, device="cuda")
    tris = torch.full((48,), 0x5A, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    fn = _bind(solrt.lib())
    for _ in range(2):
        st = fn(dv.data_ptr(), dt.data_ptr(), 1, nodes.data_ptr(), 64, tris.data_ptr(), 48, None)
        assert st == 0, solrt.lib().solrt_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(nodes.cpu().numpy(), want_nodes)
        assert np.array_equal(tris.cpu().numpy(), want_tris)
    sc.close()


def test_noalloc_rejects_too_many_triangles(solrt, ctx):
    fn = _bind(solrt.lib())
    st = fn(None, None, 65537, None, 0, None, 0, None)
    assert st == 5   # SOLRT_ERR_CAPACITY
    assert b"65536" in solrt.lib().solrt_last_error()
