"""GPU LBVH topology against the oracle's CPU LBVH: same Morton order, same
child references and bit-identical child boxes for every internal node."""
import numpy as np
import pytest

from helpers import S, single_triangle

pytestmark = pytest.mark.gpu


def _decode_bvh2(nodes_u8):
    n = nodes_u8.view(np.float32).reshape(-1, 16)
    refs = nodes_u8.view(np.int32).reshape(-1, 16)[:, 12:14]
    c0 = np.stack([n[:, 0], n[:, 2], n[:, 8], n[:, 1], n[:, 3], n[:, 9]], 1)   # lo xyz, hi xyz
    c1 = np.stack([n[:, 4], n[:, 6], n[:, 10], n[:, 5], n[:, 7], n[:, 11]], 1)
    return refs, c0, c1


def _oracle_refs(child):
    out = child.astype(np.int64)
    leaf = child >= 0x80000000
    out[leaf] = ~(child[leaf].astype(np.int64) & 0x7FFFFFFF)
    return out.astype(np.int32)


@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(50000, seed=2),
                                   lambda: S.tunnel(n_ang=128, n_ax=64, length=20.0)])
def test_bvh2_topology_bit_exact(solrt, oracle, ctx, maker):
    d = maker()
    sc = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2)
    nodes, tris = sc.bvh_export()
    o = oracle.OracleScene(d)
    child, boxes, order, morton = o.bvh()
    refs, c0, c1 = _decode_bvh2(nodes)
    n = o.tri_count
    assert refs.shape[0] == n - 1
    assert np.array_equal(refs, _oracle_refs(child))
    # child boxes: internal children carry the oracle node box, leaves the triangle box
    tw, _ = o.world()
    tri_lo = tw[:, :, 0, :3].min(1)
    tri_hi = tw[:, :, 0, :3].max(1)
    for side, cb in ((0, c0), (1, c1)):
        r = refs[:, side]
        internal = r >= 0
        want = np.zeros((len(r), 6), np.float32)
        want[internal] = boxes[r[internal]]
        lp = order[~r[~internal]]
        want[~internal, :3] = tri_lo[lp]
        want[~internal, 3:] = tri_hi[lp]
        assert np.array_equal(cb, want)
    # triangle stream in leaf order carries the original triangle index
    prim = tris.view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(prim, order)
    info = sc.bvh_info()
    assert info.tri_count == n and info.node_count == n - 1 and info.depth >= np.log2(n)


def test_single_triangle_bvh(solrt, ctx):
    sc = solrt.SceneDescription(ctx, single_triangle())
    info = sc.bvh_info()
    assert info.node_count == 1 and info.tri_count == 1


def test_rebuild_is_deterministic(solrt, ctx):
    d = S.soup(20000, seed=9)
    sc = solrt.SceneDescription(ctx, d)
    a, ta = sc.bvh_export()
    sc.tlas_regenerate()
    b, tb = sc.bvh_export()
    assert np.array_equal(a, b) and np.array_equal(ta, tb)
