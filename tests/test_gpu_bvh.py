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
                                   lambda: S.tunnel(n_ang=128, n_ax=64, length=20.0),
                                   lambda: S.soup(1_000_000, seed=2), lambda: S.tunnel()],
                         ids=["cornell", "soup50k", "tunnel_small", "soup1M_full", "tunnel4M_full"])
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
        # node slots hold the exact boxes widened outward by a relative 2^-21
        # plus an absolute 2^-80
        step, tiny = np.float32(2.0 ** -21), np.float32(2.0 ** -80)
        want[:, :3] = (want[:, :3] - np.abs(want[:, :3]) * step) - tiny
        want[:, 3:] = (want[:, 3:] + np.abs(want[:, 3:]) * step) + tiny
        assert np.array_equal(cb, want)
    # triangle stream in leaf order carries the original triangle index
    prim = tris.view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(prim, order)
    info = sc.bvh_info()
    assert info.tri_count == n and info.node_count == n - 1 and info.depth >= np.log2(n)


def _decode_bvh2_q16(nodes_u8):
    """Header (G.xyz, c.xyz) + 32-byte nodes: refs, then per child x, y, z
    words of (low | high << 16) grid planes. Boxes as lo xyz, hi xyz (FP64)."""
    hdr = nodes_u8[:32].view(np.float32).astype(np.float64)
    g, c = hdr[0:3], hdr[3:6]
    w = nodes_u8[32:].view(np.uint32).reshape(-1, 8)
    refs = w[:, 0:2].view(np.int32)

    def box(words):
        lo = (words & 0xFFFF).astype(np.float64)
        hi = (words >> 16).astype(np.float64)
        return np.concatenate([g + lo * c, g + hi * c], 1)

    return g, c, refs, box(w[:, 2:5]), box(w[:, 5:8])


@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(50000, seed=2),
                                   lambda: S.tunnel(n_ang=128, n_ax=64, length=20.0), lambda: single_triangle()])
def test_bvh2_q16_conservative(solrt, ctx, maker):
    """BVH2-q16 nodes hold the FP32 BVH2's topology, and every quantised child
    box contains the FP32 (widened) child box with two to three cells of
    margin per face; the grid cell is a power of two with the scene's extent
    within 60000 cells."""
    d = maker()
    f = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2)
    q = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2_Q16)
    nf, tf = f.bvh_export()
    nq, tq = q.bvh_export()
    assert np.array_equal(tf, tq)
    assert q.bvh_info().node_count == f.bvh_info().node_count
    assert len(nq) == 32 * (q.bvh_info().node_count + 1)
    refs, c0, c1 = _decode_bvh2(nf)
    g, c, qrefs, q0, q1 = _decode_bvh2_q16(nq)
    assert np.array_equal(qrefs, refs)
    assert np.all(np.log2(c) == np.round(np.log2(c)))
    assert np.all(np.mod(g, c) == 0)
    for fb, qb in ((c0, q0), (c1, q1)):
        fb = fb.astype(np.float64)
        assert np.all(qb[:, :3] <= fb[:, :3] - 2 * c) and np.all(qb[:, 3:] >= fb[:, 3:] + 2 * c)
        slack = 3.0001 * c   # three cells, plus the outward rounding of lo - G / hi - G
        assert np.all(qb[:, :3] >= fb[:, :3] - slack) and np.all(qb[:, 3:] <= fb[:, 3:] + slack)
    lo = np.minimum(c0[:, :3].min(0), c1[:, :3].min(0)).astype(np.float64)
    hi = np.maximum(c0[:, 3:].max(0), c1[:, 3:].max(0)).astype(np.float64)
    assert np.all((hi - lo) / c <= 60001)


def _decode_bvh8(nodes_u8):
    w = nodes_u8.view(np.uint32).reshape(-1, 20)
    p = w[:, 0:3].copy().view(np.float32).astype(np.float64)
    e = np.stack([((w[:, 3] >> (8 * a)) & 0xFF).astype(np.uint8).view(np.int8) for a in range(3)], 1)
    imask = w[:, 3] >> 24
    scale = np.ldexp(1.0, e.astype(np.int64))

    def bytes8(c0, c1):
        b = np.stack([w[:, c0], w[:, c1]], 1).copy().view(np.uint8)
        return b.reshape(-1, 8).astype(np.float64)

    qlo = np.stack([bytes8(8, 9), bytes8(10, 11), bytes8(12, 13)], 2)     # node, slot, axis
    qhi = np.stack([bytes8(14, 15), bytes8(16, 17), bytes8(18, 19)], 2)
    lo = p[:, None, :] + qlo * scale[:, None, :]
    hi = p[:, None, :] + qhi * scale[:, None, :]
    meta = np.stack([w[:, 6], w[:, 7]], 1).copy().view(np.uint8).reshape(-1, 8)
    return dict(child_base=w[:, 4], tri_base=w[:, 5], imask=imask, meta=meta, lo=lo, hi=hi)


def _decode_bvh4(nodes_u8):
    """64-byte 4-wide nodes: p.xyz | e.xyz, imask; child_base, tri_base,
    meta[4], qlo.x[4]; qlo.y, qlo.z, qhi.x, qhi.y; qhi.z."""
    w = nodes_u8.view(np.uint32).reshape(-1, 16)
    p = w[:, 0:3].copy().view(np.float32).astype(np.float64)
    e = np.stack([((w[:, 3] >> (8 * a)) & 0xFF).astype(np.uint8).view(np.int8) for a in range(3)], 1)
    imask = w[:, 3] >> 24
    scale = np.ldexp(1.0, e.astype(np.int64))

    def bytes4(c):
        return w[:, c].copy().view(np.uint8).reshape(-1, 4).astype(np.float64)

    qlo = np.stack([bytes4(7), bytes4(8), bytes4(9)], 2)
    qhi = np.stack([bytes4(10), bytes4(11), bytes4(12)], 2)
    lo = p[:, None, :] + qlo * scale[:, None, :]
    hi = p[:, None, :] + qhi * scale[:, None, :]
    meta = w[:, 6].copy().view(np.uint8).reshape(-1, 4)
    return dict(child_base=w[:, 4], tri_base=w[:, 5], imask=imask, meta=meta, lo=lo, hi=hi)


def _decode_bvh8f(nodes_u8):
    """224-byte full-precision 8-wide nodes: child_base, tri_base, meta[8],
    imask, 3 pad words; then per axis lo[8], hi[8] (float32)."""
    w = nodes_u8.view(np.uint32).reshape(-1, 56)
    f = nodes_u8.view(np.float32).reshape(-1, 56).astype(np.float64)
    planes = f[:, 8:].reshape(-1, 3, 2, 8)                              # node, axis, lo/hi, slot
    meta = np.stack([w[:, 2], w[:, 3]], 1).copy().view(np.uint8).reshape(-1, 8)
    return dict(child_base=w[:, 0], tri_base=w[:, 1], imask=w[:, 4], meta=meta,
                lo=planes[:, :, 0, :].transpose(0, 2, 1), hi=planes[:, :, 1, :].transpose(0, 2, 1))


@pytest.mark.parametrize("sah", [False, True])
@pytest.mark.parametrize("width", [8, 4, "8f"])
@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(40000, seed=3),
                                   lambda: S.tunnel(n_ang=128, n_ax=64, length=20.0), lambda: single_triangle()])
def test_wide_bvh_conservative_and_complete(solrt, ctx, maker, width, sah):
    """Every triangle is referenced by exactly one leaf slot and lies inside
    the decoded (quantised) box of that slot and of every ancestor slot."""
    d = maker()
    kind = {8: solrt.BVH8_Q8, 4: solrt.BVH4_Q8, "8f": solrt.BVH8_F32}[width]
    sc = solrt.SceneDescription(ctx, d, bvh=kind, sah=sah)
    nodes, tris = sc.bvh_export()
    info = sc.bvh_info()
    n = info.tri_count
    dec = {8: _decode_bvh8, 4: _decode_bvh4, "8f": _decode_bvh8f}[width](nodes)
    width = 4 if width == 4 else 8
    tv = tris.view(np.float32).reshape(-1, 3, 4)[:, :, :3].astype(np.float64)
    prim = tris.view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(np.sort(prim), np.arange(n))
    seen = np.zeros(n, np.int64)
    stack = [(0, np.full(3, -np.inf), np.full(3, np.inf))]
    visited = 0
    while stack:
        node, alo, ahi = stack.pop()
        visited += 1
        for s in range(width):
            m = int(dec["meta"][node, s])
            if m == 0:
                continue
            blo = np.maximum(alo, dec["lo"][node, s])
            bhi = np.minimum(ahi, dec["hi"][node, s])
            if (int(dec["imask"][node]) >> s) & 1:
                rank = bin(int(dec["imask"][node]) & ((1 << s) - 1)).count("1")
                stack.append((int(dec["child_base"][node]) + rank, blo, bhi))
            else:
                k = bin(m >> 5).count("1")
                off = m & 31
                t0 = int(dec["tri_base"][node]) + off
                v = tv[t0:t0 + k]
                assert np.all(v >= blo - 0.0) and np.all(v <= bhi + 0.0), (node, s)
                seen[t0:t0 + k] += 1
    assert visited == info.node_count
    assert np.all(seen == 1)


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


def _wide_sah_cost(dec, tv, width, c_node=1.0, c_tri=0.3):
    """SAH cost of a decoded wide BVH with exact boxes (union of the
    triangles below each slot): A(node) c_node per node plus
    A(leaf) c_tri k per leaf slot of k triangles."""
    def half_area(lo, hi):
        e = hi - lo
        return e[0] * e[1] + e[1] * e[2] + e[2] * e[0]

    def walk(node):
        lo, hi, cost = np.full(3, np.inf), np.full(3, -np.inf), 0.0
        for s in range(width):
            m = int(dec["meta"][node, s])
            if m == 0:
                continue
            if (int(dec["imask"][node]) >> s) & 1:
                rank = bin(int(dec["imask"][node]) & ((1 << s) - 1)).count("1")
                clo, chi, cc = walk(int(dec["child_base"][node]) + rank)
                cost += cc
            else:
                k = bin(m >> 5).count("1")
                t0 = int(dec["tri_base"][node]) + (m & 31)
                v = tv[t0:t0 + k].reshape(-1, 3)
                clo, chi = v.min(0), v.max(0)
                cost += half_area(clo, chi) * c_tri * k
            lo, hi = np.minimum(lo, clo), np.maximum(hi, chi)
        return lo, hi, cost + half_area(lo, hi) * c_node

    return walk(0)[2]


@pytest.mark.parametrize("width", [8, 4])
@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(20000, seed=4),
                                   lambda: S.tunnel(n_ang=96, n_ax=48, length=20.0)])
def test_sah_collapse_not_worse_than_greedy(solrt, ctx, maker, width):
    """The SAH collapse minimises the SAH cost over all collapses of the
    binary tree (with leaves of <= leaf_max triangles), so its tree costs no
    more than the largest-child-first tree; both give the oracle's hits."""
    d = maker()
    kind = solrt.BVH8_Q8 if width == 8 else solrt.BVH4_Q8
    costs = {}
    for sah in (False, True):
        sc = solrt.SceneDescription(ctx, d, bvh=kind, sah=sah)
        nodes, tris = sc.bvh_export()
        dec = _decode_bvh8(nodes) if width == 8 else _decode_bvh4(nodes)
        tv = tris.view(np.float32).reshape(-1, 3, 4)[:, :, :3].astype(np.float64)
        costs[sah] = _wide_sah_cost(dec, tv, width)
    assert costs[True] <= costs[False] * (1 + 1e-5), costs


def _bvh2_sah_cost(refs, c0, c1, c_tri=0.3):
    """SAH cost (node visit 1, triangle test c_tri, per unit of surface area,
    over the root's area) of a decoded BVH2 from its (widened) child boxes."""
    def area(b):
        e = np.maximum(b[:, 3:] - b[:, :3], 0.0).astype(np.float64)
        return 2.0 * (e[:, 0] * e[:, 1] + e[:, 1] * e[:, 2] + e[:, 2] * e[:, 0])
    a0, a1 = area(c0), area(c1)
    root = area(np.concatenate([np.minimum(c0[:1, :3], c1[:1, :3]), np.maximum(c0[:1, 3:], c1[:1, 3:])], 1))[0]
    inner = (a0 * (refs[:, 0] >= 0)).sum() + (a1 * (refs[:, 1] >= 0)).sum() + root
    leaves = (a0 * (refs[:, 0] < 0)).sum() + (a1 * (refs[:, 1] < 0)).sum()
    return (inner + c_tri * leaves) / root


@pytest.mark.parametrize("maker", [lambda: S.cornell(), lambda: S.soup(50000, seed=2),
                                   lambda: S.tunnel(n_ang=256, n_ax=128, length=25.0), lambda: single_triangle(),
                                   lambda: S.soup(2, seed=4), lambda: S.soup(3, seed=4)],
                         ids=["cornell", "soup50k", "tunnel", "tri1", "tri2", "tri3"])
def test_bvh2_treelet_restructure(solrt, ctx, maker):
    """SOLRT_BVH_SAH on the binary kind restructures the LBVH by treelets:
    the same triangles in the same leaf order, every triangle in exactly one
    leaf, every child slot's (widened) box containing everything below it,
    a SAH cost no higher than the LBVH's, and the same bytes when built
    again."""
    d = maker()
    lb = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2)
    sb = solrt.SceneDescription(ctx, d, bvh=solrt.BVH2, sah=True)
    ln, lt = lb.bvh_export()
    sn, st = sb.bvh_export()
    assert np.array_equal(lt, st)              # leaf order and triangle stream unchanged
    n = sb.bvh_info().tri_count
    refs, c0, c1 = _decode_bvh2(sn)
    ni = refs.shape[0]
    assert ni == max(n - 1, 1) and sb.bvh_info().node_count == lb.bvh_info().node_count
    tv = st.view(np.float32).reshape(-1, 3, 4)[:, :, :3]
    tlo, thi = tv.min(1), tv.max(1)
    # every leaf once, every internal node but the root once as a child
    leaf = refs < 0
    pos = ~refs[leaf]
    if n > 1:
        assert np.array_equal(np.sort(pos), np.arange(n))
        inner = np.sort(refs[~leaf])
        assert np.array_equal(inner, np.arange(1, ni))
    # exact subtree boxes bottom-up (children have no fixed order: iterate
    # to a fixed point over the node list)
    lo = np.full((ni, 3), np.inf, np.float32)
    hi = np.full((ni, 3), -np.inf, np.float32)
    for _ in range(200):
        changed = False
        for side in (0, 1):
            r = refs[:, side]
            clo = np.where((r < 0)[:, None], tlo[np.where(r < 0, ~r, 0)], lo[np.where(r >= 0, r, 0)])
            chi = np.where((r < 0)[:, None], thi[np.where(r < 0, ~r, 0)], hi[np.where(r >= 0, r, 0)])
            nlo, nhi = np.minimum(lo, clo), np.maximum(hi, chi)
            changed |= not (np.array_equal(nlo, lo) and np.array_equal(nhi, hi))
            lo, hi = nlo, nhi
        if not changed:
            break
    for side, cb in ((0, c0), (1, c1)):
        r = refs[:, side]
        want_lo = np.where((r < 0)[:, None], tlo[np.where(r < 0, ~r, 0)], lo[np.where(r >= 0, r, 0)])
        want_hi = np.where((r < 0)[:, None], thi[np.where(r < 0, ~r, 0)], hi[np.where(r >= 0, r, 0)])
        assert np.all(cb[:, :3] <= want_lo) and np.all(cb[:, 3:] >= want_hi)
    if n > 2:
        lr, l0, l1 = _decode_bvh2(ln)
        assert _bvh2_sah_cost(refs, c0, c1) <= _bvh2_sah_cost(lr, l0, l1) * (1 + 1e-6)
    sb.tlas_regenerate()
    again, _ = sb.bvh_export()
    assert np.array_equal(again, sn)
    assert sb.bvh_info().depth <= 64
