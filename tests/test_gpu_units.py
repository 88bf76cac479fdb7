"""Device unit functions against the oracle and the reference golden
vectors: TEA and nextRand bit-exact, sampling / Fresnel / miss bit-exact
against the oracle (same evaluation order, no contraction), sin/cos within
2 ulp-scale of CUDA's sinf/cosf, gamma within 1 ulp of the host pow."""
import json
import os
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "glsl_sampling.json")))


def bf(b):
    return struct.unpack("<f", struct.pack("<I", b))[0]


def test_tea_golden(ctx):
    a = np.array([r[0] for r in GOLD["tea"]], np.uint32)
    b = np.array([r[1] for r in GOLD["tea"]], np.uint32)
    want = np.array([r[2] for r in GOLD["tea"]], np.uint32)
    out = np.zeros(len(a), np.uint32)
    ctx.debug_unit(0, len(a), a=a, b=b, out_u=out)
    assert np.array_equal(out, want)


def test_next_rand_golden(ctx):
    for seq in GOLD["next_rand"]:
        n = len(seq["steps"])
        out = np.zeros(n, np.float32)
        st = np.zeros(1, np.uint32)
        ctx.debug_unit(1, 1, a=np.array([seq["seed"]], np.uint32), b=np.array([n], np.uint32), out_u=st, out_f=out)
        assert list(out.view(np.uint32)) == [s[0] for s in seq["steps"]]
        assert st[0] == seq["steps"][-1][1]


def test_sincos_bit_exact_vs_oracle_and_close_to_cuda(ctx, oracle):
    import torch
    x = np.linspace(0.0, 6.2831855, 20001, dtype=np.float32)
    out = np.zeros(2 * len(x), np.float32)
    ctx.debug_unit(2, len(x), fin=x, out_f=out)
    s, c = out[0::2], out[1::2]
    ref = np.array([oracle.sincos(float(v)) for v in x[::37]], np.float32)
    assert np.array_equal(s[::37], ref[:, 0]) and np.array_equal(c[::37], ref[:, 1])
    xt = torch.from_numpy(x).cuda()
    assert np.max(np.abs(torch.sin(xt).cpu().numpy() - s)) < 2.5e-7
    assert np.max(np.abs(torch.cos(xt).cpu().numpy() - c)) < 2.5e-7


def _vec_inputs(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3)).astype(np.float32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    m = rng.normal(size=(n, 3)).astype(np.float32)
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    fin = np.zeros((n, 8), np.float32)
    fin[:, :3] = v
    fin[:, 3:5] = rng.random((n, 2)).astype(np.float32)
    fin[:, 5] = (rng.random(n) ** 2).astype(np.float32)
    return fin, m


def test_sampling_bit_exact_vs_oracle(ctx, oracle):
    fin, _ = _vec_inputs(500, 1)
    out = np.zeros(3 * len(fin), np.float32)
    ctx.debug_unit(3, len(fin), fin=fin, out_f=out)
    ref = np.array([oracle.sample_ggx(r[:3], r[3], r[4], r[5]) for r in fin])
    assert np.array_equal(out.reshape(-1, 3), ref)
    ctx.debug_unit(4, len(fin), fin=fin, out_f=out)
    ref = np.array([oracle.sample_cosine(r[:3], r[3], r[4]) for r in fin])
    assert np.array_equal(out.reshape(-1, 3), ref)


def test_sampling_vs_reference_golden(ctx):
    recs = GOLD["sample_ggx"]
    fin = np.zeros((len(recs), 8), np.float32)
    for i, r in enumerate(recs):
        fin[i, :3] = [bf(x) for x in r[0]]
        fin[i, 3], fin[i, 4], fin[i, 5] = bf(r[1]), bf(r[2]), bf(r[3])
    out = np.zeros(3 * len(fin), np.float32)
    ctx.debug_unit(3, len(fin), fin=fin, out_f=out)
    want = np.array([[bf(x) for x in r[4]] for r in recs], np.float32)
    assert np.max(np.abs(out.reshape(-1, 3) - want)) <= 4e-7


def test_fresnel_and_miss_bit_exact(ctx, oracle, solrt):
    fin, m = _vec_inputs(300, 2)
    fin[:, 3:6] = m
    fin[:, 6] = np.float32(1.0) / np.float32(1.5)
    out = np.zeros(3 * len(fin), np.float32)
    ctx.debug_unit(5, len(fin), fin=fin, out_f=out)
    ref = np.array([oracle.fresnel(r[:3], r[3:6], r[6]) for r in fin], np.float32)
    assert np.array_equal(out[:len(fin)], ref)
    for mode in (solrt.MISS_BLACK, solrt.MISS_REF_SKY, solrt.MISS_GRADIENT):
        a = np.full(len(fin), mode, np.uint32)
        ctx.debug_unit(6, len(fin), a=a, fin=fin, out_f=out)
        ref = np.array([oracle.miss(r[:3], mode) for r in fin], np.float32)
        assert np.array_equal(out.reshape(-1, 3), ref)
    # the sun direction of pathtrace.rmiss:16 returns the sun colour
    sun = np.zeros((1, 8), np.float32)
    sun[0, :3] = np.array([0, 1, -0.25], np.float32) / np.float32(np.linalg.norm([0, 1, -0.25]))
    ctx.debug_unit(6, 1, a=np.array([solrt.MISS_REF_SKY], np.uint32), fin=sun, out_f=out)
    assert np.array_equal(out[:3], np.array([120, 100, 50], np.float32))


def test_gamma_close_to_host(ctx, oracle):
    x = np.concatenate([[0.0, 1.0, 0.5], np.random.default_rng(3).random(997)]).astype(np.float32)
    out = np.zeros(3 * len(x), np.float32)
    ctx.debug_unit(7, len(x), fin=x, out_f=out)
    ref = np.array([oracle.gamma(float(v)) for v in x], np.float32)
    assert np.max(np.abs(out[:len(x)].view(np.int32) - ref.view(np.int32))) <= 2
