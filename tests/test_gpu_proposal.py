"""The learned proposal (no counterpart in the reference): encoder kernels against the CPU oracle
(oracle/proposal_oracle.py), training, the shortlist path of iqsim and what training gains.

Tolerances: the inference encoder runs BF16 weights with FP32 accumulation and BF16 outputs, so
its embeddings match the Float64 oracle (given the same BF16-rounded weights) within 1e-2 of the
embedding's scale; the training kernels run FP32 weights, and the loss and every gradient tensor
match the oracle within 2e-3 (relative, 2-norm). A shortlist that holds every position gives
realizations equal to the full scan's bit for bit (same candidates, same draws).
"""
import math

import numpy as np
import pytest

from oracle import iqsim_oracle as O
from oracle import proposal_oracle as Q

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(iq):
    c = iq.Context(0)
    yield c
    c.close()


def _params(flat, tile):
    p, off = {}, 0
    for k, s in Q.param_shapes(tile).items():
        n = int(np.prod(s))
        p[k] = flat[off:off + n].astype(np.float64).reshape(s)
        off += n
    assert off == flat.size
    return p


def _bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def _window(ti, tile, dist, p):
    x, y, z = np.unravel_index(p, dist, order="F")
    return ti[x:x + tile[0], y:y + tile[1], z:z + tile[2]]


def _mask(tile, box):
    m = np.ones(tile, bool)
    m[box[0]:box[3], box[1]:box[4], box[2]:box[5]] = False
    return m


def _cat_ti(shape, seed, ncodes=4):
    import scipy.ndimage as ndi
    rng = np.random.default_rng(seed)
    f = np.stack([ndi.gaussian_filter(rng.standard_normal(shape), (4, 4, 2), mode="wrap")
                  for _ in range(ncodes)])
    return np.argmax(f, axis=0).astype(np.float32)


def test_encoder_forward_vs_oracle(iq, ctx):
    ti = _cat_ti((40, 36, 24), 1)
    tile = (16, 16, 8)
    box = (4, 4, 2, 16, 16, 8)
    ctx.set_ti(ti)
    ctx.lp_init(tile, seed=3)
    flat = ctx.lp_params()
    p = _params(_bf16(flat), tile)
    dist = tuple(T - t + 1 for T, t in zip(ti.shape, tile))
    pos = np.random.default_rng(2).integers(0, int(np.prod(dist)), 24)
    got = ctx.lp_embed(pos, box)
    m = _mask(tile, box)
    for i, q in enumerate(pos):
        X = Q.cell_features(_window(ti, tile, dist, q), m, tile)
        ref = Q.forward(p, X)[0]
        assert np.allclose(got[i], ref, rtol=1e-2, atol=1e-2 * np.abs(ref).max()), (i, got[i], ref)


def test_encoder_gradients_vs_oracle(iq, ctx):
    ti = _cat_ti((40, 36, 24), 2)
    tile = (16, 16, 8)
    box = (4, 4, 2, 16, 16, 8)
    ctx.set_ti(ti)
    ctx.lp_init(tile, seed=5)
    flat = ctx.lp_params()
    p = _params(flat, tile)
    dist = tuple(T - t + 1 for T, t in zip(ti.shape, tile))
    rng = np.random.default_rng(7)
    nA, nneg, temp = 3, 4, 8.0
    m = _mask(tile, box)
    apos = rng.integers(0, int(np.prod(dist)), nA)
    pos = rng.integers(0, int(np.prod(dist)), nA)
    neg = rng.integers(0, int(np.prod(dist)), nA * nneg)
    feats = lambda q: Q.cell_features(_window(ti, tile, dist, q), m, tile)  # noqa: E731
    A = np.stack([feats(q) for q in apos])
    loss, grad = ctx.lp_loss_grad(np.stack([a.reshape(3, -1, order="F") for a in A]).astype(np.float32),
                                  pos, neg, box, temp)
    ref_loss, ref_g = Q.batch_loss_and_grads(p, A, np.stack([feats(q) for q in pos]),
                                             np.stack([feats(q) for q in neg]).reshape(
                                                 (nA, nneg) + A.shape[1:]), temp)
    assert abs(loss - ref_loss) <= 2e-3 * max(1.0, abs(ref_loss))
    g = _params(grad, tile)
    for k in ref_g:
        num = np.linalg.norm(g[k] - ref_g[k])
        den = np.linalg.norm(ref_g[k])
        assert num <= 2e-3 * den + 1e-6, (k, num, den)


@pytest.mark.parametrize("ncodes", [4, 6])
def test_shortlist_of_every_position_equals_full_scan(iq, ctx, ncodes):
    """With a shortlist that holds every position the proposal's pick sees the full candidate
    set, so the realizations equal the full scan's; capture and training run on the way. Four
    codes are summed from the 2-bit plane form of the image, six from its byte form."""
    ti = _cat_ti((30, 28, 14), 3, ncodes)
    tile, simsize = (8, 8, 6), (30, 28, 14)
    kw = dict(overlap=(0.25, 0.25, 0.34), nreal=3, rng=9, ctx=ctx)
    ctx.set_ti(ti)
    ctx.lp_init(tile, seed=1)
    ctx.set_option("lp.capture", 4000)
    full = iq.iqsim(ti, tile, simsize, **kw)
    assert ctx.lp_stats()["captured"] > 0
    l0, l1 = ctx.lp_train(60, batch=64, nneg=16, lr=2e-3, temp=8.0, seed=4)
    assert np.isfinite(l0) and np.isfinite(l1)
    ctx.set_option("lp.capture", 0)
    ctx.set_option("lp.enable", 1)
    ctx.set_option("lp.k", 1 << 20)
    ctx.set_option("lp.monitor", 1)
    try:
        lp = iq.iqsim(ti, tile, simsize, **kw)
        st = ctx.lp_stats()
    finally:
        ctx.set_option("lp.enable", 0)
        ctx.set_option("lp.k", 8192)
        ctx.set_option("lp.monitor", 16)
    assert st["cols_shortlist"] > 0 and st["recall"] == 1.0 and st["fell_back"] == 0
    for a, b in zip(full, lp):
        assert np.array_equal(np.ma.getdata(a), np.ma.getdata(b))
    # the oracle agrees with both
    r = O.iqsim(ti, tile, simsize, overlap=(0.25, 0.25, 0.34), nreal=3, seed=9)
    for a, b in zip(lp, r):
        assert np.array_equal(np.ma.getdata(a), b)


def test_training_gains_recall(iq, ctx):
    """Ablation: at the same shortlist length the trained encoder recalls more of the exact
    candidate sets than the untrained one (recall measured against the full scan)."""
    ti = _cat_ti((96, 96, 40), 11)
    tile, simsize = (16, 16, 8), (64, 64, 24)
    kw = dict(overlap=(0.25, 0.25, 0.25), nreal=4, ctx=ctx)
    ctx.set_ti(ti)
    ctx.lp_init(tile, seed=2)
    untrained = ctx.lp_params()

    def recall(params):
        ctx.lp_set_params(tile, params)
        ctx.set_option("lp.enable", 1)
        ctx.set_option("lp.k", 1024)
        ctx.set_option("lp.monitor", 1)
        ctx.set_option("lp.fallback", 0)
        try:
            iq.iqsim(ti, tile, simsize, rng=777, **kw)
            return ctx.lp_stats()
        finally:
            ctx.set_option("lp.enable", 0)
            ctx.set_option("lp.fallback", 1)
            ctx.set_option("lp.monitor", 16)
            ctx.set_option("lp.k", 8192)

    r0 = recall(untrained)
    ctx.set_option("lp.capture", 20000)
    for s in range(1, 6):
        iq.iqsim(ti, tile, simsize, rng=s, **kw)
    l0, l1 = ctx.lp_train(300, batch=128, nneg=32, lr=2e-3, temp=8.0, seed=6)
    ctx.set_option("lp.capture", 0)
    trained = ctx.lp_params()
    r1 = recall(trained)
    print("loss %.3f -> %.3f; recall untrained %.3f, trained %.3f (shortlist %d of %d)" % (
        l0, l1, r0["recall"], r1["recall"], r1["mean_shortlist"], 81 * 81 * 33))
    assert l1 < l0
    assert r1["monitored"] > 0 and r1["recall"] > r0["recall"]
