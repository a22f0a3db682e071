"""Exact re-rank of continuous data: the CUDA path against the Float64 oracle.

The FP32 distance maps of the tensor cores (and of the SIMT kernel) differ from the Float64
distance by at most kappa (A^2 + B^2) + eabs, where kappa follows the arithmetic of the form
that computed the map (imagequilting.jl_gb300/csrc/iq_corr_tc.cu, iq_map_kappa). The pick
re-evaluates every position whose decision that error could change, up to the oracle's own
Float64 sequence (oracle/direct.c), so candidate sets, tau-model ranks, draws, cuts and whole
realizations equal the oracle's bit for bit on continuous data too; positions within 1e-6 of a
decision value are counted as near-ties, and the count equals the oracle's.
"""
import math

import numpy as np
import pytest

from oracle import iqsim_oracle as O

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def kappa(K, form):
    """Mirror of iq_map_kappa for continuous data (form 1: FP16 halves, 2: TF32, 0: SIMT)."""
    nsteps = math.ceil(K / 16) if form == 1 else math.ceil(K / 8) if form == 2 else 0
    acc = K if form == 0 else 3 * nsteps * 4
    return (acc + 24) * U * 1.01


@pytest.fixture(scope="module")
def ctx(iq):
    c = iq.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ctx_tf32(iq):
    c = iq.Context(0)
    c.set_option("corr.engine", 1)
    yield c
    c.close()


def _scale(ti, tmpl, w):
    ti = np.asarray(ti, np.float64)
    w = np.ones(tmpl.shape) if w is None else np.asarray(w, np.float64)
    return O.imfilter_valid_direct(ti ** 2, w) + np.sum(w * np.asarray(tmpl, np.float64) ** 2)


@pytest.mark.parametrize("form,spread", [(1, 1.0), (2, 1.0), (1, 2.5)])
def test_map_error_within_model_bound(iq, ctx, ctx_tf32, form, spread):
    """|D32 - D64| <= kappa (A^2 + B^2) on overlap-shaped masks: the bound the re-rank trusts,
    with margin (the observed ratio is printed)."""
    rng = np.random.default_rng(61)
    ti = np.exp(spread * rng.normal(size=(48, 44, 20))).astype(np.float32)
    tile = (12, 12, 6)
    w = np.ones(tile, bool)
    w[3:, 3:, 2:] = False  # tile minus an inner box, K = 864 - 9*9*4
    K = int(w.sum())
    worst = 0.0
    c = ctx if form == 1 else ctx_tf32
    for t in range(6):
        tmpl = np.exp(spread * rng.normal(size=tile)).astype(np.float32)
        got = iq.fastdistance(ti, tmpl, w, ctx=c).astype(np.float64)
        ref = O.fastdistance(ti, tmpl, w, "direct")
        ratio = np.max(np.abs(got - ref) / _scale(ti, tmpl, w))
        worst = max(worst, ratio)
    print("form %d: max |D32 - D64| / (A2 + B2) = %.3g, kappa = %.3g" % (form, worst,
                                                                        kappa(K, form)))
    assert worst <= kappa(K, form)


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x), np.asarray(y)), int(np.sum(np.asarray(x) != np.asarray(y)))


@pytest.mark.parametrize("case", ["3d", "2d", "3d_random", "3d_tol_wide"])
def test_iqsim_continuous_bit_exact(iq, ctx, case):
    """Whole continuous simulations equal the oracle (direct Float64 distances) bit for bit,
    realizations and boundary cuts, and the near-tie counts agree."""
    rng = np.random.default_rng(62)
    if case.startswith("3d"):
        ti = np.exp(rng.normal(size=(20, 20, 20))).astype(np.float32)
        tile, simsize = (8, 8, 6), (20, 20, 20)
    else:
        ti = np.exp(rng.normal(size=(40, 36))).astype(np.float32)
        tile, simsize = (10, 10), (44, 40)
    path = "random" if case == "3d_random" else "raster"
    tol = 0.6 if case == "3d_tol_wide" else 0.1
    g = iq.iqsim(ti, tile, simsize, overlap=(0.25,) * len(tile), tol=tol, path=path, nreal=3,
                 rng=17, debug=True, ctx=ctx)
    gt = ctx.ties
    ties = []
    r = O.iqsim(ti, tile, simsize, overlap=(0.25,) * len(tile), tol=tol, path=path, nreal=3,
                seed=17, debug=True, ties=ties)
    _same(g[0], r[0])
    _same(g[1], r[1])
    assert g[2] == r[2]
    assert gt == sum(ties)


def test_iqsim_continuous_hard_and_soft_bit_exact(iq, ctx):
    """Relaxation on continuous maps (hard data, a soft variable): every top-k boundary of the
    relaxation is refined; realizations and near-ties equal the oracle's."""
    rng = np.random.default_rng(63)
    ti = np.exp(rng.normal(size=(24, 22, 12))).astype(np.float32)
    simsize = (26, 24, 12)
    field = np.exp(rng.normal(size=simsize)).astype(np.float32)
    hard = {}
    for _ in range(12):
        c = tuple(int(rng.integers(0, s)) for s in simsize)
        hard[c] = float(field[c])
    aux = np.exp(0.5 * rng.normal(size=simsize)).astype(np.float32)
    auxti = np.exp(0.5 * rng.normal(size=ti.shape)).astype(np.float32)
    for kw in (dict(hard=hard), dict(soft=[(aux, auxti)]), dict(hard=hard, soft=[(aux, auxti)])):
        g = iq.iqsim(ti, (8, 8, 6), simsize, overlap=(0.25,) * 3, nreal=2, rng=29, ctx=ctx, **kw)
        gt = ctx.ties
        ties = []
        r = O.iqsim(ti, (8, 8, 6), simsize, overlap=(0.25,) * 3, nreal=2, seed=29, ties=ties, **kw)
        _same(g, r)
        assert gt == sum(ties)


def test_cfg2_sample_bit_exact(iq, ctx):
    """The benchmark's continuous workload (lognormal TI, 500 hard data, one soft variable),
    first 90 tiles of the data-first path for 2 realizations: equal to the oracle bit for bit,
    with the same near-tie count."""
    import bench
    W = bench.workload("cfg2")
    steps = 90
    ctx.set_option("sim.max_steps", steps)
    try:
        g = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], soft=W["soft"],
                     hard=W["hard"], tol=W["tol"], path=W["path"], nreal=2, rng=5, ctx=ctx)
        gt = ctx.ties
    finally:
        ctx.set_option("sim.max_steps", -1)
    ties = []
    r = O.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], soft=W["soft"],
                hard=W["hard"], tol=W["tol"], path=W["path"], nreal=2, seed=5, max_steps=steps,
                ties=ties)
    _same(g, r)
    assert gt == sum(ties)
    print("cfg2 sample: near-ties %d over %d picks" % (gt, len(ties)))


def test_pick_ties_match_oracle(iq, ctx):
    """Near-tie counts of iq_pick on given maps (taken as exact): threshold and relaxation."""
    rng = np.random.default_rng(64)
    P = 30000
    D = (rng.random(P) * 50 + 1).astype(np.float32)
    m = float(D.min())
    thr = (1 + 0.1) * m
    D[:40] = np.float32(thr * (1 + 3e-7))  # inside the window
    D[40:60] = np.float32(thr * (1 + 5e-6))  # outside it
    idx, c, w = iq.pick(D, [], 0.1, 3, 5, 1, ctx=ctx)
    ties = []
    O.pick(D.astype(np.float64), [], 0.1, 3, 5, 1, ties)
    assert ctx.ties == ties[0] and ties[0] >= 40
    S = (rng.random(P) * 9).astype(np.float32)
    iq.pick(D, [S], 0.1, 3, 5, 1, ctx=ctx)
    ties = []
    O.pick(D.astype(np.float64), [S.astype(np.float64)], 0.1, 3, 5, 1, ties)
    assert ctx.ties == ties[0]
