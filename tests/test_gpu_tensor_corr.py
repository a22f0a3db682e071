"""Tensor-core (tcgen05) distance maps against the oracle and against the SIMT kernel.

The tensor-core kernel serves every mask of the form "tile minus a box" (overlap masks, the
full tile of soft data). `corr.engine`: 2 (default) FP16 halves with power-of-two scaling when
the data's range allows, else TF32 halves; 1 TF32 halves; 0 the SIMT kernel. Tolerance of a
distance map as in test_gpu_parity: 1e-5 * (A^2 + B^2). Integer-valued data are exact in every
engine, so the maps and whole realizations must then be identical.
"""
import numpy as np
import pytest

from oracle import iqsim_oracle as O

pytestmark = pytest.mark.gpu

DIST_RTOL = 1e-5


@pytest.fixture(scope="module")
def ctx(iq):
    c = iq.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ctx_simt(iq):
    c = iq.Context(0)
    c.set_option("corr.engine", 0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ctx_tf32(iq):
    c = iq.Context(0)
    c.set_option("corr.engine", 1)
    yield c
    c.close()


def _mask(tile, kind):
    if kind == "full":
        return None
    w = np.ones(tile, bool)
    if kind == "prev":  # overlap with the previous tiles along every axis (raster path)
        w[tuple(slice(max(1, t // 4), t) for t in tile)] = False
    else:  # overlap on both sides (random path): an inner box strictly inside
        w[tuple(slice(1, t - 1) if t > 2 else slice(0, t) for t in tile)] = False
    return w


def _scale(ti, tmpl, w):
    w = np.ones(tmpl.shape) if w is None else np.asarray(w, np.float64)
    return (O.imfilter_valid_direct(np.asarray(ti, np.float64) ** 2, w) +
            np.sum(w * np.asarray(tmpl, np.float64) ** 2))


@pytest.mark.parametrize("shape,tile,kind", [
    ((70, 40, 9), (30, 9, 4), "prev"),     # tile wider than one 24-offset group
    ((70, 40, 9), (30, 9, 4), "inner"),
    ((64, 33, 20), (12, 12, 6), "full"),
    ((90, 70), (25, 13), "prev"),
    ((300,), (49,), "full"),
])
def test_tensor_vs_oracle_continuous(iq, ctx, shape, tile, kind):
    rng = np.random.default_rng(31)
    ti = np.exp(rng.normal(size=shape)).astype(np.float32)
    tm = np.exp(rng.normal(size=(3,) + tile)).astype(np.float32)
    w = _mask(tile, kind)
    got = iq.fastdistance(ti, tm, w, ctx=ctx)
    for i in range(3):
        ref = O.fastdistance(ti, tm[i], w, "direct")
        err = np.abs(got[i].astype(np.float64) - ref) / _scale(ti, tm[i], w)
        assert err.max() <= DIST_RTOL, err.max()


def test_tensor_many_templates_exact(iq, ctx, ctx_simt):
    # 300 templates: two launches (256 + 48 columns, the last 4 padding)
    rng = np.random.default_rng(32)
    ti = rng.integers(0, 6, (40, 30, 8)).astype(np.float32)
    ti[3, 4, 2] = np.nan
    tm = rng.integers(-2, 5, (300, 9, 7, 3)).astype(np.float32)
    w = _mask((9, 7, 3), "prev")
    got = iq.fastdistance(ti, tm, w, ctx=ctx)
    simt = iq.fastdistance(ti, tm, w, ctx=ctx_simt)
    assert np.array_equal(got, simt)
    for i in (0, 137, 255, 256, 299):
        ref = O.fastdistance(np.nan_to_num(ti), tm[i], w, "direct")
        ref[O.finddisabled(ti, (9, 7, 3))] = np.inf
        assert np.array_equal(got[i], ref.astype(np.float32))


@pytest.mark.parametrize("kind", ["full", "prev", "inner"])
def test_tensor_matches_simt_continuous(iq, ctx, ctx_simt, kind):
    rng = np.random.default_rng(33)
    ti = rng.normal(size=(50, 44, 12)).astype(np.float32)
    tm = rng.normal(size=(20, 10, 10, 5)).astype(np.float32)
    w = _mask((10, 10, 5), kind)
    a = iq.fastdistance(ti, tm, w, ctx=ctx).astype(np.float64)
    b = iq.fastdistance(ti, tm, w, ctx=ctx_simt).astype(np.float64)
    for i in range(20):
        assert (np.abs(a[i] - b[i]) / _scale(ti, tm[i], w)).max() <= 2 * DIST_RTOL


@pytest.mark.parametrize("path", ["raster", "random"])
def test_iqsim_engines_identical_integer_ti(iq, ctx, ctx_simt, path):
    rng = np.random.default_rng(34)
    ti = rng.integers(0, 4, (30, 28, 14)).astype(np.float32)
    simsize = (40, 36, 14)
    hard = {(int(rng.integers(0, 40)), int(rng.integers(0, 36)), int(rng.integers(0, 14))):
            float(rng.integers(0, 4)) for _ in range(10)}
    aux = rng.integers(0, 5, simsize).astype(np.float32)
    auxti = rng.integers(0, 5, ti.shape).astype(np.float32)
    kw = dict(overlap=(0.25, 0.25, 0.25), path=path, nreal=3, rng=99, hard=hard,
              soft=[(aux, auxti)])
    a = iq.iqsim(ti, (9, 8, 6), simsize, ctx=ctx, **kw)
    b = iq.iqsim(ti, (9, 8, 6), simsize, ctx=ctx_simt, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float), equal_nan=True)
    r = O.iqsim(ti, (9, 8, 6), simsize, overlap=(0.25, 0.25, 0.25), path=path, nreal=3, seed=99,
                hard=hard, soft=[(aux, auxti)])
    for x, y in zip(a, r):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float), equal_nan=True)


@pytest.mark.parametrize("scale", [1.0, 1e5, 3e-4])
def test_fp16_and_tf32_vs_oracle_scaled(iq, ctx, ctx_tf32, scale):
    # values far from 1 exercise the power-of-two scaling of the FP16 halves
    rng = np.random.default_rng(35)
    ti = (scale * np.exp(rng.normal(size=(48, 40, 10)))).astype(np.float32)
    tm = (scale * np.exp(rng.normal(size=(4, 11, 9, 4)))).astype(np.float32)
    w = _mask((11, 9, 4), "prev")
    for c in (ctx, ctx_tf32):
        got = iq.fastdistance(ti, tm, w, ctx=c)
        for i in range(4):
            ref = O.fastdistance(ti, tm[i], w, "direct")
            err = np.abs(got[i].astype(np.float64) - ref) / _scale(ti, tm[i], w)
            assert err.max() <= DIST_RTOL, (scale, err.max())


def test_wide_range_falls_back_to_tf32(iq, ctx, ctx_tf32):
    # magnitudes spanning 2^30 are outside the FP16 halves' range: engine 2 must give the
    # TF32 result
    rng = np.random.default_rng(36)
    ti = (np.exp(rng.uniform(-10, 10, size=(40, 30, 8))) * rng.choice([-1, 1], (40, 30, 8))).astype(np.float32)
    tm = rng.normal(size=(3, 8, 6, 3)).astype(np.float32)
    w = _mask((8, 6, 3), "inner")
    a = iq.fastdistance(ti, tm, w, ctx=ctx)
    b = iq.fastdistance(ti, tm, w, ctx=ctx_tf32)
    assert np.array_equal(a, b)
    for i in range(3):
        ref = O.fastdistance(ti, tm[i], w, "direct")
        assert (np.abs(a[i].astype(np.float64) - ref) / _scale(ti, tm[i], w)).max() <= DIST_RTOL


@pytest.mark.parametrize("path", ["raster", "random"])
def test_iqsim_fp16_tf32_identical_integer_ti(iq, ctx, ctx_tf32, path):
    rng = np.random.default_rng(37)
    ti = rng.integers(0, 5, (28, 26, 12)).astype(np.float32)
    aux = rng.integers(0, 3, (34, 32, 12)).astype(np.float32)
    auxti = rng.integers(0, 3, ti.shape).astype(np.float32)
    kw = dict(overlap=(0.3, 0.3, 0.3), path=path, nreal=2, rng=7, soft=[(aux, auxti)])
    a = iq.iqsim(ti, (10, 9, 5), (34, 32, 12), ctx=ctx, **kw)
    b = iq.iqsim(ti, (10, 9, 5), (34, 32, 12), ctx=ctx_tf32, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float))


def test_engine_option_validation(iq, ctx):
    with pytest.raises(Exception):
        ctx.set_option("corr.engine", 3)


@pytest.fixture(scope="module")
def ctx_2streams(iq):
    c = iq.Context(0)
    c.set_option("sim.streams", 2)
    yield c
    c.close()


@pytest.mark.parametrize("path,nreal", [("raster", 3), ("random", 2), ("dilation", 5)])
def test_iqsim_one_and_two_streams_identical(iq, ctx, ctx_2streams, path, nreal):
    # two realization groups on two streams (uneven when nreal is odd) against one stream,
    # with hard and soft data; integer data make every distance exact, so realizations,
    # cuts and voxel reuse must be identical, and equal the oracle's
    rng = np.random.default_rng(38)
    ti = rng.integers(0, 4, (30, 26, 12)).astype(np.float32)
    simsize = (38, 34, 12)
    hard = {(int(rng.integers(0, 38)), int(rng.integers(0, 34)), int(rng.integers(0, 12))):
            float(rng.integers(0, 4)) for _ in range(12)}
    aux = rng.integers(0, 5, simsize).astype(np.float32)
    auxti = rng.integers(0, 5, ti.shape).astype(np.float32)
    kw = dict(overlap=(0.25, 0.25, 0.3), path=path, nreal=nreal, rng=5, hard=hard,
              soft=[(aux, auxti)], debug=True)
    a = iq.iqsim(ti, (9, 8, 5), simsize, ctx=ctx, **kw)
    b = iq.iqsim(ti, (9, 8, 5), simsize, ctx=ctx_2streams, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float), equal_nan=True)
    r = O.iqsim(ti, (9, 8, 5), simsize, overlap=(0.25, 0.25, 0.3), path=path, nreal=nreal,
                seed=5, hard=hard, soft=[(aux, auxti)])
    for x, y in zip(a[0] if isinstance(a, tuple) else a, r):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float), equal_nan=True)


def test_streams_option_validation(iq, ctx):
    for bad in (0, 3):
        with pytest.raises(Exception):
            ctx.set_option("sim.streams", bad)


@pytest.mark.parametrize("nreal", [1, 4])
def test_iqsim_single_tile(iq, ctx, nreal):
    # one tile: no overlap anywhere, so the tensor-core launches have columns but no stages
    rng = np.random.default_rng(39)
    ti = rng.integers(0, 3, (20, 18, 9)).astype(np.float32)
    a = iq.iqsim(ti, (8, 7, 4), (8, 7, 4), overlap=(0.25, 0.25, 0.25), nreal=nreal, rng=3, ctx=ctx)
    r = O.iqsim(ti, (8, 7, 4), (8, 7, 4), overlap=(0.25, 0.25, 0.25), nreal=nreal, seed=3)
    for x, y in zip(a, r):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float))


def test_iqsim_slabs_in_global_scratch(iq, ctx):
    # tile 32x32x16 with overlap 1/4: cut slabs of 8x32x16 = 4096 nodes need more than the
    # shared memory of a CTA, so the cut works on global scratch (the large-tile workload's case)
    rng = np.random.default_rng(40)
    ti = rng.integers(0, 4, (40, 40, 20)).astype(np.float32)
    kw = dict(overlap=(0.25, 0.25, 0.25), nreal=2)
    a = iq.iqsim(ti, (32, 32, 16), (56, 56, 16), rng=11, ctx=ctx, **kw)
    r = O.iqsim(ti, (32, 32, 16), (56, 56, 16), seed=11, **kw)
    for x, y in zip(a, r):
        assert np.array_equal(np.asarray(x, float), np.asarray(y, float))


def test_tensor_large_ti_streaming_stores(iq, ctx, ctx_simt):
    # a TI of 9 MB (4.1 M voxels, 1.9 M positions): many CTAs per z-plane and maps far larger
    # than the small cases
    rng = np.random.default_rng(41)
    ti = rng.integers(0, 5, (160, 160, 90)).astype(np.float32)
    assert ti.nbytes > 8 << 20
    tm = rng.integers(0, 5, (3, 8, 8, 4)).astype(np.float32)
    w = _mask((8, 8, 4), "prev")
    got = iq.fastdistance(ti, tm, w, ctx=ctx)
    simt = iq.fastdistance(ti, tm, w, ctx=ctx_simt)
    assert np.array_equal(got, simt)
    ref = O.fastdistance(ti, tm[1], w, "direct")
    assert np.array_equal(got[1], ref.astype(np.float32))
