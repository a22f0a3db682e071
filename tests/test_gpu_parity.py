"""CUDA path vs the CPU oracle, through the C ABI (libiqgpu.so).

Tolerances (stated by the specification of this path):
  * distance maps: |D_gpu - D_oracle| <= 1e-5 * (A^2 + B^2), the scale of the terms, where
    A^2 = sum_k w_k TI[p+k]^2 and B^2 = sum_k w_k tmpl_k^2 (the FP32 correlation cancels);
  * candidate sets, tau-model weights, drawn indices and cut masks: bit-exact given the same
    distance map (or the same A/B arrays) and seed;
  * whole realizations: bit-exact on integer-valued training images, where every distance
    is an exact integer in FP32 and FP64.
"""
import os

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


def _scale(ti, tmpl, w):
    ti = np.asarray(ti, np.float64)
    w = np.ones(tmpl.shape) if w is None else np.asarray(w, np.float64)
    return O.imfilter_valid_direct(ti ** 2, w) + np.sum(w * np.asarray(tmpl, np.float64) ** 2)


# ---- a7/a8: distance maps --------------------------------------------------------------
@pytest.mark.parametrize("shape,tile,kind", [
    ((60, 50), (12, 10), "full"), ((60, 50), (12, 10), "box"), ((60, 50), (12, 10), "sparse"),
    ((30, 28, 16), (8, 7, 5), "full"), ((30, 28, 16), (8, 7, 5), "box"),
    ((30, 28, 16), (8, 7, 5), "sparse"), ((200,), (17,), "full"),
])
def test_fastdistance_vs_oracle(iq, ctx, shape, tile, kind):
    rng = np.random.default_rng(11)
    ti = np.exp(rng.normal(size=shape)).astype(np.float32)
    tmpl = np.exp(rng.normal(size=tile)).astype(np.float32)
    if kind == "full":
        w = None
    elif kind == "box":  # tile minus an inner box (overlap mask shape)
        w = np.ones(tile, bool)
        inner = tuple(slice(max(1, t // 4), t) for t in tile)
        w[inner] = False
    else:
        w = rng.random(tile) < 0.05
        w.flat[0] = True
    got = iq.fastdistance(ti, tmpl, w, ctx=ctx)
    ref = O.fastdistance(ti, tmpl, w, "direct")
    assert got.shape == ref.shape
    err = np.abs(got.astype(np.float64) - ref) / _scale(ti, tmpl, w)
    assert err.max() <= DIST_RTOL, err.max()


def test_fastdistance_batch_and_disabled(iq, ctx):
    rng = np.random.default_rng(12)
    ti = rng.integers(0, 4, (40, 36, 12)).astype(np.float32)
    ti[5, 7, 3] = np.nan
    tm = rng.integers(0, 4, (16, 10, 9, 4)).astype(np.float32)
    got = iq.fastdistance(ti, tm, ctx=ctx)
    for i in range(16):
        ref = O.fastdistance(np.nan_to_num(ti), tm[i], None, "direct")
        ref[O.finddisabled(ti, tm[i].shape)] = np.inf
        assert np.array_equal(got[i], ref.astype(np.float32))  # integer data: exact


def test_finddisabled(iq, ctx):
    ti = np.ones((20, 20, 20))
    ti[:, 4, :] = np.nan
    ti[3, 17, 11] = np.nan
    assert np.array_equal(iq.finddisabled(ti, (10, 10, 10), ctx=ctx), O.finddisabled(ti, (10, 10, 10)))


# ---- a12-a15: pick ----------------------------------------------------------------------
def _pick_both(iq, ctx, D, Ds, tol, seed, tile, real):
    gi, gc, gw = iq.pick(D, Ds, tol, seed, tile, real, ctx=ctx)
    D64 = np.asarray(D, np.float32).astype(np.float64)
    Ds64 = [np.asarray(x, np.float32).astype(np.float64) for x in Ds]
    ri, rc, rw = O.pick(D64, Ds64, tol, seed, tile, real)
    return (gi, gc, gw), (ri, rc, rw)


@pytest.mark.parametrize("case", ["continuous", "ties", "allzero", "disabled", "single"])
def test_threshold_pick_bit_exact(iq, ctx, case):
    rng = np.random.default_rng(13)
    P = 5000
    if case == "continuous":
        D = rng.random(P).astype(np.float32) * 100 + 1
    elif case == "ties":
        D = rng.integers(0, 6, P).astype(np.float32)
        D[D == 0] = 1
    elif case == "allzero":
        D = np.zeros(P, np.float32)
    elif case == "disabled":
        D = rng.random(P).astype(np.float32) + 0.5
        D[rng.random(P) < 0.3] = np.inf
    else:
        D = rng.random(P).astype(np.float32) + 1
        D[1234] = 0.1
    for seed in (0, 7, 2 ** 40 + 3):
        g, r = _pick_both(iq, ctx, D, [], 0.1, seed, 17, 3)
        assert np.array_equal(g[1], r[1])
        assert np.array_equal(g[2], r[2])  # FP64 weights, bit for bit
        assert g[0] == r[0]


@pytest.mark.parametrize("naux,case", [(1, "continuous"), (2, "continuous"), (1, "allzero"),
                                       (1, "ties"), (2, "disabled")])
def test_relaxation_pick_bit_exact(iq, ctx, naux, case):
    rng = np.random.default_rng(14 + naux)
    P = 20000
    D = (rng.random(P) * 50).astype(np.float32)
    if case == "allzero":
        D[:] = 0
    if case == "ties":
        D = rng.integers(0, 20, P).astype(np.float32)
    Ds = [(rng.random(P) * 10).astype(np.float32) for _ in range(naux)]
    if case == "ties":
        Ds = [rng.integers(0, 50, P).astype(np.float32) for _ in range(naux)]
    if case == "disabled":
        dis = rng.random(P) < 0.2
        D[dis] = np.inf
        for x in Ds:
            x[dis] = np.inf
    for seed, tol in ((1, 0.1), (99, 0.05), (5, 1.0)):
        g, r = _pick_both(iq, ctx, D, Ds, tol, seed, 3, 0)
        assert np.array_equal(g[1], r[1])
        assert np.array_equal(g[2], r[2])
        assert g[0] == r[0]


def test_pick_large_candidate_set(iq, ctx):
    # first tile of a realization: every enabled window is a candidate (D == 0)
    P = 231231
    D = np.zeros(P, np.float32)
    D[::97] = np.inf
    g, r = _pick_both(iq, ctx, D, [], 0.1, 42, 0, 5)
    assert len(g[1]) == len(r[1]) == P - len(D[::97])
    assert np.array_equal(g[1], r[1]) and g[0] == r[0]
    S = (np.random.default_rng(3).random(P) * 7).astype(np.float32)
    S[::97] = np.inf
    g, r = _pick_both(iq, ctx, D, [S], 0.1, 42, 0, 5)
    assert np.array_equal(g[1], r[1]) and np.array_equal(g[2], r[2]) and g[0] == r[0]


# ---- a16: graph cut -----------------------------------------------------------------------
def test_graphcut_known_answer(iq, ctx):
    A, B = np.ones((20, 20)), np.ones((20, 20))
    C = iq.graphcut(A, B, 0, ctx=ctx)
    assert np.all(C[:-1, :]) and not np.any(C[-1, :])
    C = iq.graphcut(A, B, 1, ctx=ctx)
    assert np.all(C[:, :-1]) and not np.any(C[:, -1])


@pytest.mark.parametrize("shape,dim", [((6, 32), 0), ((32, 6), 1), ((6, 24, 12), 0),
                                       ((24, 6, 12), 1), ((24, 24, 3), 2), ((8, 32, 16), 0),
                                       ((2, 10, 5), 0), ((3, 9), 0)])
def test_graphcut_continuous_bit_exact(iq, ctx, shape, dim):
    rng = np.random.default_rng(15)
    for trial in range(4):
        A = np.exp(rng.normal(size=shape)).astype(np.float32)
        B = np.exp(rng.normal(size=shape)).astype(np.float32)
        g = iq.graphcut(A, B, dim, ctx=ctx)
        r = O.graphcut(A, B, dim)
        assert np.array_equal(g, r), (trial, np.sum(g != r))


@pytest.mark.parametrize("shape,dim", [((6, 24, 12), 0), ((24, 24, 3), 2), ((6, 32), 0)])
def test_graphcut_categorical_ties(iq, ctx, shape, dim):
    rng = np.random.default_rng(16)
    for trial in range(6):
        A = rng.integers(0, 4, shape).astype(np.float32)
        B = rng.integers(0, 4, shape).astype(np.float32)
        g = iq.graphcut(A, B, dim, ctx=ctx)
        r = O.graphcut(A, B, dim)
        assert np.isclose(O.cut_cost(A, B, g), O.cut_cost(A, B, r), rtol=1e-12, atol=0)
        assert np.array_equal(g, r)


# ---- the whole iqsim --------------------------------------------------------------------
def _same_reals(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        x = np.ma.filled(x.astype(float), np.nan) if np.ma.isMaskedArray(x) else np.asarray(x, float)
        y = np.ma.filled(y.astype(float), np.nan) if np.ma.isMaskedArray(y) else np.asarray(y, float)
        assert np.array_equal(x, y, equal_nan=True), np.sum(x != y)


@pytest.mark.parametrize("case", ["2d", "3d", "3d_random", "3d_dilation", "2d_nreal3"])
def test_iqsim_bit_exact_integer_ti(iq, ctx, case):
    rng = np.random.default_rng(21)
    if case.startswith("2d"):
        ti = (rng.random((48, 40)) < 0.4).astype(np.float32)
        args = dict(tilesize=(12, 12), simsize=(60, 50))
    else:
        ti = rng.integers(0, 3, (24, 22, 14)).astype(np.float32)
        args = dict(tilesize=(8, 8, 6), simsize=(30, 28, 14))
    path = {"3d_random": "random", "3d_dilation": "dilation"}.get(case, "raster")
    nreal = 3 if case.endswith("nreal3") else 2
    g = iq.iqsim(ti, args["tilesize"], args["simsize"], path=path, nreal=nreal, rng=1234,
                 debug=True, ctx=ctx)
    r = O.iqsim(ti, args["tilesize"], args["simsize"], path=path, nreal=nreal, seed=1234, debug=True)
    _same_reals(g[0], r[0])
    _same_reals(g[1], r[1])
    assert np.allclose(g[2], r[2], rtol=0, atol=0)


@pytest.mark.parametrize("data", ["int", "hard_soft"])
def test_iqsim_shards_equal_whole_call(iq, ctx, data):
    """Two shards of one call (real0 = 0 and 3), run one after the other on this GPU, equal
    the whole 5-realization call bit for bit; the oracle agrees with the shards."""
    rng = np.random.default_rng(24)
    ti = rng.integers(0, 4, (22, 20, 12)).astype(np.float32)
    simsize = (26, 24, 12)
    kw = dict(overlap=(0.25, 0.25, 0.25))
    if data == "hard_soft":
        kw["hard"] = {(3, 4, 5): 1.0, (20, 11, 2): 3.0}
        kw["soft"] = [(rng.integers(0, 5, simsize).astype(np.float32),
                       rng.integers(0, 5, ti.shape).astype(np.float32))]
    whole = iq.iqsim(ti, (8, 8, 6), simsize, nreal=5, rng=13, ctx=ctx, **kw)
    parts = []
    for rank in range(2):
        r0, local = iq.iqsim_shard(iq.iqsim, ti, (8, 8, 6), simsize, nreal=5, rank=rank, world=2,
                                   rng=13, ctx=ctx, **kw)
        parts.append((r0, local))
    assert [r0 for r0, _ in parts] == [0, 3]
    _same_reals(parts[0][1] + parts[1][1], whole)
    r = O.iqsim(ti, (8, 8, 6), simsize, nreal=2, real0=3, seed=13, **kw)
    _same_reals(parts[1][1], r)


def test_iqsim_bit_exact_hard_and_soft(iq, ctx):
    rng = np.random.default_rng(22)
    ti = rng.integers(0, 4, (22, 20, 12)).astype(np.float32)
    simsize = (26, 24, 12)
    hard = {}
    for _ in range(15):
        c = tuple(int(rng.integers(0, s)) for s in simsize)
        hard[c] = float(rng.integers(0, 4))
    hard[(0, 0, 0)] = np.nan
    aux = rng.integers(0, 5, simsize).astype(np.float32)
    auxti = rng.integers(0, 5, ti.shape).astype(np.float32)
    for kw in (dict(hard=hard), dict(soft=[(aux, auxti)]), dict(hard=hard, soft=[(aux, auxti)])):
        g = iq.iqsim(ti, (8, 8, 6), simsize, overlap=(0.25, 0.25, 0.25), nreal=2, rng=77,
                     ctx=ctx, **kw)
        r = O.iqsim(ti, (8, 8, 6), simsize, overlap=(0.25, 0.25, 0.25), nreal=2, seed=77, **kw)
        _same_reals(g, r)


def test_iqsim_continuous_close(iq, ctx):
    # continuous data: FP32 vs FP64 distances may flip near-tied candidates, so compare
    # the statistics of the realizations instead of the values
    rng = np.random.default_rng(23)
    ti = np.exp(rng.normal(size=(40, 36, 10))).astype(np.float32)
    g = iq.iqsim(ti, (10, 10, 5), (40, 36, 10), nreal=2, rng=5, ctx=ctx)
    vals = set(np.unique(ti))
    for x in g:
        assert x.dtype == np.float32 and set(np.unique(x)) <= vals


# ---- the reference's own test suite (test/runtests.jl) through the CUDA path --------------
def test_runtests_basic(iq, ctx):
    TI = np.ones((20, 20, 20))
    reals = iq.iqsim(TI, (10, 10, 10), TI.shape, ctx=ctx)
    assert reals[0].dtype == np.float64 and np.array_equal(reals[0], TI)
    TI = np.random.default_rng(1).random((20, 20, 20)).astype(np.float32)
    assert iq.iqsim(TI, (10, 10, 10), TI.shape, ctx=ctx)[0].dtype == np.float32
    TI = np.random.default_rng(2).integers(1, 4, (20, 20, 20))
    r = iq.iqsim(TI, (10, 10, 10), TI.shape, ctx=ctx)[0]
    assert np.ma.isMaskedArray(r) and r.dtype == TI.dtype
    assert set(np.unique(r.compressed())) <= set(np.unique(TI))


def test_runtests_soft(iq, ctx):
    TI = np.concatenate([np.zeros((10, 20, 1)), np.ones((10, 20, 1))], axis=0)
    trend = np.concatenate([np.zeros((20, 10, 1)), np.ones((20, 10, 1))], axis=1)
    reals = iq.iqsim(TI, (10, 10, 1), TI.shape, soft=[(trend, TI)], tol=1, ctx=ctx)
    assert reals[0][:, :10, :].mean() <= reals[0][:, 10:, :].mean()
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    aux = np.full(TI.shape, 1.0)
    iq.iqsim(TI, (10, 10, 10), TI.shape, soft=[(aux, aux)], ctx=ctx)
    assert np.array_equal(aux, np.full(TI.shape, 1.0))


def test_runtests_hard(iq, ctx):
    TI = np.ones((20, 20, 20))
    obs = np.zeros(TI.shape)
    data = {c: obs[c] for c in np.ndindex(*TI.shape)}
    assert np.array_equal(iq.iqsim(TI, (10, 10, 10), TI.shape, hard=data, ctx=ctx)[0], obs)
    reals = iq.iqsim(TI, (10, 10, 10), TI.shape, hard={(19, 19, 19): 10}, nreal=3, ctx=ctx)
    assert all(r[19, 19, 19] == 10 for r in reals)


def test_runtests_masked(iq, ctx):
    TI = np.ones((20, 20, 20))
    shape, active = {}, np.ones(TI.shape, bool)
    for i, j, k in np.ndindex(20, 20, 20):
        if (i - 9) ** 2 + (j - 9) ** 2 + (k - 9) ** 2 < 25:
            shape[(i, j, k)] = np.nan
            active[i, j, k] = False
    r = iq.iqsim(TI, (10, 10, 10), TI.shape, hard=shape, ctx=ctx)[0]
    assert np.all(np.isnan(r[~active])) and np.all(~np.isnan(r[active]))
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    assert np.array_equal(iq.iqsim(TI, (10, 10, 10), TI.shape, ctx=ctx)[0], np.ones((20, 20, 20)))
    TI[0, 4, :] = 0
    assert np.array_equal(iq.iqsim(TI, (10, 10, 10), TI.shape, ctx=ctx)[0], np.ones((20, 20, 20)))
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    aux = np.full(TI.shape, 1.0)
    shape = {(i, 4, k): np.nan for i in range(20) for k in range(20)}
    for kw in ({}, {"soft": [(aux, aux)]}):
        r = iq.iqsim(TI, (10, 10, 10), TI.shape, hard=shape, ctx=ctx, **kw)[0]
        assert np.all(np.isnan(r[:, 4, :])) and np.all(r[:, :4, :] == 1) and np.all(r[:, 5:, :] == 1)


def test_runtests_cut_and_voxelreuse(iq, ctx):
    TI = np.ones((20, 20, 20))
    _, _, voxs = iq.iqsim(TI, (10, 10, 10), TI.shape, overlap=(1 / 3,) * 3, debug=True, ctx=ctx)
    assert 0 <= voxs[0] <= 1
    mu, _ = iq.voxelreuse(np.random.default_rng(3).random((20, 20, 20)), (10, 10, 10), nreal=1,
                          ctx=ctx)
    assert 0 <= mu <= 1


@pytest.mark.parametrize("shape,tile,overlap", [((30, 28, 14), (8, 8, 6), (0.25, 0.25, 0.34)),
                                                ((40, 36), (12, 10), None)])
def test_voxelreuse_vs_oracle(iq, ctx, shape, tile, overlap):
    """voxelreuse (src/voxelreuse.jl:18-41): a 2-tile grid per dimension, nreal debug runs,
    mean and standard deviation of the reuse. Integer data, so equal to the oracle's bits."""
    ti = np.random.default_rng(19).integers(0, 3, shape).astype(np.float32)
    kw = dict(nreal=5, rng=41) if overlap is None else dict(overlap=overlap, nreal=5, rng=41)
    mu, sd = iq.voxelreuse(ti, tile, ctx=ctx, **kw)
    kw_o = {k: v for k, v in kw.items() if k != "rng"}
    mu_o, sd_o = O.voxelreuse(ti, tile, seed=41, **kw_o)
    assert mu == mu_o and sd == sd_o
    assert 0 <= mu <= 1


def test_errors_are_reported(iq, ctx):
    TI = np.ones((20, 20))
    with pytest.raises(AssertionError, match="invalid tile size"):
        iq.iqsim(TI, (30, 10), ctx=ctx)
    with pytest.raises(AssertionError, match="tolerance"):
        iq.iqsim(TI, (10, 10), tol=0, ctx=ctx)
    with pytest.raises(iq.IQError):
        iq.graphcut(np.ones((4, 4)), np.ones((4, 4)), 5, ctx=ctx)


# ---- the committed golden fixtures (tests/golden/make_golden.py) ------------------------
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_golden_fixtures(iq, ctx):
    f = np.load(os.path.join(GOLDEN, "iqsim_int3d.npz"))
    hard = {tuple(int(v) for v in c): float(x) for c, x in zip(f["hard_coords"], f["hard_values"])}
    reals = iq.iqsim(f["ti"], tuple(int(t) for t in f["tilesize"]),
                     tuple(int(t) for t in f["simsize"]), overlap=tuple(float(o) for o in f["overlap"]),
                     path="raster", nreal=int(f["nreal"]), rng=int(f["seed"]), hard=hard,
                     soft=[(f["aux"], f["auxti"])], ctx=ctx)
    assert len(reals) == len(f["reals"])
    for x, y in zip(reals, f["reals"]):
        assert np.array_equal(np.asarray(x, np.float32), y)
    g = np.load(os.path.join(GOLDEN, "graphcut_cont3d.npz"))
    assert np.array_equal(iq.graphcut(g["A"], g["B"], int(g["dim"]), ctx=ctx), g["mask"])
    d = np.load(os.path.join(GOLDEN, "fastdistance_int3d.npz"))
    got = iq.fastdistance(d["ti"], d["tmpl"], d["weights"], ctx=ctx)
    assert np.array_equal(got, d["maps"])


# ---- the benchmark workload at full size: size-independent properties (tests/props.py) ---
def test_full_size_properties(iq, ctx):
    import bench
    from props import check_realizations
    W = bench.workload("cfg2")  # 16 realizations of 200x200x100, 500 hard data, 1 soft pair
    kw = dict(overlap=W["overlap"], soft=W["soft"], hard=W["hard"], tol=W["tol"],
              path=W["path"], nreal=W["nreal"], rng=7, ctx=ctx)
    a = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], **kw)
    assert len(a) == W["nreal"] and a[0].shape == W["simsize"]
    check_realizations(a, W["ti"], W["hard"])
    b = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], **kw)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


# ---- the cut cost clause on the GPU's masks (tests/cutcost.py) ----------------------------
@pytest.mark.parametrize("shape,dim,kind", [((6, 24, 12), 0, "cont"), ((24, 24, 3), 2, "cont"),
                                            ((6, 12, 5), 0, "cat")])
def test_gpu_cut_is_a_minimum_cut_of_the_unquantized_graph(iq, ctx, shape, dim, kind):
    import cutcost
    rng = np.random.default_rng(18)
    for trial in range(2):
        if kind == "cont":
            A = np.exp(rng.normal(size=shape)).astype(np.float32)
            B = np.exp(rng.normal(size=shape)).astype(np.float32)
        else:
            A = rng.integers(0, 4, shape).astype(np.float32)
            B = rng.integers(0, 4, shape).astype(np.float32)
        M = iq.graphcut(A, B, dim, ctx=ctx)
        cost = cutcost.cut_cost(A, B, M)
        flow = cutcost.maxflow_value(A, B, dim)
        big = max(c for _, _, c in cutcost.edges(A, B))
        assert abs(cost - flow) <= max(1e-9 * flow, 1e-12 * big), (trial, cost, flow)


# ---- the benchmark's configurations (bench.workload) ----------------------------------------
def test_cfg1_full_size_bit_exact(iq, ctx):
    """Config 1 in full (128x128 binary TI, 256x256 output, 100 tiles): realizations, boundary
    cuts and voxel reuse equal to the oracle's."""
    import bench
    W = bench.workload("cfg1")
    kw = dict(overlap=W["overlap"], tol=W["tol"], path=W["path"], nreal=2, debug=True)
    g = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], rng=3, ctx=ctx, **kw)
    r = O.iqsim(W["ti"], W["tilesize"], W["simsize"], seed=3, **kw)
    _same_reals(g[0], r[0])
    _same_reals(g[1], r[1])
    assert g[2] == r[2]


def test_cfg3_sample_bit_exact(iq, ctx):
    """Config 3's categorical workload (256x256x128 TI, 32x32x16 tiles, 5.7 M positions): the
    first 10 tiles of the path for one realization equal the oracle's."""
    import bench
    W = bench.workload("cfg3")
    steps = 10
    ctx.set_option("sim.max_steps", steps)
    try:
        g = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], tol=W["tol"],
                     path=W["path"], nreal=1, rng=8, ctx=ctx)
    finally:
        ctx.set_option("sim.max_steps", -1)
    r = O.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], tol=W["tol"],
                path=W["path"], nreal=1, seed=8, max_steps=steps)
    _same_reals(g, r)
    assert np.count_nonzero(np.asarray(g[0])) > 0


def test_cfg3_full_size_properties(iq, ctx):
    """Config 3 at full size for two realizations: every voxel a TI value, identical calls
    identical, realizations distinct (tests/props.py)."""
    import bench
    from props import check_realizations
    W = bench.workload("cfg3")
    kw = dict(overlap=W["overlap"], tol=W["tol"], path=W["path"], nreal=2, rng=4, ctx=ctx)
    a = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], **kw)
    assert len(a) == 2 and a[0].shape == W["simsize"]
    check_realizations(a, W["ti"], {})
    b = iq.iqsim(W["ti"], W["tilesize"], W["simsize"], **kw)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
