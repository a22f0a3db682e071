"""The CPU oracle against the reference's own tests (test/runtests.jl) and published vectors.

These run without a GPU. They pin the oracle before it is trusted as the checker of the CUDA
path: every invariant and known answer of test/runtests.jl:9-162 is restated here.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import iqsim_oracle as O
from oracle import philox


# ---- Philox4x32-10 published known-answer vectors ---------------------------------------
@pytest.mark.parametrize("ctr,key,expect", [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
])
def test_philox_kat(ctr, key, expect):
    assert philox.philox4x32_10(ctr, key) == expect


# ---- geometry (src/iqsim.jl:91-115) at the benchmark configurations ----------------------
def test_geometry_configs():
    g = O.geometry((128, 128), (32, 32), (256, 256), (1 / 6, 1 / 6))
    assert g.ovlsize == (6, 6) and g.spacing == (26, 26) and g.ntiles == (10, 10)
    assert g.padsize == (266, 266) and g.distsize == (97, 97)
    g = O.geometry((100, 100, 50), (24, 24, 12), (200, 200, 100), (0.25,) * 3)
    assert g.ovlsize == (6, 6, 3) and g.spacing == (18, 18, 9) and g.ntiles == (12, 12, 12)
    assert g.padsize == (222, 222, 111) and g.distsize == (77, 77, 39)
    g = O.geometry((256, 256, 128), (32, 32, 16), (512, 512, 128), (0.25,) * 3)
    assert g.ntiles == (22, 22, 11) and g.distsize == (225, 225, 113)


# ---- "Basic checks" test/runtests.jl:9-27 ----------------------------------------------
def test_basic_homogeneous():
    TI = np.ones((20, 20, 20))
    reals = O.iqsim(TI, (10, 10, 10), TI.shape)
    assert reals[0].dtype == np.float64
    assert np.array_equal(reals[0], TI)


def test_basic_float32_preserved():
    TI = np.random.default_rng(1).random((20, 20, 20)).astype(np.float32)
    reals = O.iqsim(TI, (10, 10, 10), TI.shape)
    assert reals[0].dtype == np.float32


def test_basic_categorical():
    TI = np.random.default_rng(2).integers(1, 4, (20, 20, 20))
    reals = O.iqsim(TI, (10, 10, 10), TI.shape)
    assert np.ma.isMaskedArray(reals[0]) and reals[0].dtype == TI.dtype
    assert set(np.unique(reals[0].compressed())) <= set(np.unique(TI))


# ---- "Soft data" test/runtests.jl:29-48 ------------------------------------------------
def test_soft_trend():
    TI = np.concatenate([np.zeros((10, 20, 1)), np.ones((10, 20, 1))], axis=0)
    trend = np.concatenate([np.zeros((20, 10, 1)), np.ones((20, 10, 1))], axis=1)
    reals = O.iqsim(TI, (10, 10, 1), TI.shape, soft=[(trend, TI)], tol=1)
    assert reals[0][:, :10, :].mean() <= reals[0][:, 10:, :].mean()


def test_soft_no_side_effects():
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    aux = np.full(TI.shape, 1.0)
    O.iqsim(TI, (10, 10, 10), TI.shape, soft=[(aux, aux)])
    assert np.array_equal(aux, np.full(TI.shape, 1.0))
    TI = np.ones((20, 20, 20))
    aux = np.fromfunction(lambda i, j, k: i + 1, (20, 20, 20), dtype=int)
    ref = aux.copy()
    O.iqsim(TI, (10, 10, 10), TI.shape, soft=[(aux, aux)])
    assert np.array_equal(aux, ref)


# ---- "Hard data" test/runtests.jl:50-65 ------------------------------------------------
def test_hard_honoured_everywhere():
    TI = np.ones((20, 20, 20))
    obs = np.zeros(TI.shape)
    data = {c: obs[c] for c in np.ndindex(*TI.shape)}
    reals = O.iqsim(TI, (10, 10, 10), TI.shape, hard=data)
    assert np.array_equal(reals[0], obs)


def test_hard_multiple_realizations():
    TI = np.ones((20, 20, 20))
    reals = O.iqsim(TI, (10, 10, 10), TI.shape, hard={(19, 19, 19): 10}, nreal=3)
    assert len(reals) == 3
    for r in reals:
        assert r[19, 19, 19] == 10


# ---- "Masked grids" test/runtests.jl:67-104 --------------------------------------------
def test_masked_domain():
    TI = np.ones((20, 20, 20))
    shape, active = {}, np.ones(TI.shape, bool)
    for i, j, k in np.ndindex(20, 20, 20):
        if (i - 9) ** 2 + (j - 9) ** 2 + (k - 9) ** 2 < 25:
            shape[(i, j, k)] = np.nan
            active[i, j, k] = False
    reals = O.iqsim(TI, (10, 10, 10), TI.shape, hard=shape)
    assert np.all(np.isnan(reals[0][~active]))
    assert np.all(~np.isnan(reals[0][active]))


def test_masked_training_image():
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    reals = O.iqsim(TI, (10, 10, 10), TI.shape)
    assert np.array_equal(reals[0], np.full(TI.shape, 1.0))
    TI[0, 4, :] = 0
    reals = O.iqsim(TI, (10, 10, 10), TI.shape)
    assert np.array_equal(reals[0], np.full(TI.shape, 1.0))


def test_masked_domain_and_training_image():
    TI = np.ones((20, 20, 20))
    TI[:, 4, :] = np.nan
    aux = np.full(TI.shape, 1.0)
    shape = {(i, 4, k): np.nan for i in range(20) for k in range(20)}
    for kw in ({}, {"soft": [(aux, aux)]}):
        reals = O.iqsim(TI, (10, 10, 10), TI.shape, hard=shape, **kw)
        assert np.all(np.isnan(reals[0][:, 4, :]))
        assert np.all(reals[0][:, :4, :] == 1)
        assert np.all(reals[0][:, 5:, :] == 1)


# ---- "Minimum error cut" test/runtests.jl:106-120 (known answer) -------------------------
def test_cut_known_answer():
    TI = np.ones((20, 20, 20))
    _, _, voxs = O.iqsim(TI, (10, 10, 10), TI.shape, overlap=(1 / 3,) * 3, debug=True)
    assert 0 <= voxs[0] <= 1
    A, B = np.ones((20, 20)), np.ones((20, 20))
    C = O.graphcut(A, B, 0)
    assert np.all(C[:-1, :]) and not np.any(C[-1, :])
    C = O.graphcut(A, B, 1)
    assert np.all(C[:, :-1]) and not np.any(C[:, -1])


# ---- "Simulation paths" test/runtests.jl:122-134 ---------------------------------------
@pytest.mark.parametrize("kind", ["raster", "dilation", "random"])
def test_paths_length(kind):
    p = O.genpath(123, (10, 10, 10), kind, [])
    assert len(p) == 1000 and sorted(p) == list(range(1000))


def test_path_data_first():
    p = O.genpath(123, (10, 10, 10), "data", [0, 999])
    assert p[:2] in ([0, 999], [999, 0])
    assert sorted(p) == list(range(1000))


# ---- "Voxel reuse" test/runtests.jl:136-141 --------------------------------------------
def test_voxel_reuse_range():
    TI = np.random.default_rng(3).random((20, 20, 20))
    mu, _ = O.voxelreuse(TI, (10, 10, 10), nreal=1)
    assert 0 <= mu <= 1


# ---- "CPU vs GPU" imfilter test/runtests.jl:143-162: FFT form vs direct sum -------------
def test_imfilter_fft_vs_direct_2d():
    rng = np.random.default_rng(4)
    img, krn = rng.random((200, 100)), rng.random((30, 10))
    a = O.imfilter_valid(img, krn)
    b = O.imfilter_valid_direct(img, krn)
    assert a.shape == b.shape == (171, 91)
    assert np.max(np.abs(a - b)) < 1e-2


def test_imfilter_fft_vs_direct_3d():
    rng = np.random.default_rng(5)
    img, krn = rng.random((30, 40, 50)), rng.random((6, 8, 10))
    a = O.imfilter_valid(img, krn)
    b = O.imfilter_valid_direct(img, krn)
    assert a.shape == b.shape
    assert np.max(np.abs(a - b)) < 1e-2


def test_fastdistance_forms_agree():
    rng = np.random.default_rng(6)
    img = rng.random((30, 25, 12))
    kern = rng.random((8, 7, 5))
    w = rng.random(kern.shape) < 0.5
    a = O.fastdistance(img, kern, w, "fft")
    b = O.fastdistance(img, kern, w, "direct")
    scale = O.imfilter_valid(img ** 2, w.astype(float)) + np.sum(w * kern ** 2)
    assert np.max(np.abs(a - b) / scale) < 1e-10


# ---- pick, relaxation, taumodel, draw -------------------------------------------------
def test_threshold_pick_zero_min_quirk():
    D = np.array([[0.0, 1e-9], [0.0, 2.0]])
    # (1 + tol) * 0 = 0: only exact zeros are candidates (src/iqsim.jl:237)
    assert list(O.threshold_pick(D, 0.5)) == [0, 1]  # column-major: D[1,0] is index 1


def test_taumodel_single_source():
    w = O.taumodel(np.arange(4), np.array([3.0, 1.0, 1.0, 2.0]), [])
    # dense ranks 3,1,1,2 -> P = (n - r + 1)/sum = (2,4,4,3)/13
    assert np.allclose(w, np.array([2, 4, 4, 3]) / 13, rtol=1e-14)
    assert list(O.taumodel(np.array([7]), np.zeros(10), [])) == [1.0]


def test_relaxation_intersection_grows():
    rng = np.random.default_rng(7)
    D = rng.random(1000)
    S = rng.random(1000)
    cands = O.relaxation(D, [S], 0.1)
    assert len(cands) > 0 and np.all(np.diff(cands) > 0)
    top = set(np.argsort(D, kind="stable")[:100])
    assert set(cands) <= top
    # brute force of the relaxation rule: smallest softdbsize in the sequence with a hit
    rankS = np.empty(1000, int)
    rankS[np.argsort(S, kind="stable")] = np.arange(1, 1001)
    for s in O.relaxation_frac_sequence(1000, 100):
        hit = sorted(p for p in top if rankS[p] <= s)
        if hit:
            assert list(cands) == hit
            break


def test_sample_index_matches_sequential_walk():
    rng = np.random.default_rng(8)
    for n in (1, 2, 5, 255, 256, 257, 1000, 5000):
        w = rng.random(n)
        for u in (0.0, 0.3, 0.999999):
            i = O.sample_index(u, w)
            cs = np.cumsum(w)
            t = u * cs[-1]
            j = int(np.argmax(cs >= t))
            assert abs(i - j) <= 1  # sums are ordered differently; they differ only at ties


# ---- graph cut: BK vs an independent max-flow (networkx) --------------------------------
def _reach_t_mask(A, B, dim):
    nx = pytest.importorskip("networkx")
    A = np.asarray(A)
    caps = O.capacities(A, B)
    shape = A.shape
    G = nx.DiGraph()
    idx = np.arange(A.size).reshape(shape, order="F")
    i = 0
    for d in range(A.ndim):
        if shape[d] < 2:
            continue
        lo = [slice(None)] * A.ndim
        hi = [slice(None)] * A.ndim
        lo[d] = slice(0, shape[d] - 1)
        hi[d] = slice(1, shape[d])
        us = idx[tuple(lo)].ravel(order="F")
        vs = idx[tuple(hi)].ravel(order="F")
        for u, v in zip(us, vs):
            c = float(caps[i])
            i += 1
            G.add_edge(int(u), int(v), capacity=c)
            G.add_edge(int(v), int(u), capacity=c)
    first = np.take(idx, 0, axis=dim).ravel()
    last = np.take(idx, shape[dim] - 1, axis=dim).ravel()
    for u in first:
        G.add_edge("s", int(u))  # no capacity attribute = infinite
    for v in last:
        G.add_edge(int(v), "t")
    R = nx.algorithms.flow.edmonds_karp(G, "s", "t")
    val = R.graph["flow_value"]
    # nodes that can reach t with residual > 0: the capacities are multiples of one power of
    # two far below 2^53 of it, so networkx's float arithmetic is exact too
    reach = {"t"}
    stack = ["t"]
    while stack:
        v = stack.pop()
        for u in R.predecessors(v):
            e = R[u][v]
            res = e["capacity"] - e["flow"]
            if u not in reach and res > 0:
                reach.add(u)
                stack.append(u)
    M = np.ones(A.size, bool)
    for v in reach:
        if v not in ("s", "t"):
            M[v] = False
    return M.reshape(shape, order="F"), val


@pytest.mark.parametrize("seed,shape,dim", [(0, (6, 24), 0), (1, (24, 6), 1), (2, (6, 10, 8), 0),
                                            (3, (10, 6, 8), 1), (4, (10, 8, 3), 2)])
def test_bk_matches_independent_maxflow(seed, shape, dim):
    rng = np.random.default_rng(seed)
    A = rng.random(shape).astype(np.float32)
    B = rng.random(shape).astype(np.float32)
    M, cost = O.graphcut(A, B, dim, return_cost=True)
    Mnx, val = _reach_t_mask(A, B, dim)
    assert np.array_equal(M, Mnx)
    assert math.isclose(cost, val, rel_tol=1e-9)
    assert math.isclose(O.cut_cost(A, B, M), val, rel_tol=1e-9)


@pytest.mark.parametrize("shape", [(6, 12, 5), (3, 8, 6), (4, 7, 5)])
def test_bk_categorical_ties(shape):
    # integer data: zero gradient sums give eps-denominator capacities ~2^52 times the others,
    # the case where unquantized Float64 flows stop at different minimum cuts
    rng = np.random.default_rng(9)
    for trial in range(10):
        A = rng.integers(0, 4, shape).astype(np.float32)
        B = rng.integers(0, 4, shape).astype(np.float32)
        M, cost = O.graphcut(A, B, 0, return_cost=True)
        Mnx, val = _reach_t_mask(A, B, 0)
        assert math.isclose(cost, val, rel_tol=1e-12)
        assert np.array_equal(M, Mnx)


def test_capacities_are_quantized():
    rng = np.random.default_rng(10)
    A = rng.integers(0, 3, (3, 6, 4)).astype(np.float32)
    B = rng.integers(0, 3, (3, 6, 4)).astype(np.float32)
    c = O.capacities(A, B)
    q = 2.0 ** (math.frexp(c.max())[1] - 1 - 47)
    assert c.max() > 2.0 ** 50  # some eps-denominator edges
    assert np.all(np.mod(c, q) == 0)


# ---- golden fixtures (tests/golden/make_golden.py) -------------------------------------
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_golden_philox_vectors():
    for e in json.load(open(os.path.join(GOLDEN, "philox_kat.json"))):
        ctr = tuple(int(x, 16) for x in e["counter"])
        key = tuple(int(x, 16) for x in e["key"])
        assert philox.philox4x32_10(ctr, key) == tuple(int(x, 16) for x in e["output"])


def test_golden_oracle_reproduces_iqsim():
    f = np.load(os.path.join(GOLDEN, "iqsim_int3d.npz"))
    hard = {tuple(int(v) for v in c): float(x) for c, x in zip(f["hard_coords"], f["hard_values"])}
    reals = O.iqsim(f["ti"], tuple(int(t) for t in f["tilesize"]),
                    tuple(int(t) for t in f["simsize"]), overlap=tuple(f["overlap"]),
                    path="raster", nreal=int(f["nreal"]), seed=int(f["seed"]), hard=hard,
                    soft=[(f["aux"], f["auxti"])])
    for x, y in zip(reals, f["reals"]):
        assert np.array_equal(np.asarray(x, np.float32), y)


def test_golden_oracle_reproduces_cut_and_distances():
    g = np.load(os.path.join(GOLDEN, "graphcut_cont3d.npz"))
    assert np.array_equal(O.graphcut(g["A"], g["B"], int(g["dim"])), g["mask"])
    d = np.load(os.path.join(GOLDEN, "fastdistance_int3d.npz"))
    dis = O.finddisabled(d["ti"], d["tmpl"].shape[1:])
    for t, m in zip(d["tmpl"], d["maps"]):
        ref = O.fastdistance(np.nan_to_num(d["ti"]), t, d["weights"], "direct")
        ref[dis] = np.inf
        assert np.array_equal(ref.astype(np.float32), m)


# ---- the full-size property checks (tests/props.py) hold on the oracle's output ---------------
def test_properties_hold_on_oracle_output():
    from props import check_realizations
    rng = np.random.default_rng(60)
    ti = np.exp(rng.normal(size=(20, 18, 8))).astype(np.float32)
    hard = {(2, 3, 1): 0.5, (17, 20, 5): 7.25}
    reals = O.iqsim(ti, (8, 8, 4), (24, 26, 8), overlap=(0.25,) * 3, hard=hard, nreal=2, seed=5)
    check_realizations(reals, ti, hard)
    # a planted mistake is caught: a value that is neither a TI value nor a hard datum
    bad = [r.copy() for r in reals]
    bad[1][5, 5, 5] = -1.0
    with pytest.raises(AssertionError):
        check_realizations(bad, ti, hard)


# ---- the Float64 evaluation the exact re-rank reproduces (oracle/direct.c) ----------------
def test_direct_distance_is_the_sequential_column_major_sum():
    rng = np.random.default_rng(71)
    img = np.exp(rng.normal(size=(14, 12, 9))).astype(np.float32)
    k = np.exp(rng.normal(size=(5, 4, 3))).astype(np.float32)
    w = rng.random((5, 4, 3)) < 0.6
    got = O.fastdistance(img, k, w, "direct")
    out_shape = tuple(i - t + 1 for i, t in zip(img.shape, k.shape))
    ref = np.zeros(out_shape)
    I, K = img.astype(np.float64), k.astype(np.float64)
    for lin in np.flatnonzero(w.ravel(order="F")):
        kk = np.unravel_index(lin, w.shape, order="F")
        d = I[tuple(slice(o, o + s) for o, s in zip(kk, out_shape))] - K[kk]
        ref = ref + d * d
    assert np.array_equal(got, ref)
    # 1-D and 2-D go through the same 3-D routine
    a1 = rng.normal(size=40)
    assert np.allclose(O.fastdistance(a1, a1[:7], None, "direct"),
                       O.fastdistance(a1, a1[:7], None, "fft"), atol=1e-9)


def test_count_ties_rules():
    d = np.array([1.0, 2.0, 2.0 * (1 + 5e-7), 2.0 * (1 - 9e-7), 2.0 * (1 + 2e-6), np.inf])
    assert O.count_ties(d, 2.0, False) == 3
    assert O.count_ties(d, 2.0, True) == 2  # the boundary position itself is not counted
    assert O.count_ties(d, 0.0, False) == 0 and O.count_ties(d, np.inf, True) == 0
    ties = []
    O.threshold_pick(np.array([1.0, 1.1, 1.1 * (1 + 1e-7), 3.0]), 0.1, ties)
    assert ties == [2]


# ---- the cut cost clause: equal cost with unquantized capacities (tests/cutcost.py) --------
@pytest.mark.parametrize("shape,dim,kind", [((6, 20), 0, "cont"), ((6, 10, 8), 0, "cont"),
                                            ((10, 8, 3), 2, "cont"), ((4, 9, 6), 0, "cat")])
def test_quantized_cut_is_a_minimum_cut_of_the_unquantized_graph(shape, dim, kind):
    import cutcost
    rng = np.random.default_rng(17)
    for trial in range(3):
        if kind == "cont":
            A = np.exp(rng.normal(size=shape)).astype(np.float32)
            B = np.exp(rng.normal(size=shape)).astype(np.float32)
        else:
            A = rng.integers(0, 4, shape).astype(np.float32)
            B = rng.integers(0, 4, shape).astype(np.float32)
        M = O.graphcut(A, B, dim)
        cost = cutcost.cut_cost(A, B, M)
        flow = cutcost.maxflow_value(A, B, dim)
        # quantization keeps 47 bits relative to the largest capacity
        tol = 1e-9 if kind == "cont" else 1e-12 * max(c for _, _, c in cutcost.edges(A, B)) / max(flow, 1e-300)
        assert abs(cost - flow) <= max(tol, 1e-9) * max(flow, 1e-300), (trial, cost, flow)
