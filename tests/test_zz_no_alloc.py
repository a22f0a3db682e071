"""iq_pick_noalloc, the pick entry point that allocates no device memory.

It serves hosts that cannot call cudaMalloc from the code that drives the library -- a
framework whose device memory belongs to its own pool allocator, or a latency-bound loop that
cannot take the device-wide synchronization of an allocation. Its scratch is a fixed
__device__ array inside libiqgpu.so. This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, D, Ds, tol, seed, tile, real, stream=None):
    d = np.ascontiguousarray(D, np.float32)
    aux = [np.ascontiguousarray(x, np.float32) for x in Ds]
    P = d.size
    arr = (ctypes.c_void_p * max(len(aux), 1))(*[a.ctypes.data for a in aux])
    idx = ctypes.c_int64()
    nc = ctypes.c_int64()
    cands = np.empty(P, np.int64)
    w = np.empty(P, np.float64)
    rc = lib.iq_pick_noalloc(d.ctypes.data, P, len(aux), arr if aux else None, tol, seed, tile,
                             real, ctypes.byref(idx), ctypes.byref(nc),
                             cands.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), P, stream)
    return rc, idx.value, cands[:nc.value].copy(), w[:nc.value].copy()


def test_noalloc_pick_matches_iq_pick(iq):
    lib = iq.load()
    ctx = iq.Context(0)
    rng = np.random.default_rng(31)
    P = 231231
    D = (rng.random(P) * 40).astype(np.float32)
    D[rng.random(P) < 0.1] = np.inf
    S = (rng.random(P) * 9).astype(np.float32)
    S[np.isinf(D)] = np.inf
    cases = [([], 0.1, 3, 17, 2), ([S], 0.1, 5, 18, 0)]
    for Ds, tol, seed, tile, real in cases:
        ref = iq.pick(D, Ds, tol, seed, tile, real, ctx=ctx)
        for _ in range(2):  # two calls in a row share the scratch array
            rc, i, c, w = _noalloc(lib, D, Ds, tol, seed, tile, real)
            assert rc == 0, lib.iq_last_error()
            assert i == ref[0]
            assert np.array_equal(c, ref[1])
            assert np.array_equal(w, ref[2])  # bit-exact, like iq_pick against the oracle
    ctx.close()


def test_noalloc_pick_at_its_limits_on_a_caller_stream(iq):
    """P = 2^18 and three auxiliary maps fill every region of the scratch array; the calls run
    on the context's (non-default) stream."""
    lib = iq.load()
    ctx = iq.Context(0)
    rng = np.random.default_rng(47)
    P = 1 << 18
    D = (rng.random(P) * 25).astype(np.float32)
    D[rng.random(P) < 0.05] = np.inf
    Ds = []
    for scale in (7.0, 3.0, 11.0):
        S = np.floor(rng.random(P) * scale).astype(np.float32)  # ties inside every aux map
        S[np.isinf(D)] = np.inf
        Ds.append(S)
    ref = iq.pick(D, Ds, 0.1, 9, 40, 3, ctx=ctx)
    stream = ctx.stream
    for _ in range(2):
        rc, i, c, w = _noalloc(lib, D, Ds, 0.1, 9, 40, 3, stream=stream)
        assert rc == 0, lib.iq_last_error()
        assert i == ref[0]
        assert np.array_equal(c, ref[1])
        assert np.array_equal(w, ref[2])
    ctx.close()


def test_noalloc_pick_rejects_oversized_maps(iq):
    lib = iq.load()
    rc, *_ = _noalloc(lib, np.zeros((1 << 18) + 1, np.float32), [], 0.1, 0, 0, 0)
    assert rc == 7  # IQ_ERR_LIMIT
    assert b"at most" in lib.iq_last_error()
