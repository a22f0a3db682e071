"""Host-side mirror of ImageQuilting.jl's public interface over libiqgpu.so.

`iqsim` keeps the reference's signature, defaults, assertion messages and return types
(src/iqsim.jl:50-63,145,314); every simulation step runs in the CUDA library. Arrays use the
Julia shape (axis 0 = Julia dim 1) and coordinates are 0-based. `rng` is a 64-bit seed (or a
numpy Generator a seed is drawn from): it keys the Philox4x32-10 streams of the library,
which replace Julia's Xoshiro stream.
"""
import ctypes
import math
import threading

import numpy as np

from . import _lib
from ._lib import IQError, check, i64arr, load

_local = threading.local()


def _float_type(dtype):
    dtype = np.dtype(dtype)
    return dtype if np.issubdtype(dtype, np.floating) else np.dtype(np.float64)


def _as_float_fortran(a, dtype=None):
    """Array with NaN for missing (masked) entries, column-major, float32/float64."""
    data = np.ma.getdata(a)
    F = _float_type(data.dtype) if dtype is None else np.dtype(dtype)
    out = np.array(data, dtype=F, order="F", copy=True)
    if np.ma.isMaskedArray(a):
        out[np.ma.getmaskarray(a)] = np.nan
    return out


def _seed(rng):
    if rng is None:
        return int.from_bytes(np.random.default_rng().bytes(8), "little")
    if isinstance(rng, (int, np.integer)):
        return int(rng) & ((1 << 64) - 1)
    if isinstance(rng, np.random.Generator):
        return int(rng.integers(0, 2 ** 63))
    raise TypeError("rng must be an integer seed or a numpy Generator")


class Context:
    """A library context on one device: a stream, the resident TI and reusable buffers."""

    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.iq_ctx_create(int(device), ctypes.byref(h)))
        self.h = h
        self._ti_key = None
        self.ndim = None
        self.tisize = None

    def close(self):
        if self.h:
            load().iq_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return load().iq_ctx_stream(self.h)

    def set_ti(self, ti, key=None):
        """Upload the training image (NaN or masked = inactive) unless `key` matches."""
        if key is not None and key == self._ti_key:
            return
        arr = ti if isinstance(ti, np.ndarray) and not np.ma.isMaskedArray(ti) else ti
        data = _as_float_fortran(arr)
        dt = _lib.IQ_F32 if data.dtype == np.float32 else _lib.IQ_F64
        if data.dtype not in (np.float32, np.float64):
            data = data.astype(np.float64, order="F")
            dt = _lib.IQ_F64
        check(load().iq_set_ti(self.h, data.ctypes.data, dt, data.ndim, i64arr(data.shape)))
        self._ti_key = key
        self.ndim = data.ndim
        self.tisize = data.shape

    def profile(self, enable=True):
        check(load().iq_profile(self.h, 1 if enable else 0))

    def profile_get(self, kernel):
        """(milliseconds, launches, algorithmic work) of a kernel since profile(True)."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        w = ctypes.c_double()
        check(load().iq_profile_get(self.h, kernel.encode(), ctypes.byref(ms), ctypes.byref(n),
                                    ctypes.byref(w)))
        return ms.value, n.value, w.value

    @property
    def ties(self):
        """Near-ties (|D - t| <= 1e-6 t at a decision value t) of the last iqsim or pick."""
        v = ctypes.c_int64()
        check(load().iq_ties(self.h, ctypes.byref(v)))
        return int(v.value)

    # ---- learned proposal (no counterpart in the reference) ------------------------------
    def lp_init(self, tilesize, seed=0):
        """Fresh encoder parameters for tiles of this shape."""
        check(load().iq_lp_init(self.h, len(tilesize), i64arr(tilesize), int(seed)))
        self._lp_tile = tuple(int(t) for t in tilesize)

    def lp_params(self):
        """The encoder's FP32 parameters (flat, the layout of oracle/proposal_oracle.py)."""
        n = ctypes.c_int64()
        check(load().iq_lp_params(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float32)
        check(load().iq_lp_params(self.h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def lp_set_params(self, tilesize, params):
        p = np.ascontiguousarray(params, np.float32)
        check(load().iq_lp_set_params(self.h, len(tilesize), i64arr(tilesize), p.ctypes.data,
                                      p.size))
        self._lp_tile = tuple(int(t) for t in tilesize)

    def lp_embed(self, positions, box):
        """Window embeddings (n x 64) of the resident TI at linear distance-map positions under
        the mask "tile minus box" (box = (lo0, lo1, lo2, hi0, hi1, hi2))."""
        pos = np.ascontiguousarray(positions, np.int64)
        b = np.ascontiguousarray(box, np.int32)
        out = np.empty((pos.size, 64), np.float32)
        check(load().iq_lp_embed(self.h, pos.size, pos.ctypes.data_as(_lib.c_i64p), b.ctypes.data,
                                 out.ctypes.data))
        return out

    def lp_loss_grad(self, anchor_feats, pos_positions, neg_positions, box, temp):
        a = np.ascontiguousarray(anchor_feats, np.float32)
        pp = np.ascontiguousarray(pos_positions, np.int64)
        nn = np.ascontiguousarray(neg_positions, np.int64)
        b = np.ascontiguousarray(box, np.int32)
        nA = pp.size
        nneg = nn.size // max(nA, 1)
        loss = ctypes.c_double()
        grad = np.empty(self.lp_params().size, np.float32)
        check(load().iq_lp_loss_grad(self.h, nA, nneg, a.ctypes.data, pp.ctypes.data_as(_lib.c_i64p),
                                     nn.ctypes.data_as(_lib.c_i64p), b.ctypes.data, float(temp),
                                     ctypes.byref(loss), grad.ctypes.data))
        return loss.value, grad

    def lp_train(self, steps, batch=128, nneg=16, lr=1e-3, temp=8.0, seed=0):
        """Adam steps on the captured pairs; returns (first batch loss, last batch loss)."""
        l0, l1 = ctypes.c_double(), ctypes.c_double()
        check(load().iq_lp_train(self.h, int(steps), int(batch), int(nneg), float(lr), float(temp),
                                 int(seed), ctypes.byref(l0), ctypes.byref(l1)))
        return l0.value, l1.value

    def lp_stats(self):
        """Statistics of the last iqsim call (see include/iqgpu.h, iq_lp_stats)."""
        out = np.zeros(12)
        check(load().iq_lp_stats(self.h, out.ctypes.data, 12))
        keys = ("cols_shortlist", "cols_full", "monitored", "true_candidates", "shortlisted",
                "recall", "fell_back", "mean_shortlist", "captured", "k_final",
                "recall_final", "sampled_final")
        return dict(zip(keys, out.tolist()))

    @property
    def launches(self):
        return int(load().iq_ctx_launches(self.h))

    def set_option(self, name, value):
        """Set a knob of this context (include/iqgpu.h lists them). Launch shapes, chunk sizes,
        stream groups and `corr.engine` (tensor cores vs SIMT) change how the distances are
        summed: continuous distances move within the stated tolerance, integer-data results not
        at all."""
        check(load().iq_set_option(self.h, name.encode(), int(value)))


def default_context():
    ctx = getattr(_local, "ctx", None)
    if ctx is None:
        ctx = Context(0)
        _local.ctx = ctx
    return ctx


def iqsim(trainimg, tilesize, simsize=None, *, overlap=None, soft=(), hard=None, tol=0.1,
          path="raster", nreal=1, debug=False, showprogress=False, rng=None, ctx=None,
          real0=0):
    """Image quilting simulation (src/iqsim.jl:5-49 documents the arguments).

    `real0` (not in the reference) is the global index of the first realization: calls with
    the same `rng` seed and disjoint ranges [real0, real0 + nreal) are shards of one call, on
    one device or several, and their realizations equal those of the whole call.

    Returns a list of `nreal` arrays of shape `simsize` ("reals"), or (reals, cuts, voxs)
    with debug=True. Float training images give arrays of their float type; other types give
    masked arrays of that type where NaN becomes masked (the reference's `missing`).
    """
    ti_dtype = np.ma.getdata(trainimg).dtype
    tisize = tuple(np.shape(trainimg))
    N = len(tisize)
    tilesize = tuple(int(t) for t in tilesize)
    simsize = tisize if simsize is None else tuple(int(s) for s in simsize)
    overlap = tuple([1 / 6] * N) if overlap is None else tuple(float(o) for o in overlap)
    hard = {} if hard is None else hard
    soft = list(soft)

    # sanity checks (src/iqsim.jl:68-89)
    assert len(tilesize) == N and len(simsize) == N and len(overlap) == N, "dimension mismatch"
    assert all(0 < t <= T for t, T in zip(tilesize, tisize)), "invalid tile size"
    assert all(s >= t for s, t in zip(simsize, tilesize)), "invalid grid size"
    assert all(0 < o < 1 for o in overlap), "overlaps must be in range (0,1)"
    assert 0 < tol <= 1, "tolerance must be in range (0,1]"
    assert path in _lib.PATHS, "invalid simulation path"
    assert nreal > 0, "invalid number of realizations"
    for aux, auxTI in soft:
        assert all(a >= s for a, s in zip(np.shape(aux), simsize)), "soft data size < grid size"
        assert tuple(np.shape(auxTI)) == tisize, "auxiliary TI must have the same size as TI"
    if hard:
        coords = np.array([tuple(k) for k in hard.keys()], dtype=np.int64).reshape(len(hard), N)
        assert np.all(coords.max(axis=0) < np.array(simsize)), "hard data coordinates outside of grid"
        assert np.all(coords.min(axis=0) >= 0), "hard data coordinates must be positive indices"
        values = np.array([np.nan if v is None else float(v) for v in hard.values()], np.float64)
    else:
        coords = np.zeros((0, N), np.int64)
        values = np.zeros(0, np.float64)

    ctx = ctx or default_context()
    ctx.set_ti(trainimg)
    lib = load()
    p = _lib.SimParams()
    p.ndim = N
    for d in range(N):
        p.tilesize[d] = tilesize[d]
        p.simsize[d] = simsize[d]
        p.overlap[d] = overlap[d]
    p.tol = float(tol)
    p.path = _lib.PATHS[path]
    p.nreal = int(nreal)
    p.debug = 1 if debug else 0
    p.seed = _seed(rng)
    p.real0 = int(real0)
    coords = np.ascontiguousarray(coords)
    hd = _lib.HardData(len(values), coords.ctypes.data if len(values) else None,
                       values.ctypes.data if len(values) else None)
    keep = []
    sd = (_lib.SoftData * max(len(soft), 1))()
    for i, (aux, auxTI) in enumerate(soft):
        a = _as_float_fortran(aux, np.float32)
        b = _as_float_fortran(auxTI, np.float32)
        keep += [a, b]
        sd[i].aux = a.ctypes.data
        sd[i].auxti = b.ctypes.data
        for d in range(3):
            sd[i].auxsize[d] = a.shape[d] if d < N else 1
    simvol = int(np.prod(simsize))
    out = np.empty(simvol * nreal, np.float32)
    cuts = np.empty(simvol * nreal, np.float32) if debug else None
    voxs = np.zeros(nreal, np.float64) if debug else None
    check(lib.iq_simulate(ctx.h, ctypes.byref(p), ctypes.byref(hd), len(soft),
                          sd if soft else None, out.ctypes.data,
                          cuts.ctypes.data if debug else None,
                          voxs.ctypes.data if debug else None))
    F = _float_type(ti_dtype)
    reals = []
    for r in range(nreal):
        g = out[r * simvol:(r + 1) * simvol].reshape(simsize, order="F")
        if np.issubdtype(ti_dtype, np.floating):
            reals.append(np.array(g, dtype=F))
        else:
            m = np.isnan(g)
            reals.append(np.ma.masked_array(np.where(m, 0, g).astype(ti_dtype), mask=m))
    if not debug:
        return reals
    cutl = [np.array(cuts[r * simvol:(r + 1) * simvol].reshape(simsize, order="F"),
                     dtype=np.float64) for r in range(nreal)]
    return reals, cutl, [float(v) for v in voxs]


def voxelreuse(trainimg, tilesize, *, overlap=None, nreal=10, **kwargs):
    """Mean and standard deviation of the voxel reuse (src/voxelreuse.jl:18-41)."""
    N = np.ndim(trainimg)
    overlap = tuple([1 / 6] * N) if overlap is None else tuple(overlap)
    ovlsize = [math.ceil(o * t) for o, t in zip(overlap, tilesize)]
    ntiles = [2 if o > 1 else 1 for o in ovlsize]
    simsize = tuple(n * (t - o) + o for n, t, o in zip(ntiles, tilesize, ovlsize))
    _, _, voxs = iqsim(trainimg, tilesize, simsize, overlap=overlap, nreal=nreal, debug=True,
                       **kwargs)
    mu = float(np.mean(voxs))
    sd = float(np.std(voxs, ddof=1)) if len(voxs) > 1 else float("nan")
    return mu, sd


# ---- per-operation entry points (parity surface of the hot path) ----------------------
def fastdistance(ti, tmpl, weights=None, ctx=None):
    """fastdistance(TI, kern; weights) (src/utils.jl:5-13) for one or more templates.

    tmpl: array of the tile shape, or a stack (ntmpl, *tileshape). Returns float32 maps of
    shape TIsize - tilesize + 1 (stacked when several templates are given)."""
    ctx = ctx or default_context()
    ctx.set_ti(ti)
    t = np.asarray(tmpl, np.float32)
    stacked = t.ndim == np.ndim(ti) + 1
    if not stacked:
        t = t[None]
    tshape = t.shape[1:]
    nt = t.shape[0]
    buf = np.empty(int(np.prod(tshape)) * nt, np.float32)
    for i in range(nt):
        buf[i * int(np.prod(tshape)):(i + 1) * int(np.prod(tshape))] = t[i].ravel(order="F")
    w = None
    if weights is not None:
        w = np.asarray(weights, np.uint8).ravel(order="F").copy()
    dshape = tuple(T - k + 1 for T, k in zip(np.shape(ti), tshape))
    P = int(np.prod(dshape))
    out = np.empty(P * nt, np.float32)
    check(load().iq_fastdistance(ctx.h, i64arr(tshape), nt, buf.ctypes.data,
                                 w.ctypes.data if w is not None else None, out.ctypes.data))
    maps = [out[i * P:(i + 1) * P].reshape(dshape, order="F") for i in range(nt)]
    return np.stack(maps) if stacked else maps[0]


def pick(D, Ds=(), tol=0.1, seed=0, tile=0, real=0, ctx=None):
    """Candidate pick, tau-model weights and draw of one tile (src/iqsim.jl:236-246).

    Returns (drawn linear index, candidate indices, weights); indices are column-major."""
    ctx = ctx or default_context()
    d = np.asarray(D, np.float32).ravel(order="F").copy()
    aux = [np.asarray(x, np.float32).ravel(order="F").copy() for x in Ds]
    P = d.size
    arr = (ctypes.c_void_p * max(len(aux), 1))(*[a.ctypes.data for a in aux])
    idx = ctypes.c_int64()
    nc = ctypes.c_int64()
    cands = np.empty(P, np.int64)
    w = np.empty(P, np.float64)
    check(load().iq_pick(ctx.h, d.ctypes.data, P, len(aux), arr if aux else None, float(tol),
                         int(seed) & ((1 << 64) - 1), int(tile), int(real), ctypes.byref(idx),
                         ctypes.byref(nc), cands.ctypes.data_as(_lib.c_i64p),
                         w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), P))
    n = nc.value
    return idx.value, cands[:n].copy(), w[:n].copy()


def graphcut(A, B, dim, ctx=None):
    """Boundary cut mask along `dim` (0-based), True = keep A (src/graphcut.jl:5-84)."""
    ctx = ctx or default_context()
    A = np.asarray(A)
    B = np.asarray(B)
    assert A.shape == B.shape, "arrays must have the same size for cut"
    a = np.asfortranarray(A, np.float32)
    b = np.asfortranarray(B, np.float32)
    m = np.zeros(A.shape, np.uint8, order="F")
    check(load().iq_graphcut(ctx.h, a.ctypes.data, b.ctypes.data, A.ndim, i64arr(A.shape),
                             int(dim), m.ctypes.data))
    return m.astype(bool)


def finddisabled(ti, tilesize, ctx=None):
    """Windows of the TI covering an inactive voxel (src/utils.jl:115-129)."""
    ctx = ctx or default_context()
    ctx.set_ti(ti)
    dshape = tuple(T - k + 1 for T, k in zip(np.shape(ti), tilesize))
    out = np.zeros(int(np.prod(dshape)), np.uint8)
    check(load().iq_finddisabled(ctx.h, i64arr(tilesize), out.ctypes.data))
    return out.reshape(dshape, order="F").astype(bool)


def genpath(seed, extent, kind, datainds=()):
    """Tile visiting order (src/utils.jl:158-204); runs on the host side of the library."""
    n = int(np.prod(extent))
    out = (ctypes.c_int64 * n)()
    di = i64arr(datainds) if len(datainds) else None
    k = _lib.PATHS.get(kind, 0)
    check(load().iq_genpath(int(seed) & ((1 << 64) - 1), len(extent), i64arr(extent), k,
                            len(datainds), di, out))
    return list(out)
