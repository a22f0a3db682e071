"""CPU oracle of the image-quilting hot path.

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
import this module, and only as the checker or the timed CPU baseline; the product library
(imagequilting.jl_gb300) never imports, links or calls it.

It restates ImageQuilting.jl v1.3.1 in Float64 NumPy/SciPy (max-flow in C, oracle/bkcut.c):

  geometry ............ src/iqsim.jl:91-127
  prepare/unprepare ... src/utils.jl:96-113, padding src/utils.jl:69-92
  finddisabled ........ src/utils.jl:115-129
  indicator/event/activation on dense hard-data grids ... src/utils.jl:18-55
  findskipped ......... src/utils.jl:131-156
  genpath ............. src/utils.jl:158-204
  fastdistance ........ src/utils.jl:5-13 (direct masked SSD, or the FFT form of
                        src/imfilter.jl:5-7 / :9-26)
  relaxation .......... src/relaxation.jl:5-48
  taumodel ............ src/taumodel.jl:5-45
  weighted draw ....... src/iqsim.jl:243 (StatsBase.sample inverse-CDF walk)
  graphcut ............ src/graphcut.jl:5-84 (oracle/bkcut.c)
  iqsim loop .......... src/iqsim.jl:50-315

Third-party semantics restated from their published behaviour (not vendored in the reference):
  * ImageFiltering `padarray(..., Pad(:symmetric, ...))`: mirror with the edge sample repeated,
    period 2n (…c b a | a b c | c b a…).
  * ImageMorphology `dilate(grid)`: max filter over the 3^N box, outside = false.
  * StatsBase `sample(rng, a, weights(w))`: t = u * sum(w), first i with cumsum(w)[i] >= t.
    The sums run in a fixed order (chunks of 256 summed left to right, chunk totals summed left
    to right), which the GPU draw reproduces bit for bit.
  * Julia's Xoshiro stream is replaced by Philox4x32-10 (oracle/philox.py).

Conventions: arrays keep the Julia shapes (dim 0 = Julia dim 1) and every linear index is
column-major and 0-based (Julia index minus one). Hard data is a dict {coordinate tuple
(0-based): value}.

Parity pins (tests/test_oracle.py): the known-answer and invariant tests of
test/runtests.jl:9-141 and the imfilter check of test/runtests.jl:143-162 run against this
module; exact Julia-stream outputs are unpinned because no Julia toolchain exists here.
"""
import ctypes
import math
import os
import subprocess
from typing import NamedTuple

import numpy as np
import scipy.fft

from . import philox

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "liboracle.so")
_lib = None


def build_native(force=False):
    """Compile oracle/bkcut.c and oracle/direct.c into oracle/liboracle.so (gcc; plain C)."""
    srcs = [os.path.join(_HERE, f) for f in ("bkcut.c", "direct.c")]
    if (not force and os.path.exists(_LIBPATH)
            and all(os.path.getmtime(_LIBPATH) >= os.path.getmtime(s) for s in srcs)):
        return _LIBPATH
    tmp = _LIBPATH + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp]
                          + srcs + ["-lm", "-lpthread"])
    os.replace(tmp, _LIBPATH)
    return _LIBPATH


def _native():
    global _lib
    if _lib is None:
        build_native()
        lib = ctypes.CDLL(_LIBPATH)
        lib.oracle_graphcut.restype = ctypes.c_int
        lib.oracle_graphcut.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.c_int, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_double)]
        lib.oracle_direct_ssd.restype = ctypes.c_int
        lib.oracle_direct_ssd.argtypes = [ctypes.c_void_p] + [ctypes.c_longlong] * 3 + [
            ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_longlong] * 3 + [ctypes.c_void_p,
                                                                           ctypes.c_int]
        lib.oracle_capacities.restype = ctypes.c_longlong
        lib.oracle_capacities.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.c_void_p]
        _lib = lib
    return _lib


# --------------------------------------------------------------------------------------
# geometry (src/iqsim.jl:91-127) and argument checks (src/iqsim.jl:68-89)
# --------------------------------------------------------------------------------------
class Geometry(NamedTuple):
    ntiles: tuple
    tilesize: tuple
    ovlsize: tuple
    spacing: tuple
    TIsize: tuple
    simsize: tuple
    padsize: tuple
    distsize: tuple
    ovlvol: int


def geometry(tisize, tilesize, simsize, overlap):
    tilesize = tuple(int(t) for t in tilesize)
    simsize = tuple(int(s) for s in simsize)
    ovlsize = tuple(math.ceil(o * t) for o, t in zip(overlap, tilesize))
    spacing = tuple(t - o for t, o in zip(tilesize, ovlsize))
    ntiles = tuple(math.ceil(s / max(sp, 1)) for s, sp in zip(simsize, spacing))
    padsize = tuple(n * (t - o) + o for n, t, o in zip(ntiles, tilesize, ovlsize))
    distsize = tuple(T - t + 1 for T, t in zip(tisize, tilesize))
    ovlvol = int(np.prod(padsize)) - int(np.prod([p - (n - 1) * o
                                                   for p, n, o in zip(padsize, ntiles, ovlsize)]))
    return Geometry(ntiles, tilesize, ovlsize, spacing, tuple(tisize), simsize, padsize, distsize,
                    ovlvol)


def check_args(tisize, tilesize, simsize, overlap, tol, path, nreal, soft, hard):
    N = len(tisize)
    assert len(tilesize) == N and len(simsize) == N and len(overlap) == N, "dimension mismatch"
    assert all(0 < t <= T for t, T in zip(tilesize, tisize)), "invalid tile size"
    assert all(s >= t for s, t in zip(simsize, tilesize)), "invalid grid size"
    assert all(0 < o < 1 for o in overlap), "overlaps must be in range (0,1)"
    assert 0 < tol <= 1, "tolerance must be in range (0,1]"
    assert path in ("raster", "dilation", "random"), "invalid simulation path"
    assert nreal > 0, "invalid number of realizations"
    for aux, auxTI in soft:
        assert all(a >= s for a, s in zip(np.shape(aux), simsize)), "soft data size < grid size"
        assert tuple(np.shape(auxTI)) == tuple(tisize), \
            "auxiliary TI must have the same size as TI"
    if hard:
        coords = np.array(list(hard.keys()), dtype=np.int64).reshape(len(hard), N)
        assert np.all(coords.max(axis=0) < np.array(simsize)), \
            "hard data coordinates outside of grid"
        assert np.all(coords.min(axis=0) >= 0), "hard data coordinates must be positive indices"


# --------------------------------------------------------------------------------------
# pre/post processing (src/utils.jl:69-113)
# --------------------------------------------------------------------------------------
def float_type(dtype):
    """Element type after `prepare`: floats keep their type, anything else becomes Float64."""
    dtype = np.dtype(dtype)
    return dtype if np.issubdtype(dtype, np.floating) else np.dtype(np.float64)


def nanmask(img):
    """True where the voxel is inactive (NaN or missing)."""
    if np.ma.isMaskedArray(img):
        m = np.ma.getmaskarray(img).copy()
        data = np.ma.getdata(img)
    else:
        m = np.zeros(np.shape(img), bool)
        data = np.asarray(img)
    if np.issubdtype(data.dtype, np.floating):
        m |= np.isnan(data)
    return m


def prepare(img):
    """missing -> NaN -> 0, cast to the float type (src/utils.jl:96-102)."""
    F = float_type(np.ma.getdata(img).dtype)
    data = np.array(np.ma.getdata(img), dtype=F, copy=True)
    data[nanmask(img)] = 0
    return data


def symmetric_index(n, m):
    """Indices 0..m-1 into an axis of length n padded by mirroring with the edge repeated."""
    i = np.arange(m) % (2 * n)
    return np.where(i < n, i, 2 * n - 1 - i)


def pad_symmetric(aux, padsize):
    """padarray(aux, Pad(:symmetric, 0, padsize - min(padsize, size(aux)))) (src/utils.jl:74-79)."""
    shape = np.shape(aux)
    out_shape = tuple(max(a, p) for a, p in zip(shape, padsize))
    idx = np.ix_(*[symmetric_index(a, o) for a, o in zip(shape, out_shape)])
    if np.ma.isMaskedArray(aux):
        return aux[idx]
    return np.asarray(aux)[idx]


def unprepare(dtype, fimg):
    """Float outputs stay; other types get NaN -> missing (masked) (src/utils.jl:104-113)."""
    dtype = np.dtype(dtype)
    if np.issubdtype(dtype, np.floating):
        return fimg
    m = np.isnan(fimg)
    data = np.where(m, 0, fimg).astype(dtype)
    return np.ma.masked_array(data, mask=m)


# --------------------------------------------------------------------------------------
# disabled windows, hard data, skipped tiles, paths (src/utils.jl:18-55,115-204)
# --------------------------------------------------------------------------------------
def box_any(mask, window):
    """out[p] = any(mask[p : p + window]) over all valid p (integral-image box test)."""
    N = mask.ndim
    ii = np.zeros(tuple(s + 1 for s in mask.shape), np.int64)
    ii[tuple(slice(1, None) for _ in range(N))] = mask.astype(np.int64)
    for d in range(N):
        ii = np.cumsum(ii, axis=d)
    out_shape = tuple(s - w + 1 for s, w in zip(mask.shape, window))
    total = np.zeros(out_shape, np.int64)
    for corner in range(1 << N):
        sl = []
        sign = 1
        for d in range(N):
            if corner >> d & 1:
                sl.append(slice(window[d], window[d] + out_shape[d]))
            else:
                sl.append(slice(0, out_shape[d]))
                sign = -sign
        total += sign * ii[tuple(sl)]
    return total > 0


def finddisabled(trainimg, tilesize):
    """Windows of the TI that cover an inactive voxel (src/utils.jl:115-129)."""
    return box_any(nanmask(trainimg), tilesize)


class HardGrid(NamedTuple):
    has: np.ndarray    # key present (padsize)
    val: np.ndarray    # value, NaN where absent (padsize, float64)


def hard_grid(hard, padsize):
    has = np.zeros(padsize, bool)
    val = np.full(padsize, np.nan)
    for coord, v in hard.items():
        has[tuple(coord)] = True
        val[tuple(coord)] = np.nan if v is None else float(v)
    return HardGrid(has, val)


def tile_slices(start, tilesize):
    return tuple(slice(s, s + t) for s, t in zip(start, tilesize))


def indicator(hg, sl):
    """Hard datum present and not NaN (src/utils.jl:31-36)."""
    return hg.has[sl] & ~np.isnan(hg.val[sl])


def event(hg, sl):
    """Hard value, NaN/absent -> 0 (src/utils.jl:18-23)."""
    v = hg.val[sl]
    return np.where(np.isnan(v), 0.0, v)


def activation(hg, sl):
    """False where a hard datum is present and NaN (src/utils.jl:44-49)."""
    return ~(hg.has[sl] & np.isnan(hg.val[sl]))


def tile_start(geo, tileind):
    return tuple(i * s for i, s in zip(tileind, geo.spacing))


def lin2cart(dims, ind):
    return tuple(int(x) for x in np.unravel_index(ind, dims, order="F"))


def cart2lin(dims, cart):
    return int(np.ravel_multi_index(cart, dims, order="F"))


def findskipped(hg, geo):
    """Skipped tiles and tiles holding hard data (src/utils.jl:131-156)."""
    skipped, datainds = set(), []
    ntot = int(np.prod(geo.ntiles))
    for lin in range(ntot):
        tileind = lin2cart(geo.ntiles, lin)
        start = tile_start(geo, tileind)
        sl = tile_slices(start, geo.tilesize)
        if any(s >= S for s, S in zip(start, geo.simsize)) or not activation(hg, sl).any():
            skipped.add(lin)
        elif indicator(hg, sl).any():
            datainds.append(lin)
    return skipped, datainds


def dilate(grid):
    """3^N box dilation, outside = false (ImageMorphology.dilate)."""
    N = grid.ndim
    p = np.pad(grid, 1, constant_values=False)
    out = np.zeros_like(grid)
    for off in np.ndindex(*([3] * N)):
        out |= p[tuple(slice(o, o + s) for o, s in zip(off, grid.shape))]
    return out


def genpath(seed, extent, kind, datainds):
    """Tile visiting order (src/utils.jl:158-204); `seed` drives the Philox path stream."""
    rs = philox.PathStream(seed)
    extent = tuple(extent)
    n = int(np.prod(extent))
    path = []
    if len(datainds) == 0:
        if kind == "raster":
            path = list(range(n))
        elif kind == "random":
            path = rs.randperm(n)
        elif kind == "dilation":
            pivot = rs.below(n)
            grid = np.zeros(extent, bool)
            grid[lin2cart(extent, pivot)] = True
            path.append(pivot)
            while not grid.all():
                dil = dilate(grid)
                path.extend(int(i) for i in np.flatnonzero((dil & ~grid).ravel(order="F")))
                grid = dil
    else:
        datainds = list(datainds)
        rs.shuffle(datainds)
        grid = np.zeros(extent, bool)
        for pivot in datainds:
            grid[lin2cart(extent, pivot)] = True
            path.append(pivot)
        while not grid.all():
            dil = dilate(grid)
            path.extend(int(i) for i in np.flatnonzero((dil & ~grid).ravel(order="F")))
            grid = dil
    return path


# --------------------------------------------------------------------------------------
# distances (src/utils.jl:5-13, src/imfilter.jl:5-26)
# --------------------------------------------------------------------------------------
def imfilter_valid(img, krn, workers=None):
    """Valid cross-correlation out[p] = sum_k img[p+k] krn[k], by FFT (src/imfilter.jl:5-26)."""
    img = np.asarray(img, np.float64)
    krn = np.asarray(krn, np.float64)
    out_shape = tuple(i - k + 1 for i, k in zip(img.shape, krn.shape))
    fshape = tuple(scipy.fft.next_fast_len(i, real=True) for i in img.shape)
    axes = tuple(range(img.ndim))
    Fi = scipy.fft.rfftn(img, fshape, axes=axes, workers=workers)
    Fk = scipy.fft.rfftn(krn, fshape, axes=axes, workers=workers)
    c = scipy.fft.irfftn(Fi * np.conj(Fk), fshape, axes=axes, workers=workers)
    return c[tuple(slice(0, s) for s in out_shape)]


def imfilter_valid_direct(img, krn):
    """Same correlation by direct summation (Float64)."""
    img = np.asarray(img, np.float64)
    krn = np.asarray(krn, np.float64)
    out_shape = tuple(i - k + 1 for i, k in zip(img.shape, krn.shape))
    out = np.zeros(out_shape)
    for k in np.ndindex(*krn.shape):
        if krn[k] != 0:
            out += krn[k] * img[tuple(slice(o, o + s) for o, s in zip(k, out_shape))]
    return out


def fastdistance(img, kern, weights=None, method="direct", workers=None):
    """D[p] = |sum_k w_k img[p+k]^2 - 2 sum_k w_k kern_k img[p+k] + sum_k w_k kern_k^2|.

    method="fft" follows src/utils.jl:5-13 literally (two FFT correlations); "direct" sums
    w_k (img[p+k] - kern_k)^2 over the nonzero weights in a fixed Float64 order (direct_ssd),
    which equals it for 0/1 weights, is exact for integer-valued data and is the value the
    library's exact re-rank reproduces."""
    img = np.asarray(img, np.float64)
    kern = np.asarray(kern, np.float64)
    w = np.ones(kern.shape) if weights is None else np.asarray(weights, np.float64)
    if method == "fft":
        wk = w * kern
        A2 = imfilter_valid(img ** 2, w, workers)
        AB = imfilter_valid(img, wk, workers)
        B2 = float(np.sum(wk * kern))
        return np.abs(A2 - 2 * AB + B2)
    return direct_ssd(img, kern, w, workers)


def direct_ssd(img, kern, w, workers=None):
    """D[p] = sum over the mask of w_k (img[p+k] - kern_k)^2 in Float64, one fixed evaluation:
    offsets in column-major order (x fastest), each term and each partial sum a separately
    rounded Float64 operation (oracle/direct.c). The library's exact re-rank evaluates the same
    sequence bit for bit."""
    img = np.asarray(img, np.float64)
    kern = np.asarray(kern, np.float64)
    w = np.asarray(w, np.float64)
    N = img.ndim
    sh = tuple(img.shape) + (1,) * (3 - N)
    ts = tuple(kern.shape) + (1,) * (3 - N)
    out_shape = tuple(i - k + 1 for i, k in zip(img.shape, kern.shape))
    out3 = tuple(i - k + 1 for i, k in zip(sh, ts))
    a = np.asfortranarray(img.reshape(sh))
    kf = np.asfortranarray(kern.reshape(ts))
    wf = np.asfortranarray(w.reshape(ts))
    out = np.zeros(out3, np.float64, order="F")
    nt = workers if workers and workers > 0 else (os.cpu_count() or 1)
    rc = _native().oracle_direct_ssd(a.ctypes.data, sh[0], sh[1], sh[2], kf.ctypes.data,
                                     wf.ctypes.data, ts[0], ts[1], ts[2], out.ctypes.data, nt)
    if rc != 0:
        raise RuntimeError("oracle direct distance failed")
    return np.ascontiguousarray(out.reshape(out_shape, order="F"))


# --------------------------------------------------------------------------------------
# candidate pick (src/iqsim.jl:237), relaxation, taumodel, draw
# --------------------------------------------------------------------------------------
TIE_RTOL = 1e-6


def count_ties(d, t, boundary_is_member):
    """Near-ties of one decision: enabled positions whose distance lies within 1e-6 (relative)
    of the decision value t, |d - t| <= 1e-6 * t, evaluated in Float64. For a top-k boundary
    (t = the k-th smallest value) the k-th position itself is not counted. None when t is 0,
    Inf or NaN (no relative window)."""
    if not (np.isfinite(t) and t > 0):
        return 0
    n = int(np.count_nonzero(np.abs(d - t) <= TIE_RTOL * t))
    return n - 1 if boundary_is_member else n


def threshold_pick(D, tol, ties=None):
    """findall(vec(D .<= (1 + tol) * minimum(D))) (src/iqsim.jl:237). `ties` (a list) receives
    the number of positions within 1e-6 of the threshold."""
    d = np.asarray(D).ravel(order="F")
    thr = (1 + tol) * float(d.min())
    if ties is not None:
        ties.append(count_ties(d, thr, False))
    return np.flatnonzero(d <= thr)


def _fastintersect(A, B, nbits):
    bits = np.zeros(nbits, bool)
    bits[A] = True
    bitsB = np.zeros(nbits, bool)
    bitsB[B] = True
    return np.flatnonzero(bits & bitsB)


def relaxation(distance, auxdistances, cutoff, ties=None):
    """Candidate database under auxiliary data (src/relaxation.jl:5-39).

    partialsortperm(v, 1:k) selects the k smallest by (value, index); a stable argsort gives
    the same set. `ties` (a list) receives the near-ties (count_ties) at the dbsize boundary of
    the primary distance plus those at each auxiliary boundary of the final round."""
    d = np.asarray(distance, np.float64).ravel(order="F")
    enabled = ~np.isinf(d)
    npat = int(enabled.sum())
    if npat == 0:
        raise ValueError("relaxation: every training-image pattern is disabled")
    allzero = bool(np.all(d[enabled] == 0))
    dbsize = npat if allzero else math.ceil(cutoff * npat)
    overlapdb = np.argsort(d, kind="stable")[:dbsize]
    naux = len(auxdistances)
    softdist = [np.asarray(a, np.float64).ravel(order="F").copy() for a in auxdistances]
    softdb = [np.zeros(0, np.int64) for _ in range(naux)]
    frac = 0.1 * (dbsize / npat)
    while True:
        softdbsize = math.ceil(frac * npat)
        patterndb = np.sort(overlapdb)
        for n in range(naux):
            softdist[n][softdb[n]] = np.inf
            k = softdbsize - len(softdb[n])
            new = np.argsort(softdist[n], kind="stable")[:max(k, 0)]
            softdb[n] = np.concatenate([softdb[n], new])
            patterndb = _fastintersect(patterndb, softdb[n], len(d))
            if len(patterndb) == 0:
                break
        if len(patterndb):
            break
        frac = min(frac + 0.1, 1.0)
    if ties is not None:
        # boundaries of proper top-k selections only (0 < k < number of positions)
        nt = 0
        if dbsize < len(d):
            nt += count_ties(d, d[np.argsort(d, kind="stable")[dbsize - 1]], True)
        for n in range(naux):
            a = np.asarray(auxdistances[n], np.float64).ravel(order="F")
            k = len(softdb[n])
            if 0 < k < len(a):
                nt += count_ties(a, a[np.argsort(a, kind="stable")[k - 1]], True)
        ties.append(nt)
    return patterndb


def relaxation_frac_sequence(npat, dbsize):
    """softdbsize values visited by the relaxation loop, in order (src/relaxation.jl:20-36)."""
    seq = []
    frac = 0.1 * (dbsize / npat)
    while True:
        seq.append(math.ceil(frac * npat))
        if frac >= 1.0:
            break
        frac = min(frac + 0.1, 1.0)
    return seq


def dense_ranks(values):
    """Rank of each value among the distinct values, ties sharing a rank (src/taumodel.jl:19-28)."""
    order = np.argsort(values, kind="stable")
    sv = values[order]
    step = np.ones(len(sv), np.int64)
    step[1:] = (sv[1:] > sv[:-1]).astype(np.int64)
    r = np.empty(len(sv), np.int64)
    r[order] = np.cumsum(step)
    return r


def taumodel(events, D1, Dn):
    """Tau-model pattern weights (src/taumodel.jl:5-45), same operation order."""
    n = len(events)
    if n == 1:
        return np.array([1.0])
    srcs = [np.asarray(D1, np.float64).ravel(order="F")[events]]
    srcs += [np.asarray(Dj, np.float64).ravel(order="F")[events] for Dj in Dn]
    Pcols = []
    for v in srcs:
        r = dense_ranks(v).astype(np.float64)
        P = n - r + 1
        P = P / P.sum()
        Pcols.append(P)
    x0 = (1 - 1 / n) / (1 / n)
    prod = np.ones(n)
    for P in Pcols:
        X = (1 - P) / P
        prod = prod * (X / x0)
    x = x0 * prod
    return 1 / (1 + x)


DRAW_CHUNK = 256


def sample_index(u, w):
    """Index i of the draw: t = u * sum(w), first i with cumsum(w)[i] >= t (StatsBase walk).

    Sums: chunks of DRAW_CHUNK summed left to right; the running total over chunk totals
    left to right; within the chosen chunk, base + (left-to-right partial sum)."""
    w = np.asarray(w, np.float64)
    n = len(w)
    nch = (n + DRAW_CHUNK - 1) // DRAW_CHUNK
    pad = np.zeros(nch * DRAW_CHUNK)
    pad[:n] = w
    csum = np.cumsum(pad.reshape(nch, DRAW_CHUNK), axis=1)
    prefix = np.cumsum(csum[:, -1])
    total = prefix[-1]
    t = u * total
    j = int(np.argmax(prefix >= t)) if np.any(prefix >= t) else nch - 1
    base = 0.0 if j == 0 else prefix[j - 1]
    cw = base + csum[j]
    lo = j * DRAW_CHUNK
    hits = np.flatnonzero(cw[: min(DRAW_CHUNK, n - lo)] >= t)
    return lo + (int(hits[0]) if len(hits) else min(DRAW_CHUNK, n - lo) - 1)


def pick(D, Ds, tol, seed, tile, real, ties=None):
    """Candidate set, weights and the drawn linear index for one tile of one realization.
    `ties` (a list) receives the pick's near-tie count."""
    if len(Ds) == 0:
        cands = threshold_pick(D, tol, ties)
    else:
        cands = relaxation(D, Ds, tol, ties)
    w = taumodel(cands, D, Ds)
    u = philox.draw_uniform(seed, tile, real)
    i = sample_index(u, w)
    return int(cands[i]), cands, w


# --------------------------------------------------------------------------------------
# graph cut (src/graphcut.jl:5-84) via oracle/bkcut.c
# --------------------------------------------------------------------------------------
def graphcut(A, B, dim, return_cost=False):
    """Boolean mask of the min-error cut along `dim` (0-based); True = keep A."""
    A = np.asarray(A)
    B = np.asarray(B)
    assert A.shape == B.shape, "arrays must have the same size for cut"
    dt = np.float32 if (A.dtype == np.float32 and B.dtype == np.float32) else np.float64
    Af = np.asfortranarray(A, dtype=dt)
    Bf = np.asfortranarray(B, dtype=dt)
    sz = (ctypes.c_longlong * A.ndim)(*A.shape)
    mask = np.zeros(A.shape, np.uint8, order="F")
    cost = ctypes.c_double(0)
    rc = _native().oracle_graphcut(Af.ctypes.data, Bf.ctypes.data, Af.itemsize, A.ndim, sz, dim,
                                   mask.ctypes.data, ctypes.byref(cost))
    if rc != 0:
        raise RuntimeError("oracle graphcut failed (%d)" % rc)
    m = mask.astype(bool)
    return (m, cost.value) if return_cost else m


def capacities(A, B):
    """Edge capacities in the order of oracle_capacities (tests)."""
    A = np.asarray(A)
    dt = np.float32 if A.dtype == np.float32 else np.float64
    Af = np.asfortranarray(A, dtype=dt)
    Bf = np.asfortranarray(B, dtype=dt)
    sz = (ctypes.c_longlong * A.ndim)(*A.shape)
    n = _native().oracle_capacities(Af.ctypes.data, Bf.ctypes.data, Af.itemsize, A.ndim, sz, None)
    out = np.zeros(n)
    _native().oracle_capacities(Af.ctypes.data, Bf.ctypes.data, Af.itemsize, A.ndim, sz,
                                out.ctypes.data)
    return out


def cut_cost(A, B, mask):
    """Sum of capacities of lattice edges whose ends lie on different sides of `mask`."""
    A = np.asarray(A)
    caps = capacities(A, B)
    shape = A.shape
    i = 0
    total = 0.0
    for d in range(A.ndim):
        if shape[d] < 2:
            continue
        lo = [slice(None)] * A.ndim
        hi = [slice(None)] * A.ndim
        lo[d] = slice(0, shape[d] - 1)
        hi[d] = slice(1, shape[d])
        diff = (mask[tuple(lo)] != mask[tuple(hi)]).ravel(order="F")
        n = diff.size
        total += float(np.sum(caps[i:i + n][diff]))
        i += n
    return total


# --------------------------------------------------------------------------------------
# the simulation (src/iqsim.jl:50-315)
# --------------------------------------------------------------------------------------
def iqsim(trainimg, tilesize, simsize=None, overlap=None, soft=(), hard=None, tol=0.1,
          path="raster", nreal=1, debug=False, seed=0, method="direct", workers=None,
          trace=None, max_steps=None, real0=0, ties=None):
    """Image quilting simulation, the reference's loop in Float64.

    `seed` keys the Philox streams (path and draws). `method` picks the distance form
    ("direct" exact SSD or "fft" as the reference). `trace`, when a list, receives one tuple
    (real, tile, rind, ncand) per simulated tile. `max_steps` stops each realization after
    that many tiles (used to time a bounded sample). `real0` is the global index of the first
    realization (its Philox draws use counter (tile, real0 + r)). `ties`, when a list, receives
    the near-tie count of every pick (count_ties)."""
    tisize = tuple(np.shape(trainimg))
    N = len(tisize)
    tilesize = tuple(int(t) for t in tilesize)
    simsize = tisize if simsize is None else tuple(int(s) for s in simsize)
    overlap = tuple([1 / 6] * N) if overlap is None else tuple(overlap)
    hard = {} if hard is None else {tuple(int(c) for c in k): v for k, v in hard.items()}
    soft = list(soft)
    check_args(tisize, tilesize, simsize, overlap, tol, path, nreal, soft, hard)
    geo = geometry(tisize, tilesize, simsize, overlap)

    T = np.ma.getdata(trainimg).dtype
    TI = prepare(trainimg)
    SOFT = [(prepare(pad_symmetric(aux, geo.padsize)), prepare(auxTI)) for aux, auxTI in soft]
    disabled = finddisabled(trainimg, tilesize)
    hg = hard_grid(hard, geo.padsize)
    skipped, datainds = findskipped(hg, geo)
    simpath = genpath(seed, geo.ntiles, path, datainds)

    reals, cuts, voxs = [], [], []
    for real in range(nreal):
        simgrid = np.zeros(geo.padsize, TI.dtype)
        cutgrid = np.zeros(geo.padsize) if debug else None
        pasted = set()
        nsteps = 0
        for ind in simpath:
            if ind in skipped:
                continue
            if max_steps is not None and nsteps >= max_steps:
                break
            nsteps += 1
            tileind = lin2cart(geo.ntiles, ind)
            start = tile_start(geo, tileind)
            tsl = tile_slices(start, tilesize)
            simdev = simgrid[tsl]

            ovlmask = np.zeros(tilesize, bool)
            slabs = []
            for d in range(N):
                prev = tuple(t - 1 if i == d else t for i, t in enumerate(tileind))
                nxt = tuple(t + 1 if i == d else t for i, t in enumerate(tileind))
                if geo.ovlsize[d] > 1 and prev in pasted:
                    sl = tuple(slice(0, geo.ovlsize[d]) if i == d else slice(None) for i in range(N))
                    ovlmask[sl] = True
                    slabs.append((d, sl, False))
                if geo.ovlsize[d] > 1 and nxt in pasted:
                    sl = tuple(slice(geo.spacing[d], tilesize[d]) if i == d else slice(None)
                               for i in range(N))
                    ovlmask[sl] = True
                    slabs.append((d, sl, True))
            ovldist = fastdistance(TI, simdev, ovlmask, method, workers)
            ovldist[disabled] = np.inf

            hardtile = False
            if hard:
                hm = indicator(hg, tsl)
                if hm.any():
                    harddist = fastdistance(TI, event(hg, tsl), hm, method, workers)
                    harddist[disabled] = np.inf
                    hardtile = True

            softdists = []
            for AUX, AUXTI in SOFT:
                sd = fastdistance(AUXTI, AUX[tsl], None, method, workers)
                sd[disabled] = np.inf
                softdists.append(sd)

            if hardtile:
                D, Ds = harddist, [ovldist] + softdists
            else:
                D, Ds = ovldist, softdists

            rind, cands, _ = pick(D, Ds, tol, seed, ind, real0 + real, ties)
            if trace is not None:
                trace.append((real, ind, rind, len(cands)))
            rstart = lin2cart(geo.distsize, rind)
            TIdev = TI[tile_slices(rstart, tilesize)]

            cutmask = np.zeros(tilesize, bool)
            for d, sl, is_next in slabs:
                M = graphcut(simdev[sl], TIdev[sl], d)
                cutmask[sl] |= (~M) if is_next else M
            simdev[~cutmask] = TIdev[~cutmask]
            if debug:
                cutgrid[tsl] = cutmask
            pasted.add(tileind)

        if debug:
            voxs.append(float(np.sum(cutgrid)) / geo.ovlvol)
        for coord, val in hard.items():
            simgrid[coord] = np.nan if val is None else val
        if debug:
            for coord, val in hard.items():
                if val is None or np.isnan(val):
                    cutgrid[coord] = np.nan
        crop = tuple(slice(0, s) for s in simsize)
        reals.append(unprepare(T, simgrid[crop].copy()))
        if debug:
            cuts.append(cutgrid[crop].copy())
    return (reals, cuts, voxs) if debug else reals


def voxelreuse(trainimg, tilesize, overlap=None, nreal=10, **kw):
    """Mean and std of the voxel reuse on a 2-tile grid (src/voxelreuse.jl:18-41)."""
    N = np.ndim(trainimg)
    overlap = tuple([1 / 6] * N) if overlap is None else tuple(overlap)
    ovlsize = [math.ceil(o * t) for o, t in zip(overlap, tilesize)]
    ntiles = [2 if o > 1 else 1 for o in ovlsize]
    simsize = tuple(n * (t - o) + o for n, t, o in zip(ntiles, tilesize, ovlsize))
    _, _, voxs = iqsim(trainimg, tilesize, simsize, overlap=overlap, nreal=nreal, debug=True, **kw)
    mu = float(np.mean(voxs))
    sd = float(np.std(voxs, ddof=1)) if len(voxs) > 1 else float("nan")
    return mu, sd
