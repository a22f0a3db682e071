"""Benchmark of the GB300 image-quilting path: simulated voxels/s.

Default workload (N=1), config 4: a 4-facies categorical TI 256x256x128 (argmax over four
seeded Gaussian fields smoothed with sigma=(10,10,3), codes 0..3), tile 32x32x16, overlap 1/4,
tol 0.05, output 512x512x128, nreal 64, through the learned proposal: training pairs are
captured from full-scan runs (seeds 1..n, the first tiles of the path), the encoder is trained
by the library's own kernels, and then a step is one complete iqsim call (64 realizations,
2.1 G voxels) with shortlists, exact sums at the shortlisted positions and the recall monitor
(full-scan fallback below 0.99 sampled recall). One step of the plain full-scan form on the
same workload is timed beside it (`plain`, `speedup_vs_plain`). Other workloads: cfg3 (the
same with 32 realizations), cfg2 (3-D continuous with hard and soft data, plain form:
TI 100x100x50 lognormal, tile 24x24x12, tol 0.1, output 200x200x100, nreal 16, 500 hard
data, one soft variable), cfg1 (2-D binary, plain).

  value : voxels/s with inputs resident in HBM (TI uploaded before timing; hard and soft
          data and the outputs in device memory), CUDA events on the library's stream
  e2e   : the same through the C ABI with host buffers: TI upload, hard/soft upload and the
          copy of the realizations back to the host inside the timed region
  cpu_baseline / --impl reference : the CPU oracle (Float64, FFT correlation with scipy.fft
          on all host cores, C Boykov-Kolmogorov cut) on a bounded sample of the same
          workload: realization 0, the first tiles of the path, scaled to voxels/s
N>1 (torchrun): the ranks are shards of one call (weak scaling, no data-path collective):
every rank runs nreal realizations with the same seed and real0 = rank * nreal, so N ranks
together produce realizations [0, N * nreal) of one call, each drawing the Philox streams of
its global realization index.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("simulated voxels/s on 1 GB300: plain vs BF16+learned-proposal form at "
          "≥0.99 recall")


# ---------------------------------------------------------------------------------------
# synthetic workloads (seeded)
# ---------------------------------------------------------------------------------------
def gaussian_field(shape, sigma, seed):
    import scipy.ndimage as ndi
    rng = np.random.default_rng(seed)
    f = ndi.gaussian_filter(rng.standard_normal(shape), sigma, mode="wrap")
    return (f - f.mean()) / f.std()


def workload(name):
    import scipy.ndimage as ndi
    if name == "cfg2":
        ti = np.exp(gaussian_field((100, 100, 50), (6, 6, 2), 1)).astype(np.float32)
        simsize = (200, 200, 100)
        f2 = np.exp(gaussian_field(simsize, (6, 6, 2), 2)).astype(np.float32)
        rng = np.random.default_rng(3)
        pts = np.stack([rng.integers(0, s, 500) for s in simsize], axis=1)
        hard = {}
        for c in pts:
            hard[tuple(int(v) for v in c)] = float(f2[tuple(c)])
        aux = ndi.gaussian_filter(f2, 4).astype(np.float32)
        auxti = ndi.gaussian_filter(ti, 4).astype(np.float32)
        return dict(name="cfg2", ti=ti, tilesize=(24, 24, 12), simsize=simsize,
                    overlap=(0.25, 0.25, 0.25), tol=0.1, nreal=16, hard=hard,
                    soft=[(aux, auxti)], path="raster",
                    desc="3-D continuous: TI 100x100x50 f32 lognormal, tile 24x24x12, "
                         "overlap 1/4, tol 0.1, out 200x200x100, nreal 16, 500 hard, 1 soft")
    if name in ("cfg3", "cfg4"):
        # four facies: argmax over four independent fields, codes 0..3
        f = np.stack([gaussian_field((256, 256, 128), (10, 10, 3), 10 + i) for i in range(4)])
        ti = np.argmax(f, axis=0).astype(np.float32)
        nreal = 32 if name == "cfg3" else 64
        return dict(name=name, ti=ti, tilesize=(32, 32, 16), simsize=(512, 512, 128),
                    overlap=(0.25, 0.25, 0.25), tol=0.05, nreal=nreal, hard={}, soft=[],
                    path="raster",
                    desc="3-D categorical: TI 256x256x128 (4 facies, codes 0..3), tile 32x32x16, "
                         "overlap 1/4, tol 0.05, out 512x512x128, nreal %d" % nreal)
    if name == "cfg1":
        f = gaussian_field((128, 128), 8, 1)
        ti = (f > np.quantile(f, 0.6)).astype(np.float64)
        return dict(name="cfg1", ti=ti, tilesize=(32, 32), simsize=(256, 256),
                    overlap=(1 / 6, 1 / 6), tol=0.1, nreal=1, hard={}, soft=[],
                    path="raster",
                    desc="2-D binary: TI 128x128 f64, tile 32x32, overlap 1/6, tol 0.1, "
                         "out 256x256, nreal 1")
    raise ValueError(name)


# ---------------------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------------------
class Clocks:
    """nvidia-smi clock/throttle samples taken during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(kernel, workload_name, columns=None):
    """DRAM bytes per launch of `kernel` from a committed ncu summary, if one exists.

    The summary gives `dram_bytes_per_launch:` of the captured launch and, for the correlation,
    `columns_per_launch:` of that launch; the distance maps it writes dominate its traffic and
    grow with the columns, so the figure is scaled to `columns` (this run's mean)."""
    fn = os.path.join(ROOT, "profiles", "%s_%s.txt" % (kernel, workload_name))
    if not os.path.exists(fn):
        return None
    vals = {}
    for ln in open(fn):
        if ":" in ln:
            k, v = ln.split(":", 1)
            try:
                vals[k.strip()] = float(v.split()[0])
            except (ValueError, IndexError):
                pass
    b = vals.get("dram_bytes_per_launch")
    if b is None:
        return None
    c = vals.get("columns_per_launch")
    if c and columns:
        b *= columns / c
    return b


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        return dist, rank, world
    return None, 0, 1


def reduce_max(dist, value):
    if dist is None:
        return value
    import torch
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def step_seed(step):
    """Seed of one simulation call, the same on every rank."""
    return 1000 + 7919 * step


def step_real0(rank, nreal):
    """First global realization of `rank`'s shard: the ranks' blocks of nreal realizations
    are consecutive, so together they are the realizations of one call (no data moves)."""
    return rank * nreal


def aggregate_rate(units_per_rank_step, steps, world, ms_max):
    """Whole-job rate: the units every rank processed over the slowest rank's time."""
    return units_per_rank_step * steps * world / (ms_max / 1e3)


# ---------------------------------------------------------------------------------------
# CPU oracle baseline (bounded sample)
# ---------------------------------------------------------------------------------------
def cpu_sample(W, budget_s=15.0, max_steps=None):
    """Run the oracle on realization 0 for a bounded number of tiles; returns voxels/s
    scaled from the fraction of tiles done, plus a description."""
    from oracle import iqsim_oracle as O
    workers = os.cpu_count()
    simvol = int(np.prod(W["simsize"]))
    geo = O.geometry(W["ti"].shape, W["tilesize"], W["simsize"], W["overlap"])
    hg = O.hard_grid(W["hard"], geo.padsize)
    skipped, _ = O.findskipped(hg, geo)
    ntiles = int(np.prod(geo.ntiles)) - len(skipped)
    # calibrate: time a few tiles, then size the sample to the budget
    steps = max_steps
    if steps is None:
        t0 = time.perf_counter()
        O.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], soft=W["soft"],
                hard=W["hard"], tol=W["tol"], path=W["path"], nreal=1, seed=0, method="fft",
                workers=workers, max_steps=4)
        per = (time.perf_counter() - t0) / 4
        steps = int(max(4, min(ntiles, budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    O.iqsim(W["ti"], W["tilesize"], W["simsize"], overlap=W["overlap"], soft=W["soft"],
            hard=W["hard"], tol=W["tol"], path=W["path"], nreal=1, seed=0, method="fft",
            workers=workers, max_steps=steps)
    dt = time.perf_counter() - t0
    vps = simvol * (steps / ntiles) / dt
    return vps, steps, ntiles, dt, workers


# ---------------------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------------------
def run_reference(args, W, dist, rank, world):
    if rank != 0:
        return
    vals = []
    for i in range(args.warmup + args.steps):
        vps, steps, ntiles, dt, cores = cpu_sample(W, budget_s=args.cpu_budget)
        if i >= args.warmup:
            vals.append((vps, dt))
    v = float(np.mean([x[0] for x in vals]))
    ms = float(np.mean([x[1] for x in vals])) * 1e3
    line = {"metric": METRIC, "value": v, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (seeded Gaussian fields)",
            "config": {"workload": W["desc"], "global_batch": W["nreal"],
                       "sample": "realization 0, first %d of %d tiles per step" % (steps, ntiles)},
            "cpu_baseline": {"value": v, "unit": "voxels/s", "cores": cores, "kind": "port",
                             "sample": "realization 0, first %d of %d tiles, scaled by the "
                                       "tile fraction" % (steps, ntiles)},
            "e2e": {"value": v, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FORMS = {"plain": "plain: every training-image position scanned (tensor-core correlation, "
                  "FP32-accurate split FP16/TF32 MMAs, exact re-rank near each decision)",
         "proposal": "BF16 + learned proposal: a 3-D conv encoder (BF16 weights, FP32 "
                     "accumulation) shortlists positions, the exact distance is summed there, "
                     "full-scan fallback below 0.99 sampled recall"}


def train_proposal(args, W, ctx, lib, _lib, p, hd, sd, out_d):
    """Training pairs from full-scan runs (seeds 1..n, the first tiles of the path), then Adam
    steps of the library's own forward and backward kernels. Returns what was done."""
    import ctypes
    t0 = time.perf_counter()
    ctx.lp_init(W["tilesize"], seed=0)
    ctx.set_option("lp.capture", args.lp_pairs)
    nreal0, seed0 = p.nreal, p.seed
    p.nreal = args.lp_capture_reals
    ctx.set_option("sim.max_steps", args.lp_capture_steps)
    for s in range(1, args.lp_seeds + 1):
        p.seed = s
        _lib.check(lib.iq_simulate(ctx.h, ctypes.byref(p), ctypes.byref(hd), len(W["soft"]),
                                   sd if W["soft"] else None, out_d.data_ptr(), None, None))
        if ctx.lp_stats()["captured"] >= args.lp_pairs:
            break
    ctx.set_option("sim.max_steps", -1)
    p.nreal, p.seed = nreal0, seed0
    pairs = int(ctx.lp_stats()["captured"])
    t1 = time.perf_counter()
    l0, l1 = ctx.lp_train(args.lp_train_steps, batch=128, nneg=32, lr=2e-3, temp=8.0, seed=7)
    t2 = time.perf_counter()
    ctx.set_option("lp.capture", 0)
    return {"pairs": pairs, "capture_s": t1 - t0, "train_steps": args.lp_train_steps,
            "train_s": t2 - t1, "loss_first": l0, "loss_last": l1,
            "pairs_from": "full-scan runs, seeds 1..%d, first %d tiles x %d realizations" % (
                args.lp_seeds, args.lp_capture_steps, args.lp_capture_reals)}


def proposal_roofline(dom, prof, lp_kernels, W, peaks, peak_kind, st, args):
    """Roofline of the proposal's dominant kernel: the scan against the measured tensor peak
    (2 x positions x columns x 64 FLOPs per launch); the shortlist pick against HBM (4 bytes of
    the training image read per shortlisted position and mask offset, the direct sums)."""
    ms, n, work = prof[dom]
    if dom == "lp.scan":
        ach = work / (ms / 1e3) / 1e12
        return {"bound": "tensor", "kernel": dom, "achieved": ach, "unit": "TFLOP/s",
                "peak": peaks.get("bf16_tflops"), "peak_kind": "%s (bf16 dense, burst)" % peak_kind,
                "frac": ach / peaks.get("bf16_tflops"), "traffic": None,
                "flops_per_launch": work / n if n else None}
    ovl = [math.ceil(o * t) for o, t in zip(W["overlap"], W["tilesize"])]
    K = int(np.prod(W["tilesize"])) - int(np.prod([t - o for t, o in zip(W["tilesize"], ovl)]))
    cols = st["cols_shortlist"] if st else 0
    planes = bool(np.isin(W["ti"], (0, 1, 2, 3)).all()) and W["tilesize"][0] <= 32
    per = 0.25 if planes else 1.0
    byts = cols * (st["mean_shortlist"] if st else 0) * K * per
    ach = byts / (ms / 1e3) / 1e9 if ms else None
    return {"bound": "hbm", "kernel": dom, "achieved": ach, "unit": "GB/s",
            "peak": peaks.get("hbm_gbs"), "peak_kind": "%s (copy)" % peak_kind,
            "frac": ach / peaks.get("hbm_gbs") if ach else None,
            "traffic": profile_traffic("lp_pick_kernel", W["name"]),
            "bytes_note": "algorithmic bytes = shortlisted positions x interior mask offsets x "
                          "%s B (the %s the exact sums read; the image is L2-resident and the "
                          "kernel is bound by L1 line lookups and integer issue, not by HBM)" % (
                              per, "2-bit codes" if planes else "byte codes")}


def cut_roofline(prof, cut_nodes, peaks, peak_kind, W):
    """Roofline of the graph cut: the slab values it must read (A and B, 4 bytes each per node)
    and the mask it writes (1 byte per node), over its time, against HBM; the kernel itself is
    bound by barrier and atomic latency (push-relabel rounds), not by bandwidth."""
    ms, n, _ = prof["graphcut"]
    nodes = cut_nodes[2]
    byts = 9.0 * nodes
    ach = byts / (ms / 1e3) / 1e9 if ms else None
    return {"bound": "hbm", "kernel": "graphcut", "achieved": ach, "unit": "GB/s",
            "peak": peaks.get("hbm_gbs"), "peak_kind": "%s (copy)" % peak_kind,
            "frac": ach / peaks.get("hbm_gbs") if ach else None,
            "traffic": profile_traffic("cut_kernel", W["name"]),
            "bytes_note": "algorithmic bytes = 9 per slab node (A and B read, mask written); "
                          "%d slabs of %.0f nodes on average; latency-bound rounds" % (
                              cut_nodes[1], nodes / cut_nodes[1] if cut_nodes[1] else 0)}


def run_ours(args, W, dist, rank, world):
    import ctypes

    import torch
    from __graft_entry__ import _package
    iq = _package()
    from iqgpu import _lib
    lib = _lib.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = iq.Context(dev)
    for opt in args.option:
        name, val = opt.split("=", 1)
        ctx.set_option(name, int(val))
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    N = W["ti"].ndim
    nreal = W["nreal"]
    simvol = int(np.prod(W["simsize"]))
    voxels = simvol * nreal

    # host inputs (column-major)
    ti_h = np.asfortranarray(W["ti"])
    ti_dt = _lib.IQ_F32 if ti_h.dtype == np.float32 else _lib.IQ_F64
    coords_h = np.array(list(W["hard"].keys()), dtype=np.int64).reshape(len(W["hard"]), N)
    vals_h = np.array(list(W["hard"].values()), dtype=np.float64)
    soft_h = [(np.asfortranarray(a, np.float32), np.asfortranarray(b, np.float32))
              for a, b in W["soft"]]
    out_h = np.empty(voxels, np.float32)
    # device copies for the resident arm
    coords_d = torch.from_numpy(coords_h).cuda(dev) if len(vals_h) else None
    vals_d = torch.from_numpy(vals_h).cuda(dev) if len(vals_h) else None
    soft_d = [(torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda(dev),
               torch.from_numpy(np.ascontiguousarray(b.ravel(order="F"))).cuda(dev))
              for a, b in soft_h]
    out_d = torch.empty(voxels, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    p = _lib.SimParams()
    p.ndim = N
    for d in range(N):
        p.tilesize[d] = W["tilesize"][d]
        p.simsize[d] = W["simsize"][d]
        p.overlap[d] = W["overlap"][d]
    p.tol = W["tol"]
    p.path = _lib.PATHS[W["path"]]
    p.nreal = nreal
    p.debug = 0

    def make_io(device):
        if device:
            hd = _lib.HardData(len(vals_h), coords_d.data_ptr() if coords_d is not None else None,
                               vals_d.data_ptr() if vals_d is not None else None)
            srcs = [(a.data_ptr(), b.data_ptr()) for a, b in soft_d]
        else:
            hd = _lib.HardData(len(vals_h), coords_h.ctypes.data if len(vals_h) else None,
                               vals_h.ctypes.data if len(vals_h) else None)
            srcs = [(a.ctypes.data, b.ctypes.data) for a, b in soft_h]
        sd = (_lib.SoftData * max(len(srcs), 1))()
        for i, (a, b) in enumerate(srcs):
            sd[i].aux = a
            sd[i].auxti = b
            for d in range(3):
                sd[i].auxsize[d] = soft_h[i][0].shape[d] if d < N else 1
        return hd, sd

    hd_dev, sd_dev = make_io(True)
    hd_host, sd_host = make_io(False)
    size = _lib.i64arr(ti_h.shape)

    p.real0 = step_real0(rank, nreal)

    def step_resident(i):
        p.seed = step_seed(i)
        _lib.check(lib.iq_simulate(ctx.h, ctypes.byref(p), ctypes.byref(hd_dev), len(soft_d),
                                   sd_dev if soft_d else None, out_d.data_ptr(), None, None))

    def step_e2e(i):
        p.seed = step_seed(i)
        _lib.check(lib.iq_set_ti(ctx.h, ti_h.ctypes.data, ti_dt, N, size))
        _lib.check(lib.iq_simulate(ctx.h, ctypes.byref(p), ctypes.byref(hd_host), len(soft_h),
                                   sd_host if soft_h else None, out_h.ctypes.data, None, None))

    # ---- resident arm ----
    _lib.check(lib.iq_set_ti(ctx.h, ti_h.ctypes.data, ti_dt, N, size))
    lp_info = None
    if args.form == "proposal":
        if args.lp_load:
            # parameters trained by an earlier run of this bench (--lp-save), for profiling runs
            ctx.lp_set_params(W["tilesize"], np.load(args.lp_load))
            lp_info = {"loaded": os.path.basename(args.lp_load)}
        else:
            lp_info = train_proposal(args, W, ctx, lib, _lib, p, hd_dev, sd_dev, out_d)
            if args.lp_save:
                np.save(args.lp_save, ctx.lp_params())
        ctx.set_option("lp.enable", 1)
        ctx.set_option("lp.k", args.lp_k)
        ctx.set_option("lp.kmax", args.lp_kmax)
    for i in range(args.warmup):
        step_resident(i)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = Clocks(dev)
    clocks.start()
    time.sleep(0.3)
    ctx.profile(True)
    l0 = ctx.launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for i in range(args.steps):
        step_resident(args.warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches - l0
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    prof = {k: ctx.profile_get(k) for k in ("corr", "pick", "graphcut", "paste")}
    mma = ctx.profile_get("corr.mma")
    mma16 = ctx.profile_get("corr.mma16")
    cols = ctx.profile_get("corr.columns")
    counters = {k: ctx.profile_get(k) for k in ("graphcut.rounds", "graphcut.levels",
                                                 "pick.iterations", "pick.candidates")}
    counters = {k: {"mean": (v[2] / v[1]) if v[1] else None, "ctas": v[1]}
                for k, v in counters.items()}
    for k in ("graphcut.max_rounds", "graphcut.max_levels"):
        counters[k] = ctx.profile_get(k)[2]
    # tensor-core correlation: mean SM cycles per CTA in each phase
    tc = {k: ctx.profile_get("corr." + k) for k in ("loop", "wait_full", "wait_afull",
                                                    "wait_done", "producer_wait",
                                                    "producer_loop", "epilogue", "issue",
                                                    "mma_units")}
    counters["corr_cycles_per_cta"] = {k: (v[2] / v[1]) if v[1] else None for k, v in tc.items()}
    gc = {k: ctx.profile_get("graphcut." + k) for k in ("setup_cycles", "round_cycles",
                                                        "relabel_cycles", "active_nodes",
                                                        "nodes")}
    counters["graphcut_cycles_per_cta"] = {k: (v[2] / v[1]) if v[1] else None for k, v in gc.items()}
    pk = {k: ctx.profile_get("pick." + k) for k in ("select_cycles", "weight_cycles", "draw_cycles",
                                                   "band_cycles", "ev1", "ev2", "ev3")}
    counters["pick_cycles_per_cta"] = {k: (v[2] / v[1]) if v[1] else None for k, v in pk.items()}
    cut_nodes = ctx.profile_get("graphcut.nodes")  # (ms, CTAs, nodes)
    lp_stats = ctx.lp_stats() if args.form == "proposal" else None
    lp_kernels = {k: ctx.profile_get(k) for k in ("lp.encode", "lp.scan", "lp.pick", "lp.monitor")} \
        if args.form == "proposal" else {}
    ctx.profile(False)
    ms_max = reduce_max(dist, ms)
    barrier(dist)
    plain = None
    if args.form == "proposal" and not args.no_plain:
        # the full-scan form on the same workload, for the comparison the metric names
        ctx.set_option("lp.enable", 0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ep0 = torch.cuda.Event(enable_timing=True)
        ep1 = torch.cuda.Event(enable_timing=True)
        ep0.record(stream)
        for i in range(args.plain_steps):
            step_resident(10000 + i)
        ep1.record(stream)
        torch.cuda.synchronize()
        ms_plain = max(ep0.elapsed_time(ep1), (time.perf_counter() - t0) * 1e3) / args.plain_steps
        plain = {"value": voxels * world / (ms_plain / 1e3), "unit": "voxels/s",
                 "ms_per_step": ms_plain, "steps": args.plain_steps}
        ctx.set_option("lp.enable", 1)
        barrier(dist)

    # ---- end-to-end arm (host buffers through the C ABI) ----
    if args.no_e2e:
        step_e2e = lambda i: None  # noqa: E731  (profiling runs: resident arm only)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    for i in range(1):
        step_e2e(i)
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for i in range(e2e_steps):
        step_e2e(args.warmup + i)
    e3.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3
    ms_e2e = max(e2.elapsed_time(e3), wall)
    ms_e2e_max = reduce_max(dist, ms_e2e)
    h2d = ti_h.nbytes + coords_h.nbytes + vals_h.nbytes + sum(a.nbytes + b.nbytes for a, b in soft_h)
    d2h = out_h.nbytes

    if rank != 0:
        ctx.close()
        return
    value = aggregate_rate(voxels, args.steps, world, ms_max)
    e2e_value = aggregate_rate(voxels, e2e_steps, world, ms_e2e_max)
    peaks, peak_kind = measured_peaks()
    for k, v in lp_kernels.items():
        if v[1]:
            prof[k] = v
    shares = {k: v[0] for k, v in prof.items()}
    dom = max(shares, key=lambda k: shares[k])
    corr_ms, corr_n, corr_flops = prof["corr"]
    roof = {"bound": "tensor", "kernel": "corr",
            "achieved": (corr_flops / corr_n) / (corr_ms / corr_n / 1e3) / 1e12 if corr_n else None,
            "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
            "peak_kind": "%s (bf16 dense, burst)" % peak_kind,
            "flops_per_launch": corr_flops / corr_n if corr_n else None,
            "traffic": profile_traffic("corr_tc_kernel", W["name"], cols[2] / cols[1] if cols[1] else None),
            "mma_tflops_issued": (mma[2] / (corr_ms / 1e3) / 1e12) if corr_ms and mma[2] else None,
            "mma_tflops_issued_fp16": (mma16[2] / (corr_ms / 1e3) / 1e12) if corr_ms else None,
            "note": "achieved = algorithmic FLOPs (2 x positions x mask offsets x templates) "
                    "over the correlation's time; the tensor pipe issues FP16 (or TF32) MMAs, "
                    "three per K-step for FP32 data (hi*hi + hi*lo + lo*hi), over padded "
                    "positions and offsets, counted in mma_tflops_issued; mma_frac is that work "
                    "over its peak (FP16 at the bf16 rate, TF32 at half of it)"}
    if roof["achieved"] is not None and roof["peak"]:
        roof["frac"] = roof["achieved"] / roof["peak"]
        if roof["mma_tflops_issued"]:
            f16 = roof["mma_tflops_issued_fp16"] or 0.0
            tf32 = roof["mma_tflops_issued"] - f16
            roof["mma_frac"] = f16 / roof["peak"] + tf32 / (roof["peak"] / 2)
    kernel_share = {k: {"ms": round(v[0], 3), "launches": v[1],
                        "share_of_step": round(v[0] / ms, 4) if ms else None}
                    for k, v in prof.items()}
    cpu = None
    if not args.no_cpu_baseline:
        vps, steps, ntiles, dt, cores = cpu_sample(W, budget_s=args.cpu_budget)
        cpu = {"value": vps, "unit": "voxels/s", "cores": cores, "kind": "port",
               "sample": "realization 0, first %d of %d tiles (%.1f s), scaled by the tile "
                         "fraction" % (steps, ntiles, dt)}
    # working set: simulation grids (padded) and the soft maps (one per tile and variable)
    ovl = [math.ceil(o * t) for o, t in zip(W["overlap"], W["tilesize"])]
    ntl = [math.ceil(s / (t - o)) for s, t, o in zip(W["simsize"], W["tilesize"], ovl)]
    padvol = int(np.prod([n * (t - o) + o for n, t, o in zip(ntl, W["tilesize"], ovl)]))
    npos = int(np.prod([a - t + 1 for a, t in zip(W["ti"].shape, W["tilesize"])]))
    soft_bytes = len(W["soft"]) * int(np.prod(ntl)) * npos * 4
    line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian fields)",
            "config": {"workload": W["desc"], "global_batch": nreal * world,
                       "options": args.option,
                       "voxels_per_step": voxels * world,
                       "parallelism": "realization shards x%d" % world,
                       "l2": "working set > L2 (simulation grids %.0f MB%s)" % (
                           padvol * nreal * 4 / 1e6,
                           ", soft maps %.1f GB" % (soft_bytes / 1e9) if soft_bytes else ""),
                       "form": FORMS[args.form]},
            "roofline": roof, "dominant_kernel": dom, "kernels": kernel_share,
            "counters": counters,
            "cpu_baseline": cpu,
            "e2e": None if args.no_e2e else
                   {"value": e2e_value, "unit": "voxels/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e_max / e2e_steps,
                    "steps": e2e_steps},
            "clocks": clk, "gpu_launches": int(launches)}
    if args.form == "proposal":
        line["proposal"] = dict(lp_info or {}, **{"stats": lp_stats, "k": args.lp_k})
        line["plain"] = plain
        if plain:
            line["proposal"]["speedup_vs_plain"] = value / plain["value"]
        if dom in lp_kernels:
            line["roofline"] = proposal_roofline(dom, prof, lp_kernels, W, peaks, peak_kind,
                                                 lp_stats, args)
            line["dominant_kernel"] = dom
        elif dom == "graphcut":
            line["roofline"] = cut_roofline(prof, cut_nodes, peaks, peak_kind, W)
        # the proposal's own kernels, whichever dominates
        line["proposal"]["kernel_rooflines"] = {
            k: proposal_roofline(k, prof, lp_kernels, W, peaks, peak_kind, lp_stats, args)
            for k in ("lp.pick", "lp.scan") if k in prof}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg4", choices=["cfg4", "cfg3", "cfg2", "cfg1"],
                    help="cfg4 (default): the configuration the metric is quoted on")
    ap.add_argument("--form", default=None, choices=["plain", "proposal"],
                    help="plain full scan, or the learned proposal (default: the proposal for "
                         "the categorical configurations 3 and 4, plain otherwise)")
    ap.add_argument("--lp-k", type=int, default=8192,
                    help="shortlist length a call starts with (lp.k)")
    ap.add_argument("--lp-kmax", type=int, default=65536,
                    help="longest shortlist the recall monitor may raise it to (lp.kmax)")
    ap.add_argument("--lp-pairs", type=int, default=60000, help="training pairs to capture")
    ap.add_argument("--lp-save", default=None, help="save the trained encoder parameters (.npy)")
    ap.add_argument("--lp-load", default=None,
                    help="use saved encoder parameters instead of capturing and training")
    ap.add_argument("--lp-seeds", type=int, default=50)
    ap.add_argument("--lp-capture-steps", type=int, default=1500)
    ap.add_argument("--lp-capture-reals", type=int, default=2)
    ap.add_argument("--lp-train-steps", type=int, default=3000)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-plain", action="store_true", help="skip the full-scan comparison step")
    ap.add_argument("--nreal", type=int, default=0,
                    help="realizations per call (default: the workload's; for profiling captures)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer arm")
    ap.add_argument("--e2e-steps", type=int, default=3,
                    help="timed steps of the host-buffer arm (at most --steps)")
    ap.add_argument("--option", action="append", default=[],
                    help="library tuning knob name=value (iq_set_option), repeatable")
    args = ap.parse_args()
    dist, rank, world = dist_setup()
    W = workload(args.workload)
    if args.nreal:
        W["nreal"] = args.nreal  # smaller device footprint for profiling captures
        W["desc"] += " (nreal set to %d)" % args.nreal
    if args.form is None:
        args.form = "proposal" if args.workload in ("cfg3", "cfg4") else "plain"
    if args.impl == "reference":
        run_reference(args, W, dist, rank, world)
    else:
        run_ours(args, W, dist, rank, world)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
