"""Launch-shape autotuner for one workload on one context.

The library's tuning knobs (`iq_set_option`: cut threads per CTA, rounds between global
relabels, tiles per level chunk, realization streams) change how the work is cut into launches,
never which tiles or patterns are drawn, so the best setting depends only on the workload's
shape and the GPU. `autotune` times `iqsim` on a bounded sample of the caller's own workload
(the first `sample_steps` tiles of every realization, option `sim.max_steps`) and descends one
knob at a time, keeping the fastest value of each; the chosen values are left set on the
context.
"""
import time

# the library's defaults (include/iqgpu.h) and the candidate values tried for each knob
DEFAULTS = {
    "graphcut.threads": 512,
    "graphcut.gr_period": 32,
    "sim.level_chunk": 64,
    "sim.streams": 1,
}
CANDIDATES = {
    "graphcut.threads": (256, 512, 1024),
    "graphcut.gr_period": (16, 32, 48),
    "sim.level_chunk": (16, 64, 256),
    "sim.streams": (1, 2),
}


def coordinate_descent(measure, knobs=None, start=None, sweeps=1):
    """Minimise `measure(settings) -> seconds` one knob at a time.

    knobs: {name: candidate values}; start: the initial settings (defaults to DEFAULTS). Each
    sweep tries every candidate of every knob with the others held at their current best and
    keeps a value only when it is strictly faster. Returns (best settings, best time, the list
    of (settings, time) measured)."""
    knobs = dict(CANDIDATES if knobs is None else knobs)
    best = dict(DEFAULTS if start is None else start)
    for k in knobs:
        best.setdefault(k, knobs[k][0])
    history = []
    cache = {}

    def timed(s):
        key = tuple(sorted(s.items()))
        if key not in cache:
            cache[key] = float(measure(dict(s)))
            history.append((dict(s), cache[key]))
        return cache[key]

    best_t = timed(best)
    for _ in range(max(1, int(sweeps))):
        changed = False
        for name, values in knobs.items():
            for v in values:
                if v == best[name]:
                    continue
                trial = dict(best)
                trial[name] = v
                t = timed(trial)
                if t < best_t:
                    best, best_t, changed = trial, t, True
        if not changed:
            break
    return best, best_t, history


def autotune(ctx, trainimg, tilesize, simsize=None, *, knobs=None, sample_steps=200,
             repeats=2, sweeps=1, **iqsim_kwargs):
    """Tune `ctx`'s knobs for `iqsim(trainimg, tilesize, simsize, **iqsim_kwargs)`.

    Each setting is timed as the fastest of `repeats` calls (after one untimed call that
    warms the context's buffers), each simulating the first `sample_steps` tiles of every
    realization. The best settings are applied to `ctx` and `sim.max_steps` is restored to
    -1 (all tiles). Returns (settings, seconds per sampled call, history)."""
    from .api import iqsim

    kw = dict(iqsim_kwargs)
    kw["ctx"] = ctx

    def apply(s):
        for name, v in s.items():
            ctx.set_option(name, int(v))

    def measure(s):
        apply(s)
        iqsim(trainimg, tilesize, simsize, **kw)  # warm: buffers sized for this setting
        t = float("inf")
        for _ in range(max(1, int(repeats))):
            t0 = time.perf_counter()
            iqsim(trainimg, tilesize, simsize, **kw)
            t = min(t, time.perf_counter() - t0)
        return t

    ctx.set_option("sim.max_steps", int(sample_steps))
    try:
        best, best_t, history = coordinate_descent(measure, knobs, sweeps=sweeps)
    finally:
        ctx.set_option("sim.max_steps", -1)
    apply(best)
    return best, best_t, history
