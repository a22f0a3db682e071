"""The launch-shape autotuner: its search on CPU with a synthetic cost, and on the GPU the
tuned context still gives the realizations of the default one (the knobs only change how the
work is cut into launches)."""
import numpy as np
import pytest

from oracle import iqsim_oracle as O


def _cost(s):
    # separable cost with its minimum at threads 256, gr_period 48, level_chunk 64, streams 1
    return (abs(s["graphcut.threads"] - 256) / 256 + abs(s["graphcut.gr_period"] - 48) / 16 +
            abs(s["sim.level_chunk"] - 64) / 64 + (s["sim.streams"] - 1) + 1.0)


def test_coordinate_descent_finds_the_separable_minimum(iq):
    from iqgpu.autotune import DEFAULTS, coordinate_descent
    best, t, hist = coordinate_descent(_cost)
    assert best == {"graphcut.threads": 256, "graphcut.gr_period": 48, "sim.level_chunk": 64,
                    "sim.streams": 1}
    assert t == pytest.approx(1.0)
    assert hist[0][0] == DEFAULTS  # the defaults are measured first
    # every setting is measured once
    keys = [tuple(sorted(s.items())) for s, _ in hist]
    assert len(keys) == len(set(keys))


def test_coordinate_descent_keeps_defaults_on_ties(iq):
    from iqgpu.autotune import CANDIDATES, DEFAULTS, coordinate_descent
    best, _, hist = coordinate_descent(lambda s: 1.0)
    assert best == DEFAULTS
    assert len(hist) == 1 + sum(len(v) - 1 for v in CANDIDATES.values())


def test_coordinate_descent_custom_knobs_and_sweeps(iq):
    from iqgpu.autotune import coordinate_descent
    # an interaction: the best gr_period depends on the thread count, so a second sweep helps
    def cost(s):
        return abs(s["graphcut.gr_period"] - s["graphcut.threads"] // 16) / 16 + \
            (1024 - s["graphcut.threads"]) / 128
    knobs = {"graphcut.gr_period": (16, 32, 64), "graphcut.threads": (256, 512, 1024)}
    best1, t1, _ = coordinate_descent(cost, knobs, start={"graphcut.gr_period": 16,
                                                         "graphcut.threads": 256}, sweeps=1)
    best2, t2, _ = coordinate_descent(cost, knobs, start={"graphcut.gr_period": 16,
                                                         "graphcut.threads": 256}, sweeps=3)
    # one sweep moves the threads to 1024 only after gr_period was tried; the second sweep
    # then moves gr_period to the matching 64
    assert best1 == {"graphcut.gr_period": 16, "graphcut.threads": 1024} and t1 == 3
    assert best2 == {"graphcut.gr_period": 64, "graphcut.threads": 1024} and t2 == 0


@pytest.mark.gpu
def test_autotune_on_a_small_workload(iq):
    rng = np.random.default_rng(50)
    ti = rng.integers(0, 3, (24, 22, 10)).astype(np.float32)
    kw = dict(overlap=(0.25, 0.25, 0.25), nreal=3, rng=4)
    ctx = iq.Context(0)
    try:
        knobs = {"graphcut.threads": (256, 512), "sim.level_chunk": (4, 64), "sim.streams": (1, 2)}
        best, t, hist = iq.autotune(ctx, ti, (8, 8, 4), (30, 28, 10), knobs=knobs,
                                    sample_steps=6, repeats=1, **kw)
        assert set(best) >= set(knobs) and t > 0 and len(hist) >= 4
        for k, vals in knobs.items():
            assert best[k] in vals
        # the tuned context simulates every tile again and matches the oracle
        got = iq.iqsim(ti, (8, 8, 4), (30, 28, 10), ctx=ctx, **kw)
        ref = O.iqsim(ti, (8, 8, 4), (30, 28, 10), overlap=(0.25, 0.25, 0.25), nreal=3, seed=4)
        for x, y in zip(got, ref):
            assert np.array_equal(np.asarray(x, float), np.asarray(y, float))
    finally:
        ctx.close()
