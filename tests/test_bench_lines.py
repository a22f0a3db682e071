"""The bench's host-side arithmetic and the reference arm's JSON line (CPU only)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_proposal_roofline_counts_two_bit_codes():
    import bench
    W = bench.workload("cfg3")
    st = {"cols_shortlist": 100.0, "mean_shortlist": 8000.0}
    prof = {"lp.pick": (2000.0, 10, 0.0)}  # 2 s over 10 launches
    r = bench.proposal_roofline("lp.pick", prof, {}, W, {"hbm_gbs": 6000.0}, "measured", st,
                                None)
    K = 32 * 32 * 16 - 24 * 24 * 12  # interior mask of the config-3 tile
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(100 * 8000 * K * 0.25 / 2.0 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6000.0)


def test_cut_roofline_counts_nine_bytes_per_node():
    import bench
    W = bench.workload("cfg1")
    r = bench.cut_roofline({"graphcut": (500.0, 4, 0.0)}, (0.0, 4, 4096.0 * 4),
                           {"hbm_gbs": 7000.0}, "measured", W)
    assert r["achieved"] == pytest.approx(9 * 4096 * 4 / 0.5 / 1e9)
    assert r["kernel"] == "graphcut"


def test_reference_arm_line_on_config_1():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "cfg1", "--steps", "1", "--warmup", "0",
                          "--cpu-budget", "2"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
