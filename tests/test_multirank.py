"""The multi-rank path of bench.py on CPU (gloo, world size 2).

Ranks shard realizations by seed and share nothing on the data path; the only collectives
are the timing barrier and the max over ranks of the elapsed time."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    dist, r, w = bench.dist_setup()
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    bench.barrier(dist)
    m = bench.reduce_max(dist, 10.0 * rank + 1.0)
    seeds = [bench.step_seed(i, rank) for i in range(4)]
    out.put((rank, m, seeds))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_gloo_max_over_ranks_and_disjoint_seeds():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [m for _, m, _ in res] == [11.0, 11.0]  # both ranks see the slowest rank's time
    s0, s1 = set(res[0][2]), set(res[1][2])
    assert len(s0) == 4 and len(s1) == 4 and not (s0 & s1)  # realizations are sharded


def test_aggregate_rate_counts_every_rank():
    import bench
    # 2 ranks x 3 steps x 1000 voxels in 1.5 s (the slowest rank) -> 4000 voxels/s
    assert bench.aggregate_rate(1000, 3, 2, 1500.0) == pytest.approx(4000.0)


def test_reference_arm_two_ranks_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "cfg1", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-budget", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0
