"""The multi-rank path of bench.py on CPU (gloo, world size 2).

Ranks are shards of one call (consecutive realization blocks, same seed) and share nothing
on the data path; the only collectives are the timing barrier and the max over ranks of the
elapsed time, plus the host gather of the realizations (imagequilting.jl_gb300/shard.py)."""
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
    firsts = [bench.step_real0(rank, 16) + r for r in range(16)]
    out.put((rank, m, firsts))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_gloo_max_over_ranks_and_disjoint_realizations():
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
    assert len(s0) == 16 and len(s1) == 16 and not (s0 & s1)  # realizations are sharded
    assert s0 | s1 == set(range(32))  # ... and together form one call


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


def _shard_worker(rank, world, port, out):
    """One rank of a sharded call: its block of realizations (the CPU oracle stands in for the
    library, which needs a GPU), then the host gather to every rank."""
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import numpy as np

    import bench
    from oracle import iqsim_oracle as O
    sys.path.insert(0, os.path.join(ROOT, "imagequilting.jl_gb300"))
    import shard
    dist, r, w = bench.dist_setup()
    ti = np.random.default_rng(5).integers(0, 3, (20, 18)).astype(np.float32)

    def oracle_sim(trainimg, tilesize, simsize, nreal, real0, **kw):
        return O.iqsim(trainimg, tilesize, simsize, nreal=nreal, real0=real0, seed=kw["rng"])

    real0, local = shard.iqsim_shard(oracle_sim, ti, (8, 8), (26, 24), nreal=5, rank=r,
                                     world=w, rng=11)
    allr = shard.gather_realizations(dist, real0, local)
    out.put((rank, real0, len(local), [a.tolist() for a in allr]))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_sharded_call_gathers_the_whole_call():
    import numpy as np
    import torch.multiprocessing as mp

    from oracle import iqsim_oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r0, n) for _, r0, n, _ in res] == [(0, 3), (3, 2)]
    ti = np.random.default_rng(5).integers(0, 3, (20, 18)).astype(np.float32)
    whole = O.iqsim(ti, (8, 8), (26, 24), nreal=5, seed=11)
    for _, _, _, allr in res:
        assert len(allr) == 5
        for a, b in zip(allr, whole):
            assert np.array_equal(np.array(a, np.float32), b)
    assert not all(np.array_equal(whole[0], x) for x in whole[1:])


def test_shard_ranges_cover_the_call():
    sys.path.insert(0, os.path.join(ROOT, "imagequilting.jl_gb300"))
    import shard
    for nreal in (0, 1, 5, 16, 33):
        for world in (1, 2, 3, 8):
            blocks = [shard.shard_range(nreal, r, world) for r in range(world)]
            assert sum(n for _, n in blocks) == nreal
            pos = 0
            for r0, n in blocks:
                assert r0 == pos
                pos += n
    with pytest.raises(ValueError):
        shard.shard_range(4, 2, 2)
