"""The N > 1 path of bench.py (independent replicas, one per rank) on the CPU
with the gloo backend, world size 2: barrier, max-over-ranks time, summed
units, and the reference arm printing from rank 0 only."""
import os
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _replica(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist()
    d.init("gloo")
    d.barrier()
    # rank r processed 10 * (r + 1) units in 1 + r seconds
    rate = bench.replica_rate(d, 10.0 * (rank + 1), 1.0 + rank)
    q.put((rank, d.max(float(rank)), d.sum(1.0), rate))
    d.barrier()
    d.pg.destroy_process_group()


def test_replicas_aggregate_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_replica, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, total, rate in out:
        assert mx == 1.0 and total == 2.0
        assert rate == pytest.approx((10.0 + 20.0) / 2.0)  # all units over the slowest rank's time


def test_reference_arm_prints_from_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
