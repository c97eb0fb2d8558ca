"""The N > 1 path of bench.py on the CPU: replicas only (the stepper does not shard), so the only
cross-rank step is the max of the per-replica times; two gloo ranks in spawned processes."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.5 + rank, torch.device("cpu"))
    env = bench.dist_env()
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, env))


def test_two_replicas_report_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict()
    for _ in procs:
        rank, t, env = q.get(timeout=120)
        got[rank] = (t, env)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0][0] == got[1][0] == 2.5
    assert got[0][1] == (2, 0, 0) and got[1][1] == (2, 1, 1)


def test_replica_throughput_counts_every_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_gcups(2e9, 1.0, 1) == pytest.approx(2.0)
    assert bench.replica_gcups(2e9, 2.0, 4) == pytest.approx(4.0)
    assert bench.max_over_ranks(3.0, None) == 3.0  # no process group: the value itself


def test_reference_arm_prints_only_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
