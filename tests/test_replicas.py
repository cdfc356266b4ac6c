"""The multi-GPU path is replicas only (the Picard map of one ensemble does not
shard): each rank runs its own workload and bench.py reports the job time as
the max over ranks. This checks that aggregation with world_size 2 on gloo."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elapsed = 100.0 if rank == 0 else 250.0      # rank 1 is the slow replica
    job_ms, tmax = bench.aggregate(elapsed, steps=5, world=world)
    q.put((rank, job_ms, tmax))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
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
    for rank, job_ms, tmax in res:
        assert tmax == 250.0                       # max over ranks
        assert job_ms == pytest.approx(250.0 / (5 * 2))   # all ranks' steps / job time


def test_single_rank_aggregation():
    import bench
    job, tmax = bench.aggregate(120.0, steps=4, world=1)
    assert tmax == 120.0 and job == 30.0
