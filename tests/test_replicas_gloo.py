"""The N>1 bench path: independent replicas per rank, whole-job time = max over
ranks (world_size 2, gloo, CPU)."""
import os
import socket
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = bench.replica_seeds(rank, 3)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    total = bench.max_over_ranks(local_ms, dist, "cpu")
    out[rank] = (seeds, total, bench.aggregate_rate(3, world, 10, total))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    s0, t0, v0 = out[0]
    s1, t1, v1 = out[1]
    assert set(s0).isdisjoint(s1)          # every rank serves its own sessions
    assert t0 == t1 == 150.0               # max over ranks
    assert v0 == v1 == 3 * 2 * 10 / 0.150  # whole-job frames / slowest rank's time
