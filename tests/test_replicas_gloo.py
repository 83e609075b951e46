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


def _frames(seed, n=3, w=64, h=48):
    """Seeded CPU frames: a textured plane 1.2-1.8 m away, moving 2 mm per frame."""
    import numpy as np
    rng = np.random.default_rng(seed)
    a, b, z0 = rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(1200, 1800)
    yy, xx = np.mgrid[0:h, 0:w]
    tex = ((xx * 37 + yy * 11 + seed * 7) % 256).astype(np.uint8)
    out = []
    for k in range(n):
        d = (z0 + a * (xx - w / 2) + b * (yy - h / 2) - 2 * k).astype(np.uint16)
        out.append((d, np.stack([tex, tex[::-1], tex[:, ::-1]], axis=-1).copy()))
    return out


def _oracle_session(seed):
    """The CPU path (the oracle's System) on a replica's own frames: its final
    pose (16 values), then its map's block count, sdf sum and weight sum."""
    import numpy as np
    import oracle as O
    import libfusion_gb300 as L
    K = L.IntrinsicMatrix(64, 48, 52.5, 52.5, 31.5, 23.5)
    cfg = L.default_config(voxel_size=0.02, truncation=0.06, zmax_update=4.0, zmax_raycast=4.0,
                           num_buckets=1 << 14, num_blocks=1 << 12, bilateral=0)
    s = O.OracleSystem(O.config_from(cfg, threads=1), O.intrinsics_from(K))
    s.set_pose(np.eye(4))
    for d, c in _frames(seed):
        s.process(d, c)
    coords, sdf, w, _ = s.map_export()
    return np.concatenate([s.pose().reshape(16), [len(coords), float(sdf[w > 0].astype(np.float64).sum()),
                                                 float(w.astype(np.float64).sum())]])


def _worker_sessions(rank, world, port, out):
    for p in (ROOT, ROOT / "oracle"):
        sys.path.insert(0, str(p))
    import time
    import numpy as np
    import torch
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = bench.replica_seeds(rank, 2)
    dist.barrier()
    t = time.perf_counter()
    poses = [_oracle_session(s) for s in seeds]
    ms = (time.perf_counter() - t) * 1e3
    total = bench.max_over_ranks(ms, dist, "cpu")
    got = [torch.zeros(2, 19, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(got, torch.tensor(np.array(poses).reshape(2, 19)))
    out[rank] = (seeds, ms, total, [g.numpy() for g in got])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_run_their_own_sessions():
    """Each rank runs its own seeded sessions through the CPU path with no
    exchange on the data path; the ranks meet only for the timing (max over
    ranks) and to gather their results, which equal the same sessions run
    alone in this process."""
    import numpy as np
    for p in (ROOT, ROOT / "oracle"):
        sys.path.insert(0, str(p))
    import oracle as O
    O.build()
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker_sessions, args=(world, _free_port(), out), nprocs=world, start_method="spawn",
                       join=True)
    (s0, ms0, t0, g0), (s1, ms1, t1, g1) = out[0], out[1]
    assert set(s0).isdisjoint(s1)
    assert t0 == t1 == max(ms0, ms1)
    for r, seeds in ((0, s0), (1, s1)):
        for i, seed in enumerate(seeds):
            alone = _oracle_session(seed)
            assert np.array_equal(g0[r][i], alone) and np.array_equal(g1[r][i], alone)
    assert g0[0][0][16] > 0 and not np.array_equal(g0[0][0], g0[1][0])  # different sessions, different maps
