"""The multi-GPU path of bench.py is replicas only (independent bias points per rank, no
data-path collective); its two host-side pieces, the per-rank bias split and the
max-over-ranks job time, run here as two gloo ranks on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pts = bench.rank_bias_points(4, rank, world)
    t = bench.max_over_ranks(1.0 + rank, dist)
    out.put((rank, pts, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_split_bias_points_and_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (r0, p0, t0), (r1, p1, t1) = res
    assert t0 == t1 == 2.0
    assert len(p0) == len(p1) == 4 and not set(p0) & set(p1)
    sys.path.insert(0, ROOT)
    import bench

    assert sorted(p0 + p1) == sorted(bench.bias_points(8))
