"""The N > 1 path of bench.py on CPU (gloo, world size 2): replicas take
disjoint origin windows of reset(1800) at every step (weak scaling, no
data-path collective), the job time is the maximum over ranks, and the
reference arm runs on rank 0 only."""
import os
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    wins = [bench.step_window(s, rank) for s in range(9)]
    gathered = [None] * world
    dist.all_gather_object(gathered, wins)
    slowest = bench.max_over_ranks(1.0 + rank, world)
    rc_ref = None
    if rank != 0:
        # the reference arm returns at once on every rank but 0
        class A:
            gpus, steps, warmup = world, 1, 0
        rc_ref = bench.run_reference(A())
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, gathered, slowest, rc_ref))


def test_two_ranks_disjoint_windows_and_max_time():
    world, port = 2, 29517
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    gathered = res[0][1]
    for s in range(9):
        starts = [gathered[r][s] for r in range(world)]
        assert len(set(starts)) == world            # no two ranks on the same window
        assert all(0 <= x <= 1600 and x % 200 == 0 for x in starts)
    for r in range(world):
        assert sorted(gathered[r]) == list(range(0, 1800, 200))  # each rank covers reset(1800)
    assert all(r[2] == float(world) for r in res)  # max over ranks of 1, 2
    assert res[1][3] == 0
