"""Multi-rank (replica) logic on CPU with gloo, world size 2: job time is the slowest rank's,
throughput sums every rank's work; row and problem shards cover everything exactly once."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from gbblas import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = 10.0 + 5.0 * rank            # rank 1 is slower
    work_local = 1e12 * (rank + 1)
    ms, thr = replicas.job_time_and_throughput(ms_local, work_local)
    out[rank] = (ms, thr)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_job_time_and_throughput():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        ms, thr = out[r]
        assert ms == 15.0
        assert thr == pytest.approx(3e12 / 15e-3)


def test_no_group_returns_local_values():
    ms, thr = replicas.job_time_and_throughput(4.0, 8e9)
    assert ms == 4.0 and thr == pytest.approx(2e12)


@pytest.mark.parametrize("M,world", [(8192, 2), (8192, 3), (1000, 4), (256, 8)])
def test_row_shards_cover_once(M, world):
    seen = []
    for r in range(world):
        r0, r1 = replicas.shard_rows(M, r, world)
        assert r0 <= r1 and (r0 % 256 == 0 or r0 == M)
        seen.extend(range(r0, r1))
    assert seen == list(range(M))


def test_problem_shards_balanced():
    from gbblas import workloads
    sizes = [tuple(int(x) for x in row) for row in workloads.grouped_sizes(4096)]
    world = 4
    parts = [replicas.shard_problems(sizes, r, world) for r in range(world)]
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    loads = [sum(2.0 * sizes[i][0] * sizes[i][1] * sizes[i][2] for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.02
