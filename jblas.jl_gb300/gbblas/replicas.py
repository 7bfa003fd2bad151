"""Replica runs across ranks: every rank computes its own independent products (GEMM shards
by output tiles or by problems, with no data exchange), and the job is timed by its slowest
rank.  Used by bench.py under torchrun (NCCL) and tested with gloo on CPU."""
import torch
import torch.distributed as dist


def job_time_and_throughput(ms_local, work_local, device=None):
    """(max step time over ranks in ms, whole-job throughput = sum of work / max time).

    work_local is the amount of work (e.g. flops) this rank did in one step; with no
    process group the local values are returned."""
    if not (dist.is_available() and dist.is_initialized()):
        return ms_local, work_local / (ms_local * 1e-3)
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([ms_local], dtype=torch.float64, device=dev)
    w = torch.tensor([work_local], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    ms = float(t.item())
    return ms, float(w.item()) / (ms * 1e-3)


def shard_rows(M, rank, world, align=256):
    """Row range [r0, r1) of C owned by `rank` when M rows are split in tile-aligned blocks."""
    tiles = (M + align - 1) // align
    per, extra = divmod(tiles, world)
    t0 = rank * per + min(rank, extra)
    t1 = t0 + per + (1 if rank < extra else 0)
    return min(M, t0 * align), min(M, t1 * align)


def shard_problems(sizes, rank, world):
    """Indices of the grouped problems owned by `rank`: greedy flop balance, largest first."""
    order = sorted(range(len(sizes)), key=lambda i: -2.0 * sizes[i][0] * sizes[i][1] * sizes[i][2])
    load = [0.0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda j: load[j])
        owner[i] = r
        load[r] += 2.0 * sizes[i][0] * sizes[i][1] * sizes[i][2]
    return [i for i in range(len(sizes)) if owner[i] == rank]
