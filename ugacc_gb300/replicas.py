"""Replica bookkeeping for runs over several GPUs (one process per GPU).

The solver path shards without a data-path collective: every rank runs its own
replica of the workload (bench), or its own share of a batch of independent
Hamiltonians (family workflow).  The only collectives are the barrier around a timed
region and the max of the per-rank times, which any torch.distributed backend
provides (NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations


def shard(n: int, rank: int, world: int) -> range:
    """Contiguous share of n independent items for this rank (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def allmax(x: float, dist=None, device=None) -> float:
    """Maximum of x over the ranks (x itself without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(work_per_rank: float, times: list[float] | float, world: int, dist=None, device=None) -> tuple:
    """(max time over ranks, units processed by all ranks / that time)."""
    t = allmax(times if isinstance(times, float) else max(times), dist, device)
    return t, world * work_per_rank / t
