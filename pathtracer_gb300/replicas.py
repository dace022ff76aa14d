"""Replicas on N GPUs (one process per GPU): how ranks divide the work and
combine their timings.  Pixels, samples and jobs are independent and the RNG
stream depends only on (pixel, sample index), so no data crosses ranks: each
rank renders its own share and only timings (max over ranks) and per-job
results (gathered to rank 0) are exchanged, over torch.distributed.
"""
from __future__ import annotations


def job_range(rank: int, world: int, n_total: int) -> range:
    """Job indices [start, stop) of `rank` when n_total jobs are split as
    evenly as possible over `world` ranks (contiguous blocks)."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad rank, world or job count")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def job_seeds(rank: int, jobs_per_rank: int, first: int = 0) -> range:
    """Generator seeds of a rank's replica of a per-rank job set (weak scaling:
    every rank gets the same number of distinct jobs)."""
    return range(first + rank * jobs_per_rank, first + (rank + 1) * jobs_per_rank)


def frame_base(rank: int, steps_total: int, dispatches: int, spf: int) -> int:
    """First sample index of a rank's replica of a progressive render: ranks
    draw disjoint sample ranges of the same image."""
    return rank * (steps_total + 8) * dispatches * spf


def max_over_ranks(values: list[float]) -> list[float]:
    """Element-wise maximum over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def gather_to_root(obj):
    """obj from every rank, in rank order, on rank 0 (None elsewhere)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def whole_job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Units of all ranks per second of the slowest rank (the reported value)."""
    return units_per_rank * world / seconds_max
