"""Multi-GPU as independent replicas.

The out-of-memory path has no exchange step: every rank holds its own engine
(its own copy of the graph's static region on its own GPU) and serves its own
slice of the queries.  The only cross-rank operations are a barrier before and
after the timed region and the maximum of the per-rank times, so the whole-job
rate is (queries on all ranks) / (slowest rank's time).  No collective touches
the data path.
"""
from __future__ import annotations

import os


def rank_info() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def slice_queries(queries: list, rank: int, world: int) -> list:
    """Round-robin share of the query list for one replica (weak scaling: the
    per-rank count is what each rank times)."""
    return list(queries[rank::world]) if world > 1 else list(queries)


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(seconds: float, world: int, device: str = "cuda") -> float:
    """Slowest rank's time (all ranks receive it)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, slowest_seconds: float) -> float:
    return units_per_rank * world / slowest_seconds
