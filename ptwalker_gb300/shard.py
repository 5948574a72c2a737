"""Walker and query sharding across processes (one process per GPU).

Walkers are independent and every draw depends on the global walker id, so
a run split over ranks equals the single-process run bit for bit once the
per-rank count vectors are summed (one all-reduce, the path's only exchange
step).  Per-vertex starts use the global id modulo n, so a weak-scaling
shard [r*W, (r+1)*W) again starts one walker per vertex.
"""
import numpy as np


def weak_range(rank, world, walkers_per_rank):
    """Rank r runs global walker ids [r * W, (r + 1) * W)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return rank * walkers_per_rank, walkers_per_rank


def strong_range(rank, world, total):
    """Contiguous near-equal split of [0, total) over `world` ranks."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def query_shard(n_queries, rank, world):
    """Indices of the queries rank `rank` runs (round robin, so uneven
    budgets spread over ranks)."""
    return np.arange(rank, n_queries, world, dtype=np.int64)


def sum_counts(counts, group=None):
    """Sums an integer count tensor over all ranks in place (torch.distributed)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(counts, op=dist.ReduceOp.SUM, group=group)
    return counts
