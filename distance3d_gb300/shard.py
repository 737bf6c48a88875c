"""Pair-parallel sharding over ranks (one process per GPU).

Pairs are independent, so a batch is split into contiguous ranges, one per
rank; every rank holds the whole collider store, computes its range with no
exchange, and the results are concatenated in rank order.  The only
collective is the host-side gather of results (or of timings, as a max).
"""
import numpy as np


def shard_range(n, rank, world):
    """[lo, hi) of rank's contiguous share of n items (sizes differ by <= 1)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def concat_results(parts):
    """Concatenate per-rank result dicts (NumPy arrays, rank order)."""
    parts = [p for p in parts if p is not None]
    if not parts:
        return {}
    return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}


def gather_results(part, group=None):
    """All ranks: gather every rank's result dict; rank 0 gets the
    concatenation, the others None.  Uses torch.distributed (any backend)."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, part, group=group)
    return concat_results(parts) if dist.get_rank(group) == 0 else None


def max_over_ranks(value, group=None):
    """Largest `value` over all ranks (e.g. the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
