"""Multi-GPU: independent replicas (one process per GPU, no data-path collective).

A DQMC chain does not shard -- slices are sequential and the proposals of a
slice depend on each other through G -- so N GPUs run N independent
ensembles.  The only cross-rank operations are the barrier around the timed
region and the max-over-ranks of the elapsed time.
"""
from __future__ import annotations


def chain_seeds(rank: int, chains_per_rank: int, base: int = 2):
    """Disjoint chain seeds of a rank (rank r owns base + r*B ... base + (r+1)*B - 1)."""
    return [base + rank * chains_per_rank + j for j in range(chains_per_rank)]


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """Largest value of x over all ranks (identity without a process group)."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world: int, elapsed_max: float) -> float:
    """Whole-job throughput: units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / elapsed_max
