"""Work partitioning for runs with one process per GPU.

Candidate supports are independent, so a multi-GPU run splits the candidate
list into contiguous ranges, one per rank, with no data-path exchange (weak
scaling: each rank owns the same number of candidates).  Every rank holds the
full bitmap matrix.
"""
from __future__ import annotations


def shard_range(n, rank, world):
    """[lo, hi) of the n units owned by ``rank`` out of ``world`` (contiguous,
    sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi
