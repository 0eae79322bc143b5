"""Transaction split of batched support counting across ranks.

The reference splits a wave's counting over transactions inside one GPU
(split-k: each block sums a slice of the bitmap words and the partial counts
are added, code/engine_tensorfim/code/engine/src/kernel_bmma.cu:715-768).
Across GPUs the same split holds: rank r keeps only its slice of every
bitmap row (a contiguous range of 64-transaction words), counts the partial
support of every candidate over that slice, and one integer sum all-reduce of
the count vector gives the full supports -- the only exchange on the data
path.  Candidates are shared by every rank.

``txn_shard`` cuts the words into ranges that start on a 16-word (1,024
transaction) boundary, so every rank's slice is a whole number of the
counting kernels' chunks except the last; ``row_slice`` copies a rank's
columns out of a [d][n_words] bitmap matrix; ``allreduce_counts`` sums a
torch int32 count vector over the process group (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

import numpy as np

CHUNK_WORDS = 16


def txn_shard(n_words, rank, world):
    """Word range [w0, w1) of bitmap columns owned by ``rank`` of ``world``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    chunks = (n_words + CHUNK_WORDS - 1) // CHUNK_WORDS
    c0 = chunks * rank // world
    c1 = chunks * (rank + 1) // world
    return min(n_words, c0 * CHUNK_WORDS), min(n_words, c1 * CHUNK_WORDS)


def row_slice(bm, w0, w1):
    """Contiguous copy of columns [w0, w1) of a [d][n_words] uint64 matrix, padded to
    an even width (the device entry points want 16-byte aligned rows)."""
    width = w1 - w0
    out = np.zeros((bm.shape[0], width + (width & 1)), np.uint64)
    out[:, :width] = bm[:, w0:w1]
    return out


def allreduce_counts(counts, dist):
    """Sum a torch int32 count vector over the default process group in place."""
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(counts, op=dist.ReduceOp.SUM)
    return counts
