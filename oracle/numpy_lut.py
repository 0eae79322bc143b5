"""The reference's numpy support counting, restated for batched candidates.

TEST INFRASTRUCTURE: used by tests and bench.py's CPU baseline only.

code/pipeline/exp_e6_cpuvec.py keeps each item's transactions as a byte-packed
bitmap (np.packbits, :46-56), counts with a 256-entry popcount table
(POP, :43) and gets a node's extension supports as
POP[sub & node_bm].sum(axis=1) (:86).  Here the same arithmetic runs per
candidate: the byte view of the candidate's first row, ANDed with the byte
views of its other rows, summed through the table.  The byte order inside a
word does not change a popcount, so the uint64 bitmaps are used as they are.
"""
from __future__ import annotations

import numpy as np

POP = np.array([bin(i).count("1") for i in range(256)], dtype=np.int32)   # exp_e6_cpuvec.py:43


def supports(bm, cand_ptr, cand_items):
    """Support of each CSR candidate over [d][n_words] uint64 bitmaps (one thread)."""
    b8 = np.ascontiguousarray(bm, dtype=np.uint64).view(np.uint8)
    n_txn_bits = b8.shape[1] * 8
    n = len(cand_ptr) - 1
    out = np.zeros(n, np.uint32)
    for c in range(n):
        items = cand_items[int(cand_ptr[c]):int(cand_ptr[c + 1])]
        if len(items) == 0:
            out[c] = n_txn_bits
            continue
        node = b8[int(items[0])]
        for e in items[1:]:
            node = node & b8[int(e)]
        out[c] = int(POP[node].sum())
    return out
