"""Online (streaming) discretisation on the GPU, shaped like the reference's
code/pipeline/online_discretize.py.

``run_file`` returns what the reference's ``run_file`` (:111-128) returns --
``[(win_idx, start, {column: bin})]`` -- with the P² estimators, edges and
window medians computed by ``sgfim_transactionize_online``; ``online_vs_offline``
is the experiment of the reference's ``main`` (:131-177): per file the online
items against the whole-file quantile items (``sgfim_transactionize``), the
per-window agreement averaged over five segments of window index.
"""
from __future__ import annotations

import numpy as np

from .engine import Engine

SEGMENTS = 5


def _values(frame, cols):
    if isinstance(frame, dict):
        return np.column_stack([np.asarray(frame[c], dtype=np.float64) for c in cols])
    v = np.asarray(frame, dtype=np.float64)
    if v.ndim != 2 or v.shape[1] != len(cols):
        raise ValueError("values must be [n_rows, len(cols)] or a dict of columns")
    return v


def run_file(eng: Engine, frame, cols, window=30, stride=15, n_bins=3):
    """online_discretize.py:111-128 -> [(win_idx, start, {col: bin})]; ``frame``
    is a dict of columns or a [n_rows, len(cols)] array."""
    v = _values(frame, cols)
    items, _, _ = eng.transactionize_online(v, window, stride, n_bins, with_edges=False)
    out = []
    for w in range(items.shape[0]):
        out.append((w, w * stride, {c: int(items[w, i] - i * n_bins) for i, c in enumerate(cols)}))
    return out


def segment_key(i):
    """The reference report's segment names (online_discretize.py:168-172)."""
    return f"{i * 20}-{(i + 1) * 20}%窗口"


def online_vs_offline(eng: Engine, frames, cols, window=30, stride=15):
    """online_discretize.py:150-172: for every file the per-window share of
    sensors whose online item equals the whole-file-quantile item, averaged
    per fifth of the window index."""
    seg = {k: [] for k in range(SEGMENTS)}
    for frame in frames:
        v = _values(frame, cols)
        on, _, _ = eng.transactionize_online(v, window, stride, 3, with_edges=False)
        if len(v) == 0:
            continue
        off, _, _ = eng.transactionize(v, window, stride, 3)
        n_win = on.shape[0]
        for w in range(n_win):
            k = min(SEGMENTS - 1, w * SEGMENTS // max(1, n_win))
            seg[k].append(float(np.count_nonzero(on[w] == off[w])) / len(cols))
    return {segment_key(i): {"files": len(frames), "windows": len(vals),
                             "item_agreement": round(float(np.mean(vals)), 4) if vals else None}
            for i, vals in seg.items()}
