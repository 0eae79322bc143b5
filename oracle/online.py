"""Pure-Python restatement of the reference's online (streaming) discretiser --
TEST INFRASTRUCTURE (small cases; ``liboracle.so``'s ``orc_online_bins`` is the
same arithmetic in C for large ones).

Follows code/pipeline/online_discretize.py:
  P2Quantile.__init__/_setup :25-36  five markers from the first five samples
                                     (sorted), positions [0, 1+2q, 1+4q, 3+2q, 4]
  P2Quantile.add             :38-66  cell k of the sample (the outer markers move
                                     out), every position +1, positions 1..k +1
                                     more, then markers 1, 2, 3 in turn move by
                                     (d + 1) * (q[i+1] - q[i-1]) / span when
                                     d >= 1, span > 1 and the moved value stays
                                     strictly between its neighbours
  P2Quantile.value           :68-71  the middle marker (the median of the
                                     samples while fewer than five arrived)
  OnlineBinner               :74-103 n_bins-1 estimators at i/n_bins; edges =
                                     sorted estimates, span = max(q[-1]-q[0],
                                     1e-9), min_gap = 0.05*span; with 3 bins a
                                     too-narrow inner pair is re-centred, else
                                     each edge is pushed up to its predecessor +
                                     min_gap; outer edges q[0]-span, q[-1]+span
  bin_index                  :106-108 searchsorted(edges, v, "right") - 1, clamped
  run_file                   :111-128 for each window (s = 0, stride, ... while
                                     s + window <= n) every row of the window is
                                     fed to every sensor's binner -- rows shared
                                     by overlapping windows are fed again -- and
                                     the window median is binned with the edges
                                     of that moment
Items are dense ids ``sensor * n_bins + bin``.  Python floats are IEEE doubles
and every operation below happens in the reference's order, so the results are
the reference's bit for bit.
"""
from __future__ import annotations

import numpy as np


class P2:
    """One quantile estimator (online_discretize.py:22-71)."""

    def __init__(self, q):
        self.q = q
        self.init = []
        self.n = None
        self.qv = None

    def add(self, x):
        if len(self.init) < 5:
            self.init.append(x)
            if len(self.init) == 5:
                self.qv = sorted(self.init)
                self.n = [0.0, 1 + 2 * self.q, 1 + 4 * self.q, 3 + 2 * self.q, 4.0]
            return
        qv, n = self.qv, self.n
        if x < qv[0]:
            qv[0] = x
            k = 0
        elif x < qv[1]:
            k = 0
        elif x < qv[2]:
            k = 1
        elif x < qv[3]:
            k = 2
        elif x <= qv[4]:
            k = 3
        else:
            qv[4] = x
            k = 3
        for i in range(5):
            n[i] = n[i] + 1
        for i in range(1, 4):
            if i <= k:
                n[i] = n[i] + 1
        for i in (1, 2, 3):
            d = n[i] - n[i - 1]
            span = n[i + 1] - n[i - 1]
            if d >= 1 and span > 1:
                qp = (d + 1) * (qv[i + 1] - qv[i - 1]) / span
                moved = qv[i] + qp
                if qv[i - 1] < moved < qv[i + 1]:
                    qv[i] = moved

    def value(self):
        if len(self.init) < 5:
            return float(np.median(self.init)) if self.init else 0.0
        return float(self.qv[2])


def binner_edges(values, n_bins):
    """Edges of one sensor's binner from its estimators' values (:87-103)."""
    q = sorted(values)
    span = max(q[-1] - q[0], 1e-9)
    min_gap = 0.05 * span
    if n_bins == 3:
        if q[1] - q[0] < min_gap:
            mid = (q[0] + q[1]) / 2
            q[0], q[1] = mid - min_gap / 2, mid + min_gap / 2
    else:
        for i in range(1, len(q)):
            if q[i] < q[i - 1] + min_gap:
                q[i] = q[i - 1] + min_gap
    return [q[0] - span] + q + [q[-1] + span]


def bin_index(value, edges):
    idx = int(np.searchsorted(edges, value, side="right") - 1)
    return min(max(idx, 0), len(edges) - 2)


def online_items(values, window=30, stride=15, n_bins=3, anomaly=None):
    """values [n_rows, n_sensors] -> (edges [n_win, S, n_bins+1], items [n_win, S]
    dense ids, labels [n_win]) as run_file produces them."""
    values = np.asarray(values, dtype=np.float64)
    n, S = values.shape
    est = [[P2(i / n_bins) for i in range(1, n_bins)] for _ in range(S)]
    cols = [[float(x) for x in values[:, c]] for c in range(S)]
    edges, items, labels = [], [], []
    for s in range(0, n - window + 1, stride):
        e = s + window
        for t in range(s, e):
            for c in range(S):
                x = cols[c][t]
                for p in est[c]:
                    p.add(x)
        w_edges, w_items = [], []
        for c in range(S):
            ed = binner_edges([p.value() for p in est[c]], n_bins)
            med = float(np.median(values[s:e, c]))
            w_edges.append(ed)
            w_items.append(c * n_bins + bin_index(med, ed))
        edges.append(w_edges)
        items.append(w_items)
        labels.append(int(np.max(anomaly[s:e])) if anomaly is not None else 0)
    n_win = len(items)
    return (np.array(edges, dtype=np.float64).reshape(n_win, S, n_bins + 1),
            np.array(items, dtype=np.int64).reshape(n_win, S),
            np.array(labels, dtype=np.int64))
