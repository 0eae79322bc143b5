"""numpy restatement of the reference's sensor-stream transactionisation --
TEST INFRASTRUCTURE.

Follows code/pipeline/skab_spike.py:
  fit_bins             :38-52  per-sensor np.quantile at linspace(0, 1, n_bins+1),
                               np.unique, a constant column gets [e0-0.5, e0+0.5]
  bin_index            :55-58  searchsorted(edges, v, side="right") - 1, clamped
  window_transactions  :62-80  windows s = 0, stride, ... while s + window <= n;
                               per sensor the window median, one item per sensor;
                               the window's label is the max of the anomaly flags
Items are returned as dense ids ``sensor * n_bins + bin`` instead of the
reference's "name=bin" strings.  pandas' Series.median on NaN-free data is
numpy's median, which is what is used here.
"""
from __future__ import annotations

import numpy as np


def fit_bins(values, n_bins=3):
    """values: [n_rows, n_sensors] float64 -> list of per-sensor edge arrays."""
    values = np.asarray(values, dtype=np.float64)
    edges = []
    qs = np.linspace(0, 1, n_bins + 1)
    for c in range(values.shape[1]):
        e = np.quantile(values[:, c], qs)
        e = np.unique(e)
        if len(e) < 2:
            e = np.array([e[0] - 0.5, e[0] + 0.5])
        edges.append(e)
    return edges


def bin_index(value, edges):
    idx = np.searchsorted(edges, value, side="right") - 1
    return int(min(max(idx, 0), len(edges) - 2))


def window_items(values, edges, window=30, stride=15, anomaly=None, n_bins=3):
    """-> (items [n_windows, n_sensors] int64 dense ids, labels [n_windows])."""
    values = np.asarray(values, dtype=np.float64)
    n, s_cnt = values.shape
    items, labels = [], []
    for s in range(0, n - window + 1, stride):
        e = s + window
        row = []
        for c in range(s_cnt):
            med = float(np.median(values[s:e, c]))
            row.append(c * n_bins + bin_index(med, edges[c]))
        items.append(row)
        labels.append(int(np.max(anomaly[s:e])) if anomaly is not None else 0)
    items = np.array(items, dtype=np.int64).reshape(-1, s_cnt)
    return items, np.array(labels, dtype=np.int64)

