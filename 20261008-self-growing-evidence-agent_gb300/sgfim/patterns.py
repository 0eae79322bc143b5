"""Pattern-fault scoring: how strongly each mined pattern concentrates in
anomalous transactions.

Reference: ``pattern_fault_analysis`` (code/pipeline/skab_spike.py:139-163),
which counts, for every MFI, the anomalous and the normal transactions that
contain it with Python set loops.  Here the two counts of every pattern are
supports on the GPU: the dataset is loaded with two label items appended
(one marks anomalous transactions, the other normal ones), and each pattern
becomes two candidates, pattern + label, in one ``sgfim_support_batch``
launch.  The arithmetic after the counts (supports as fractions, lift with
the 1e-9 guards, rounding, the (lift, sup_anom) descending order and the rank
column) follows the reference line by line.
"""
from __future__ import annotations

import numpy as np

from . import datagen


def label_dataset(rows, txn_anom):
    """CSR of ``rows`` with a label item appended to every transaction:
    ``max_id + 1`` for anomalous, ``max_id + 2`` for normal.  Returns
    (row_ptr, items, anom_item, norm_item)."""
    rp, it = datagen.txns_to_csr(rows)
    anom = np.asarray(txn_anom).astype(bool)
    if len(anom) != len(rp) - 1:
        raise ValueError("one label per transaction")
    top = int(it.max()) if len(it) else -1
    a_id, n_id = top + 1, top + 2
    lens = np.diff(rp).astype(np.int64) + 1
    rp2 = np.zeros(len(lens) + 1, np.uint64)
    np.cumsum(lens, out=rp2[1:])
    it2 = np.empty(int(rp2[-1]), np.uint32)
    # every row keeps its items and gets its label last
    pos = np.repeat(np.arange(len(lens)), lens - 1)
    dst = np.arange(len(it)) + pos            # shift item j of row r by r (one label per earlier row)
    it2[dst] = it
    it2[(rp2[1:] - 1).astype(np.int64)] = np.where(anom, a_id, n_id)
    return rp2, it2, a_id, n_id


def pattern_fault_counts(engine, patterns, rows, txn_anom):
    """(hit_anom, hit_norm) for every pattern: transactions containing it
    among the anomalous / normal ones.  Loads the labelled dataset into
    ``engine`` (replacing its dataset)."""
    rp, it, a_id, n_id = label_dataset(rows, txn_anom)
    engine.load_csr(rp, it)
    k = np.array([len(p) for p in patterns], np.int64)
    cp = np.zeros(2 * len(patterns) + 1, np.uint64)
    np.cumsum(np.repeat(k + 1, 2), out=cp[1:])
    ci = np.empty(int(cp[-1]), np.uint32)
    at = 0
    for p in patterns:
        for lab in (a_id, n_id):
            ci[at:at + len(p)] = sorted(p)
            ci[at + len(p)] = lab
            at += len(p) + 1
    sup = engine.support_batch(cp, ci).astype(np.int64)
    return sup[0::2], sup[1::2]


def pattern_fault_analysis(engine, mfis, rows, txn_anom):
    """The reference's table as a list of dicts, sorted as it sorts them, and
    the anomalous base rate.  ``mfis``: iterable of (pattern, count)."""
    anom = np.asarray(txn_anom).astype(int)
    n_anom_raw = int((anom == 1).sum())
    n_norm_raw = int((anom == 0).sum())
    n_anom = max(1, n_anom_raw)
    n_norm = max(1, n_norm_raw)
    base_rate = n_anom_raw / (n_anom_raw + n_norm_raw + 1e-9)
    pats = [tuple(p) for p, _ in mfis]
    if not pats:
        return [], base_rate
    ha, hn = pattern_fault_counts(engine, pats, rows, anom)
    out = []
    for p, a, b in zip(pats, ha, hn):
        sup_anom = int(a) / n_anom
        sup_norm = int(b) / n_norm
        lift = (sup_anom + 1e-9) / (sup_norm + 1e-9)
        out.append({"pattern": " ∧ ".join(str(x) for x in p), "len": len(p),
                    "sup_anom": round(sup_anom, 3), "sup_norm": round(sup_norm, 3), "lift": round(lift, 2)})
    # stable sort by (lift desc, sup_anom desc), then the 1-based rank
    order = sorted(range(len(out)), key=lambda i: (-out[i]["lift"], -out[i]["sup_anom"]))
    rows_out = [out[i] for i in order]
    for r, d in enumerate(rows_out):
        d["pct_of_anom_covered_rank"] = r + 1
    return rows_out, base_rate
