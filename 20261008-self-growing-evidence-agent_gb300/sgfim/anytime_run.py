"""Anytime MFI mining on the anytime-2m workload with a coverage curve.

2,000,000 transactions, 80 sensors x 8 bins = 640 items, 32 regimes,
Dirichlet(0.2) bins (sgfim.datagen, seed 0).  The miner runs at a support
floor with wall-clock checkpoints; coverage(t) = |final MFIs emitted by t| /
|final MFIs| (the cumulative-pool-versus-truth measure of the reference's
anytime experiment, code/pipeline/exp_e4_anytime.py:138-152).

    python -m sgfim.anytime_run --floor 0.02 --checkpoints 1,2,5,10,30
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib as L
from . import datagen
from .engine import Engine, SgfimError

WORKLOAD = dict(n_txn=2_000_000, n_sensors=80, n_bins=8, n_regimes=32, alpha_bin=0.2)
ITEMS = WORKLOAD["n_sensors"] * WORKLOAD["n_bins"]


def coverage_at(emit_times, checkpoints):
    t = np.sort(emit_times)
    n = max(len(t), 1)
    return {str(c): float(np.searchsorted(t, c, side="right") / n) for c in checkpoints}


def workload_rows(n_txn=WORKLOAD["n_txn"], seed=0):
    return datagen.regime_txns(n_txn, WORKLOAD["n_sensors"], WORKLOAD["n_bins"], WORKLOAD["n_regimes"],
                               WORKLOAD["alpha_bin"], seed=seed)


def run(eng, rows, floor, checkpoints=(1, 2, 5, 10, 30), order="support", time_limit_s=0.0, node_limit=0):
    """Load ``rows`` into ``eng``, mine anytime at ``floor`` (fraction of the
    transactions) and return (report, result)."""
    n_txn = len(rows)
    t0 = time.perf_counter()
    eng.load_rows(rows)
    t_load = time.perf_counter() - t0
    thr = max(1, int(np.ceil(floor * n_txn)))
    cks = [float(c) for c in checkpoints]
    recs = []
    try:
        res, _ = eng.mine_anytime(thr, cks, order=order, time_limit_s=time_limit_s, node_limit=node_limit,
                                  materialize=False, records=recs)
    except SgfimError as e:
        if e.code not in (L.ETIMEDOUT, L.ENOMEM):
            raise
        # a time or node limit ended the search: what was emitted by each checkpoint
        report = {"workload": "anytime-2m", "n_txn": n_txn, "items": ITEMS, "floor": floor, "min_count": thr,
                  "order": order, "complete": False, "stopped_by": "time limit" if e.code == L.ETIMEDOUT
                  else "node limit", "time_limit_s": time_limit_s, "node_limit": node_limit, "load_s": t_load,
                  "checkpoints": [{"t_s": r["t_s"], "elapsed_s": r["elapsed_s"],
                                   "emitted_candidates": r["n_emitted"], "nodes": r["nodes"]} for r in recs]}
        return report, None
    # every final MFI carries its emission time, so coverage(t) needs no set comparison
    cov = coverage_at(res.emit_time_s, cks)
    curve = [{"t_s": r["t_s"], "elapsed_s": r["elapsed_s"], "emitted_candidates": r["n_emitted"],
              "coverage": cov[str(r["t_s"])], "nodes": r["nodes"]} for r in recs]
    report = {"workload": "anytime-2m", "n_txn": n_txn, "items": ITEMS, "floor": floor, "min_count": thr,
              "order": order, "complete": True, "mfis": len(res), "nodes": res.nodes, "waves": res.waves, "candidates": res.candidates,
              "kernel_launches": res.kernel_launches, "mine_s": res.elapsed_s, "load_s": t_load,
              "phase_s": res.phase_s,
              "time_to": {f"{int(f * 100)}%": res.time_to_coverage(f) for f in (0.5, 0.9, 0.95, 1.0)},
              "checkpoints": curve}
    return report, res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--floor", type=float, default=0.02)
    ap.add_argument("--n-txn", type=int, default=WORKLOAD["n_txn"])
    ap.add_argument("--checkpoints", default="1,2,5,10,30")
    ap.add_argument("--order", default="support")
    ap.add_argument("--time-limit", type=float, default=0.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    rows = workload_rows(a.n_txn, a.seed)
    t_gen = time.perf_counter() - t0
    with Engine() as eng:
        report, _ = run(eng, rows, a.floor, [float(x) for x in a.checkpoints.split(",") if x], a.order, a.time_limit)
    report["gen_s"] = t_gen
    print(json.dumps(report))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
