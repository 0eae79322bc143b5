"""Anytime MFI mining on the anytime-2m workload with a coverage curve.

2,000,000 transactions, 80 sensors x 8 bins = 640 items, 32 regimes,
Dirichlet(0.2) bins (sgfim.datagen, seed 0).  The miner runs at a support
floor with wall-clock checkpoints; coverage(t) = |final MFIs emitted by t| /
|final MFIs| (the cumulative-pool-versus-truth measure of the reference's
anytime experiment, code/pipeline/exp_e4_anytime.py:138-152).  The final set
is checked by properties that do not depend on size: every support is
recounted by the batched support kernel and, on a seeded sample, by the CPU
oracle; no reported set contains another; no single-item extension of a
sample is frequent.

    python -m sgfim.anytime_run --floor 0.02 --checkpoints 1,2,5,10,30
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import datagen
from .engine import Engine

WORKLOAD = dict(n_txn=2_000_000, n_sensors=80, n_bins=8, n_regimes=32, alpha_bin=0.2)


def coverage_at(emit_times, checkpoints):
    t = np.sort(emit_times)
    n = max(len(t), 1)
    return {str(c): float(np.searchsorted(t, c, side="right") / n) for c in checkpoints}


def verify(eng, res, thr, d, sample=200, seed=0, bm=None):
    """Size-independent checks of a final MFI set (CSR arrays of the result)."""
    out = {}
    cp, ci, sup = res.ptr.astype(np.uint64), res.items.astype(np.uint32), res.support
    n = len(sup)
    out["supports_recount_equal"] = bool(np.array_equal(eng.support_batch(cp, ci), sup))
    # antichain: load the MFIs themselves as transactions; each MFI must be
    # contained in exactly one of them (itself)
    with Engine() as pool:
        pool.load_csr(cp, ci)
        contained = pool.support_batch(cp, ci)
    out["antichain"] = bool((contained == 1).all())
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(n, min(sample, n), replace=False)) if n else np.zeros(0, np.int64)
    ep, ei = [0], []
    for i in pick:
        s = ci[cp[i]:cp[i + 1]].tolist()
        ss = set(s)
        for e in range(d):
            if e not in ss:
                ei.extend(s + [e])
                ep.append(len(ei))
    if len(ep) > 1:
        ext = eng.support_batch(np.array(ep, np.uint64), np.array(ei, np.uint32))
        out["sample_maximal"] = bool((ext < thr).all())
    if bm is not None and len(pick):
        import oracle
        k = (cp[1:] - cp[:-1])[pick]
        sp = np.zeros(len(pick) + 1, np.uint64)
        sp[1:] = np.cumsum(k)
        si = np.concatenate([ci[cp[i]:cp[i + 1]] for i in pick])
        out["oracle_sample_supports_equal"] = bool(np.array_equal(oracle.support_batch(bm, sp, si), sup[pick]))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--floor", type=float, default=0.02)
    ap.add_argument("--n-txn", type=int, default=WORKLOAD["n_txn"])
    ap.add_argument("--checkpoints", default="1,2,5,10,30")
    ap.add_argument("--order", default="support")
    ap.add_argument("--time-limit", type=float, default=0.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-verify", action="store_true")
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    rows = datagen.regime_txns(a.n_txn, WORKLOAD["n_sensors"], WORKLOAD["n_bins"], WORKLOAD["n_regimes"],
                               WORKLOAD["alpha_bin"], seed=a.seed)
    t_gen = time.perf_counter() - t0
    cks = [float(x) for x in a.checkpoints.split(",") if x]
    eng = Engine()
    t0 = time.perf_counter()
    eng.load_rows(rows)
    t_load = time.perf_counter() - t0
    thr = max(1, int(np.ceil(a.floor * a.n_txn)))
    res, recs = eng.mine_anytime(thr, cks, order=a.order, time_limit_s=a.time_limit, materialize=False)
    # every final MFI carries its emission time, so coverage(t) needs no set comparison
    cov = coverage_at(res.emit_time_s, cks)
    curve = [{"t_s": r["t_s"], "elapsed_s": r["elapsed_s"], "emitted_candidates": r["n_emitted"],
              "coverage": cov[str(r["t_s"])], "nodes": r["nodes"]} for r in recs]
    report = {"workload": "anytime-2m", "n_txn": a.n_txn, "items": WORKLOAD["n_sensors"] * WORKLOAD["n_bins"],
              "floor": a.floor, "min_count": thr, "order": a.order, "mfis": len(res), "nodes": res.nodes,
              "waves": res.waves, "candidates": res.candidates, "kernel_launches": res.kernel_launches,
              "mine_s": res.elapsed_s, "load_s": t_load, "gen_s": t_gen, "phase_s": res.phase_s,
              "time_to": {f"{int(f * 100)}%": res.time_to_coverage(f) for f in (0.5, 0.9, 0.95, 1.0)},
              "checkpoints": curve}
    if not a.no_verify:
        import oracle
        rp, it = datagen.txns_to_csr(rows)
        bm, _ = oracle.build_bitmaps(rp, it, WORKLOAD["n_sensors"] * WORKLOAD["n_bins"])
        report["verify"] = verify(eng, res, thr, WORKLOAD["n_sensors"] * WORKLOAD["n_bins"], bm=bm)
    eng.close()
    print(json.dumps(report))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
