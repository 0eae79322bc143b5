"""Learned extension ordering: traces -> training -> held-out evaluation.

The order of each search node's frequent extensions shapes the tree: child
H u {f_i} gets the tail f_{i+1..}, so the extensions placed first carry the
largest tails, and HUT/FHUT prune later children against what the earlier
ones found.  Three orders, every final MFI set identical:

* plain (``support_desc``): the reference's order, one global order of
  descending item support (kernel_bitmap.cu:276-283, exp_e6_cpuvec.py:65-69);
* canonical (``support``): ascending support in the node's context;
* learned: descending score of the scoring MLP, which predicts P(the child's
  subtree emits a final MFI) from the extension's features.

The committed scorer (sgfim/data/scorer_weights.npz) was trained by the
project's own kernels on traces of the scorer-free miner (canonical order) on
200 seeded 20,000-transaction streams at a 6% floor:

    python -m sgfim.learned_order --train-seeds 200 --n-txn 20000 --floor 0.06 \
        --eval-seeds 20 --eval-n-txn 2000000 --eval-floor 0.03 \
        --save-weights sgfim/data/scorer_weights.npz --out learned.json

Workload family: the anytime-2m generator (80 sensors x 8 bins = 640 items,
one item per sensor per transaction, 32 latent regimes, Dirichlet(0.2) bin
probabilities), with a per-stream seed.  Every run's final MFI set is
compared with the plain run's.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import datagen
from .engine import Engine
from .mlp import IN_DIM, Trainer

FAMILY = dict(n_sensors=80, n_bins=8, n_regimes=32, alpha_bin=0.2)
COVERAGE = (0.5, 0.9, 0.95)
# Orders are compared at 8,192 search nodes per wave, every order alike: the
# engine's default wave (32,768) finishes the smaller 3% streams in a handful
# of waves, and a wave's candidates all come out at its end, so the time to a
# coverage level would measure the wave grid rather than the order.  Node
# counts do not depend on the wave size.
EVAL_WAVE_NODES = 8192


def stream_rows(seed, n_txn):
    return datagen.regime_txns(n_txn, FAMILY["n_sensors"], FAMILY["n_bins"], FAMILY["n_regimes"],
                               FAMILY["alpha_bin"], seed=seed)


def collect_traces(eng, seeds, n_txn, floor, order="support"):
    X, Y, stats = [], [], []
    for s in seeds:
        eng.load_rows(stream_rows(s, n_txn))
        thr = max(1, int(np.ceil(floor * n_txn)))
        r = eng.mine(thr, order=order, record_trace=True)
        X.append(r.trace_features)
        Y.append(r.trace_labels.astype(np.float32))
        stats.append(dict(seed=s, mfis=len(r), nodes=r.nodes, trace=len(r.trace_labels),
                          pos=float(r.trace_labels.mean()) if len(r.trace_labels) else 0.0))
    return np.concatenate(X), np.concatenate(Y), stats


def coverage_times(res):
    """Seconds and search nodes until 50/90/95% of the final MFIs were emitted."""
    out = {f"t{int(f * 100)}": res.time_to_coverage(f) for f in COVERAGE}
    out.update({f"n{int(f * 100)}": res.nodes_to_coverage(f) for f in COVERAGE})
    return out


def evaluate(eng, seeds, n_txn, floor, reps=1):
    rows_out = []
    for s in seeds:
        eng.load_rows(stream_rows(s, n_txn))
        thr = max(1, int(np.ceil(floor * n_txn)))
        eng.mine(thr)  # warm the handle's buffers for this dataset size
        rec = {"seed": s}
        sets = {}
        for order in ("support_desc", "learned", "support"):
            best = None
            for _ in range(reps):
                r = eng.mine(thr, order=order)
                if best is None or r.elapsed_s < best.elapsed_s:
                    best = r
            sets[order] = best.as_dict()
            rec[order] = dict(total_s=best.elapsed_s, nodes=best.nodes, mfis=len(best), **coverage_times(best))
        rec["identical"] = sets["learned"] == sets["support_desc"] == sets["support"]
        rows_out.append(rec)
    return rows_out


def summarize(rows):
    """Learned / plain (support-descending) ratios, geomean and median over seeds,
    of the time and of the search nodes to each coverage level, and the same
    for the canonical order."""
    out = {"identical_all": all(r["identical"] for r in rows), "seeds": len(rows)}
    for order in ("learned", "support"):
        for key in ("t50", "t90", "t95", "n50", "n90", "n95", "total_s", "nodes"):
            ratio = [r[order][key] / max(r["support_desc"][key], 1e-9) for r in rows]
            pre = "" if order == "learned" else "canonical_"
            out[f"{pre}{key}_ratio_median"] = float(np.median(ratio))
            out[f"{pre}{key}_ratio_geomean"] = float(np.exp(np.mean(np.log(np.maximum(ratio, 1e-9)))))
    return out


def load_weights(eng, path):
    w = np.load(path)
    eng.load_scorer(w["W1"], w["b1"], w["W2"], w["b2"], w["w3"], w["b3"])


def evaluate_committed(weights_path, n_seeds=3, n_txn=2_000_000, floor=0.03, first_seed=5010):
    """Held-out streams of the anytime-2m family with committed scorer weights:
    coverage times and nodes of the learned, canonical and plain orders, final
    sets compared."""
    with Engine(wave_nodes=EVAL_WAVE_NODES) as eng:
        load_weights(eng, weights_path)
        rows = evaluate(eng, range(first_seed, first_seed + n_seeds), n_txn, floor)
    return {"n_txn": n_txn, "floor": floor, "summary": summarize(rows), "runs": rows}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--eval-seeds", type=int, default=20)
    ap.add_argument("--n-txn", type=int, default=20000)
    ap.add_argument("--floor", type=float, default=0.06)
    ap.add_argument("--eval-n-txn", type=int, default=0)
    ap.add_argument("--eval-floor", type=float, default=0.0)
    ap.add_argument("--save-weights", default="", help="write the trained scorer (.npz)")
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    eng = Engine(wave_nodes=EVAL_WAVE_NODES)
    t0 = time.time()
    X, Y, tstats = collect_traces(eng, range(1000, 1000 + a.train_seeds), a.n_txn, a.floor)
    t_trace = time.time() - t0
    tr = Trainer(eng, in_dim=IN_DIM)
    t0 = time.time()
    hist = tr.fit(X, Y, epochs=a.epochs, batch=4096, lr=2e-3)
    t_train = time.time() - t0
    import torch
    P = tr.forward(torch.from_numpy(X)).cpu().numpy()
    acc = float(((P > 0.5) == (Y > 0.5)).mean())
    w = tr.weights()
    eng.load_scorer(w["W1"], w["b1"], w["W2"], w["b2"], w["w3"], w["b3"])
    if a.save_weights:
        np.savez(a.save_weights, **w)
    ev_n = a.eval_n_txn or a.n_txn
    ev_floor = a.eval_floor or a.floor
    rows = evaluate(eng, range(5000, 5000 + a.eval_seeds), ev_n, ev_floor)
    summ = summarize(rows)
    report = {"train": {"seeds": a.train_seeds, "n_txn": a.n_txn, "floor": a.floor, "rows": int(len(Y)),
                        "positive_rate": float(Y.mean()), "trace_s": t_trace, "train_s": t_train,
                        "loss": hist, "train_accuracy": acc},
              "eval": {"seeds": a.eval_seeds, "n_txn": ev_n, "floor": ev_floor, "summary": summ, "runs": rows}}
    print(json.dumps({"train": report["train"], "summary": summ}))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
        np.savez(a.out.replace(".json", "_weights.npz"), **w)
    eng.close()
    return report


if __name__ == "__main__":
    main()
