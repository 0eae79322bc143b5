"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run with SGFIM_REFERENCE naming a checkout of the reference project:

    SGFIM_REFERENCE=<reference checkout> python tests/golden/make_golden.py

It imports the reference's own Python miners and adapter parsers
(code/pipeline/skab_spike.py:mine_mfi, code/pipeline/exp_e6_cpuvec.py:
mine_mfi_cpuvec and load_fimi_bitmap, code/pipeline/engine_adapter.py:
parse_tensorfim_results / parse_anyfim_results), runs them on seeded
synthetic inputs, and stores their outputs as JSON.  pandas, which those
modules import at the top but never call, is replaced by an empty stub; no
bytecode is written into the reference tree.  The inputs themselves are not
stored: each case records its generator call and the SHA-256 of the FIMI text
it produces, and the tests regenerate it.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300"))
REF = os.environ.get("SGFIM_REFERENCE")
if not REF or not os.path.isdir(REF):
    sys.exit("set SGFIM_REFERENCE to a checkout of the reference project")

import numpy as np  # noqa: E402

from sgfim import datagen  # noqa: E402


def ref_modules():
    sys.dont_write_bytecode = True
    sys.modules.setdefault("pandas", types.ModuleType("pandas"))
    sys.path.insert(0, os.path.join(REF, "code", "pipeline"))
    import engine_adapter
    import exp_e6_cpuvec
    import skab_spike
    return skab_spike, exp_e6_cpuvec, engine_adapter


def fimi_text(rows, one_based=True):
    off = 1 if one_based else 0
    lines = []
    for r in rows:
        lines.append(" ".join(str(int(x) + off) for x in r))
    return "\n".join(lines) + "\n"


def sha(text):
    return hashlib.sha256(text.encode()).hexdigest()


def gen_rows(spec):
    kind = spec["kind"]
    if kind == "regime":
        rows = datagen.regime_txns(spec["n"], spec["sensors"], spec["bins"], spec["regimes"],
                                   spec["alpha"], seed=spec["seed"])
        return [list(map(int, r)) for r in rows]
    if kind == "literal":
        return [list(r) for r in spec["rows"]]
    raise ValueError(kind)


def canon(mfis):
    out = sorted(([sorted(int(x) for x in s), int(c)] for s, c in mfis), key=lambda t: (t[0], t[1]))
    return out


CASES = [
    # the config-0 workload: 20,000 txns, 8 sensors x 5 bins, 4 regimes, alpha 0.3, floor 200
    dict(name="mfi-small-seed0", gen=dict(kind="regime", n=20000, sensors=8, bins=5, regimes=4, alpha=0.3, seed=0),
         min_count=200),
    dict(name="mfi-small-seed1", gen=dict(kind="regime", n=20000, sensors=8, bins=5, regimes=4, alpha=0.3, seed=1),
         min_count=200),
    dict(name="mfi-small-seed2-sup5pct", gen=dict(kind="regime", n=20000, sensors=8, bins=5, regimes=4, alpha=0.3,
                                                  seed=2), min_sup=0.05),
    dict(name="mfi-small-seed3-mc150.7", gen=dict(kind="regime", n=20000, sensors=8, bins=5, regimes=4, alpha=0.3,
                                                  seed=3), min_count=150.7),
    # reduced anytime-2m shape (fewer sensors and rows) where mine_mfi stays under its node cap
    dict(name="anytime-shape-12x8", gen=dict(kind="regime", n=6000, sensors=12, bins=8, regimes=32, alpha=0.2,
                                             seed=11), min_sup=0.04),
    # windows of the sliding-window service shape (21 sensors x 6 bins, 8 regimes); at the
    # service's 2% floor mine_mfi exceeds its 200,000-node cap, so the golden floors are higher
    dict(name="window-21x6-L2000", gen=dict(kind="regime", n=2000, sensors=21, bins=6, regimes=8, alpha=0.3,
                                            seed=21), min_sup=0.08),
    dict(name="window-21x6-L512", gen=dict(kind="regime", n=512, sensors=21, bins=6, regimes=8, alpha=0.3,
                                           seed=22), min_sup=0.1),
    # edge cases
    dict(name="edge-empty-rows", gen=dict(kind="literal", rows=[[1, 2, 3], [], [1, 2], [], [2, 3], [1, 2, 3], []]),
         min_count=2),
    dict(name="edge-single-txn", gen=dict(kind="literal", rows=[[4, 7, 9]]), min_count=1),
    dict(name="edge-identical", gen=dict(kind="literal", rows=[[1, 5, 6]] * 5), min_count=5),
    dict(name="edge-threshold-above-all", gen=dict(kind="literal", rows=[[1, 2], [2, 3], [3, 1]]), min_count=3),
    dict(name="edge-ragged", gen=dict(kind="literal",
                                      rows=[[1], [1, 2, 3, 4, 5, 6, 7, 8, 9, 10], [2, 4, 6, 8, 10], [1, 3, 5, 7, 9],
                                            [1, 2, 3], [8, 9, 10], [1, 10], [5]]), min_count=2),
    dict(name="edge-min-count-zero", gen=dict(kind="literal", rows=[[1, 2], [2, 3], [1, 2, 3]]), min_count=0),
]


def main():
    spike, cpuvec, adapter = ref_modules()
    cases = []
    for c in CASES:
        rows = gen_rows(c["gen"])
        text = fimi_text(rows, one_based=False)
        kw = {"min_count": c["min_count"]} if "min_count" in c else {"min_sup": c["min_sup"]}
        mfis, n = spike.mine_mfi([tuple(r) for r in rows], **kw)
        rec = dict(name=c["name"], gen=c["gen"], fimi_sha256_zero_based=sha(text), n_txn=n,
                   mfis=canon(mfis), **kw)
        # the numpy CPU baseline on the same input, where it applies (1-based FIMI, relative floor)
        if "min_sup" in c:
            with tempfile.TemporaryDirectory() as td:
                p = os.path.join(td, "x.txt")
                open(p, "w").write(fimi_text(rows, one_based=True))
                bm, nt = cpuvec.load_fimi_bitmap(p)
                sets, _, _ = cpuvec.mine_mfi_cpuvec(bm, nt, c["min_sup"])
                rec["cpuvec_sets_one_based"] = sorted(sorted(int(x) + 1 for x in s) for s in sets)
        cases.append(rec)
        print(f"{c['name']}: {len(mfis)} MFIs (n={n})", flush=True)
    with open(os.path.join(HERE, "mfi_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, separators=(",", ":"))

    # adapter parsers on Results-format text (format fixtures)
    tf_text = (
        "==================================================================\n"
        "transSetFile: x.txt\ntransNum: 10\n"
        "computation_time(s): 0.5\ntotal_time(s): 0.75\n"
        "MFIsNumber: 3\n============================List of MFIs:=============================\n"
        "1th: 3 { 9 4 2 }   support: 0.5  frequency: 5\n"
        "2th: 1 { 7 }   support: 0.3  frequency: 3\n"
        "3th: 2 { 12 1 }   support: 0.2  frequency: 2\n"
        "==================================================================\n")
    af_text = (
        "=================================================================\n"
        "transNum: 10\nUptoStage: 2\npreprocessing_time(s): 0\n"
        "=================================================================\n"
        "runtimePerStage(s): 0.001, 0.002,\n\n"
        "frequencyThrePerStage: 9, 7,\nsupportThrePerStage: 0.9, 0.7,\n\n"
        "dimensionPerStage: 1, 2,\n\nMFIsNumPerStage: 1, 2,\nitemsNumPerStage: 1, 3,\n\n"
        "====================== 1th stage MFIs Number: 1 ======================\n"
        "1th: 1 { 4 }   support: 0.9  frequency: 9\n\nfrequencyThreshold: 9\n"
        "====================== 2th stage MFIs Number: 2 ======================\n"
        "1th: 2 { 7 4 }   support: 0.7  frequency: 7\n2th: 1 { 3 }   support: 0.7  frequency: 7\n\n"
        "frequencyThreshold: 7\n=================================================================\n")
    with tempfile.TemporaryDirectory() as td:
        p1, p2 = os.path.join(td, "tf.txt"), os.path.join(td, "af.txt")
        open(p1, "w").write(tf_text)
        open(p2, "w").write(af_text)
        tf = adapter.parse_tensorfim_results(p1)
        st, meta = adapter.parse_anyfim_results(p2)
    adapter_golden = {
        "tf_line": adapter.TF_LINE.pattern, "af_stage": adapter.AF_STAGE.pattern,
        "tf_comp": adapter.TF_COMP.pattern, "tf_tot": adapter.TF_TOT.pattern,
        "tf_text": tf_text, "af_text": af_text,
        "tf_parsed": sorted([sorted(k), v] for k, v in tf.items()),
        "af_parsed": {str(k): sorted([sorted(s), f] for s, f in v) for k, v in st.items()},
        "af_meta": meta,
        "cumulative": {str(k): sorted(sorted(s) for s in v) for k, v in adapter.cumulative_mfis(st).items()},
    }
    with open(os.path.join(HERE, "adapter_golden.json"), "w") as f:
        json.dump(adapter_golden, f, indent=1)
    print("adapter fixtures written")


if __name__ == "__main__":
    main()
