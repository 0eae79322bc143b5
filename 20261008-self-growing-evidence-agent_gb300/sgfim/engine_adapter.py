"""Drop-in counterpart of the reference's engine adapter.

Mirrors code/pipeline/engine_adapter.py function by function (same names,
arguments, return shapes and error behaviour):

    write_fimi               engine_adapter.py:37-56
    load_items_map           :59-60
    decode_itemset           :63-68
    run_tensorfim            :70-100   (runs the sgfim_tensorfim CLI shim)
    parse_tensorfim_results  :103-111
    run_anyfim               :115-131  (runs the sgfim_anytime CLI shim)
    parse_anyfim_results     :134-166
    cumulative_mfis          :169-177
    support_confidence_lift  :181-191

The CLI shims keep the reference's process contract: ``<exe> <fimi> <arg>``,
the result file written next to the dataset as ``<fimi>-<thr:.6f>=Results.txt``
or ``<fimi>-<stages>-stages=Results.txt``, and ``computation_time(s):`` /
``total_time(s):`` lines on stdout.  ``engine`` may be 'baseline', 'bmma' or
'gb300'; all three run the GB300 engine.
"""
from __future__ import annotations

import json
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "_lib")
TENSORFIM_EXE = os.path.join(LIBDIR, "sgfim_tensorfim")
ANYFIM_EXE = os.path.join(LIBDIR, "sgfim_anytime")

# Results.txt record: "Nth: k { i1 i2 ... } support: s frequency: f"
TF_LINE = re.compile(r"^\d+th:\s+\d+\s+\{\s*([^}]*)\}\s+support:\s+\S+\s+frequency:\s+(\d+)")
TF_COMP = re.compile(r"computation_time\(s\):\s*([\d.eE+-]+)")
TF_TOT = re.compile(r"total_time\(s\):\s*([\d.eE+-]+)")
AF_STAGE = re.compile(r"^=+ (\d+)th stage MFIs Number: (\d+) =+")

_AF_META_KEYS = (("runtimePerStage(s):", float), ("supportThrePerStage:", float),
                 ("frequencyThrePerStage:", float), ("MFIsNumPerStage:", int), ("itemsNumPerStage:", int),
                 ("dimensionPerStage:", int), ("preprocessing_time(s):", float))


def write_fimi(txns, fimi_path, items_map_path=None):
    """txns: iterable of iterables of item strings.  Items are numbered from 1
    in order of first appearance; each line holds the sorted distinct ids.
    Returns {item_str: int_id}; the map is also saved as JSON when a path is given."""
    mapping = {}
    lines = []
    for txn in txns:
        ids = []
        for it in txn:
            if it not in mapping:
                mapping[it] = len(mapping) + 1
            ids.append(mapping[it])
        lines.append(" ".join(map(str, sorted(set(ids)))))
    with open(fimi_path, "w", encoding="utf-8") as f:
        f.write("\n".join(lines) + "\n")
    if items_map_path:
        with open(items_map_path, "w", encoding="utf-8") as f:
            json.dump(mapping, f, ensure_ascii=False, indent=1)
    return mapping


def load_items_map(path):
    with open(path, encoding="utf-8") as f:
        return json.load(f)


def decode_itemset(itemset_ids, inv_map):
    def _get(i):
        if i in inv_map:
            return inv_map[i]
        return inv_map[str(i)]
    return frozenset(_get(i) for i in itemset_ids)


def run_tensorfim(engine, fimi_path, rel_thr, reps=1, timeout=1800):
    """Returns {'ok', 'mfis': {frozenset: freq}, 'comp_times', 'tot_times'}; the
    result file is removed before every repetition."""
    if engine not in ("baseline", "bmma", "gb300"):
        raise ValueError(f"unknown engine {engine!r}")
    rp = f"{fimi_path}-{rel_thr:.6f}=Results.txt"
    comp, tot = [], []
    ok = True
    mfis = {}
    for _ in range(reps):
        if os.path.exists(rp):
            os.remove(rp)
        try:
            p = subprocess.run([TENSORFIM_EXE, fimi_path, str(rel_thr)], capture_output=True, timeout=timeout)
        except subprocess.TimeoutExpired:
            ok = False
            continue
        log = p.stdout.decode("utf-8", errors="replace") + p.stderr.decode("utf-8", errors="replace")
        m = TF_COMP.findall(log)
        if m:
            comp.append(float(m[-1]))
        m = TF_TOT.findall(log)
        if m:
            tot.append(float(m[-1]))
        if os.path.exists(rp):
            mfis = parse_tensorfim_results(rp)
        else:
            ok = False
    return {"ok": ok, "mfis": mfis, "comp_times": comp, "tot_times": tot}


def parse_tensorfim_results(path):
    """{frozenset(int item ids): frequency} of every record line."""
    out = {}
    with open(path, encoding="utf-8", errors="replace") as f:
        for ln in f:
            m = TF_LINE.match(ln.strip())
            if m:
                out[frozenset(int(x) for x in m.group(1).split())] = int(m.group(2))
    return out


def run_anyfim(fimi_path, upto_stage, timeout=3600):
    """Returns {'ok', 'stages': {k: [(frozenset, freq)]}, 'meta', 'results_path'}."""
    rp = f"{fimi_path}-{upto_stage}-stages=Results.txt"
    if os.path.exists(rp):
        os.remove(rp)
    try:
        p = subprocess.run([ANYFIM_EXE, fimi_path, str(upto_stage)], capture_output=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"ok": False, "stages": {}, "meta": {}, "results_path": rp}
    if not os.path.exists(rp):
        return {"ok": False, "stages": {}, "meta": {}, "log": p.stdout.decode("utf-8", errors="replace"),
                "results_path": rp}
    stages, meta = parse_anyfim_results(rp)
    return {"ok": True, "stages": stages, "meta": meta, "results_path": rp}


def parse_anyfim_results(path):
    """(stages, meta): stages[k] = [(frozenset(ids), frequency), ...]; meta holds the
    per-stage header arrays (runtimePerStage(s), supportThrePerStage, ...)."""
    stages = {}
    meta = {}
    cur = None
    with open(path, encoding="utf-8", errors="replace") as f:
        for ln in f:
            ln = ln.strip()
            m = AF_STAGE.match(ln)
            if m:
                cur = int(m.group(1))
                stages[cur] = []
                continue
            for key, cast in _AF_META_KEYS:
                if ln.startswith(key):
                    body = ln[len(key):].strip()
                    meta[key.rstrip(":")] = [cast(x.rstrip(",")) for x in body.split() if x.strip(",")]
            if cur is not None:
                m = TF_LINE.match(ln)
                if m:
                    stages[cur].append((frozenset(int(x) for x in m.group(1).split()), int(m.group(2))))
    return stages, meta


def cumulative_mfis(stages):
    """{k: set of every itemset seen in stages <= k}."""
    cum, seen = {}, set()
    for k in sorted(stages):
        for itemset, _ in stages[k]:
            seen.add(itemset)
        cum[k] = set(seen)
    return cum


def support_confidence_lift(itemset, txns, labels):
    """(sup, conf, lift) of an itemset over integer transactions with 0/1 labels;
    lift = P(X|1) / P(X)."""
    n = len(txns)
    cnt = sum(1 for t in txns if itemset <= set(t))
    pos = sum(1 for t, lab in zip(txns, labels) if lab == 1 and itemset <= set(t))
    npos = sum(1 for lab in labels if lab == 1)
    sup = cnt / n if n else 0.0
    conf = pos / npos if npos else 0.0
    lift = (pos / npos) / (cnt / n) if cnt and npos else 0.0
    return sup, conf, lift
