"""Golden fixtures of the sensor-stream transactionisation, from the reference.

Run with SGFIM_REFERENCE naming a checkout of the reference project:

    SGFIM_REFERENCE=<reference checkout> python tests/golden/make_transact_golden.py

It imports code/pipeline/skab_spike.py and calls its own ``fit_bins`` and
``window_transactions`` on seeded synthetic sensor streams
(``sgfim.datagen.sensor_stream``).  pandas is not installed here: the module's
top-level import gets an empty stub, and the two functions receive a minimal
frame object that offers exactly what they use (``df[c].values``,
``df.iloc[s:e]``, ``block[c].median()`` = numpy's median, which is pandas'
result on NaN-free data, and ``block[c].max()``).  The inputs are not stored:
each case records its generator call and the SHA-256 of the values, and the
tests regenerate them.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300"))
REF = os.environ.get("SGFIM_REFERENCE")
if not REF or not os.path.isdir(REF):
    sys.exit("set SGFIM_REFERENCE to a checkout of the reference project")

import numpy as np  # noqa: E402

from sgfim import datagen  # noqa: E402


class _Series:
    def __init__(self, v):
        self.values = v

    def median(self):
        return float(np.median(self.values))

    def max(self):
        return self.values.max()


class _Frame:
    def __init__(self, cols):
        self.cols = cols

    def __getitem__(self, c):
        return _Series(self.cols[c])

    def __len__(self):
        return len(next(iter(self.cols.values())))

    @property
    def iloc(self):
        frame = self

        class _ILoc:
            def __getitem__(self, sl):
                return _Frame({k: v[sl] for k, v in frame.cols.items()})
        return _ILoc()


CASES = [
    dict(n_rows=1200, n_sensors=8, seed=0, constant_cols=[], window=30, stride=15, n_bins=3),
    dict(n_rows=997, n_sensors=8, seed=1, constant_cols=[5], window=30, stride=15, n_bins=3),
    dict(n_rows=5000, n_sensors=21, seed=2, constant_cols=[0, 20], window=16, stride=16, n_bins=6),
    dict(n_rows=300, n_sensors=4, seed=3, constant_cols=[], window=7, stride=3, n_bins=5),
    dict(n_rows=64, n_sensors=3, seed=4, constant_cols=[], window=1, stride=1, n_bins=2),
    dict(n_rows=20, n_sensors=2, seed=5, constant_cols=[], window=30, stride=15, n_bins=3),   # no window fits
    dict(n_rows=2000, n_sensors=6, seed=6, constant_cols=[], window=64, stride=100, n_bins=8),
]


def values_sha(v):
    return hashlib.sha256(np.ascontiguousarray(v, dtype="<f8").tobytes()).hexdigest()


def main():
    sys.dont_write_bytecode = True
    sys.modules.setdefault("pandas", types.ModuleType("pandas"))
    sys.path.insert(0, os.path.join(REF, "code", "pipeline"))
    import skab_spike as spike
    out = []
    for c in CASES:
        vals, anom = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
        cols = [f"s{i}" for i in range(c["n_sensors"])]
        frame = _Frame({**{name: vals[:, i] for i, name in enumerate(cols)}, "__anom__": anom})
        edges = spike.fit_bins(frame, cols, n_bins=c["n_bins"])
        _, txns, txn_anom = spike.window_transactions(frame, cols, edges, c["window"], c["stride"])
        name_to_id = {f"{name}={b}": i * c["n_bins"] + b for i, name in enumerate(cols) for b in range(c["n_bins"])}
        items = [[name_to_id[x] for x in t] for t in txns]
        out.append(dict(case=c, values_sha256=values_sha(vals),
                        edges=[[float(x).hex() for x in edges[n]] for n in cols],
                        items=items, labels=[int(x) for x in txn_anom]))
        print(f"case seed={c['seed']}: {len(items)} windows", flush=True)
    with open(os.path.join(HERE, "transact_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_transact_golden.py", "cases": out}, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
