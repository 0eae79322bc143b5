"""Golden fixtures of the online (streaming) discretiser, from the reference.

Run with SGFIM_REFERENCE naming a checkout of the reference project:

    SGFIM_REFERENCE=<reference checkout> python tests/golden/make_online_golden.py

It imports code/pipeline/online_discretize.py and calls its own ``run_file``
on seeded synthetic sensor streams (``sgfim.datagen.sensor_stream``).  pandas
is not installed here: the module's top-level import gets an empty stub, and
``run_file`` receives a minimal frame object that offers exactly what it uses
(``len(df)``, ``df[c].iloc[t]``, ``df[c].iloc[s:e].median()`` = numpy's
median, which is pandas' result on NaN-free data).  ``run_file`` builds its
binners with the default of three bins; the cases with other bin counts set
``OnlineBinner``'s default for the call.  The edges of every window are
recorded by wrapping ``OnlineBinner.edges`` (``run_file`` asks for them once
per window and sensor, in that order): the first windows' edges are stored as
hex floats, all of them as the SHA-256 of the little-endian float64 array
[windows, sensors, n_bins + 1].  The inputs are not stored: each case
records its generator call and the SHA-256 of the values, and the tests
regenerate them.
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


class _ILoc:
    def __init__(self, v):
        self.v = v

    def __getitem__(self, key):
        if isinstance(key, slice):
            return _Series(self.v[key])
        return self.v[key]


class _Series:
    def __init__(self, v):
        self.values = v

    @property
    def iloc(self):
        return _ILoc(self.values)

    def median(self):
        return float(np.median(self.values))


class _Frame:
    def __init__(self, cols):
        self.cols = cols

    def __getitem__(self, c):
        return _Series(self.cols[c])

    def __len__(self):
        return len(next(iter(self.cols.values())))


CASES = [
    dict(n_rows=1200, n_sensors=8, seed=0, constant_cols=[], window=30, stride=15, n_bins=3),
    dict(n_rows=997, n_sensors=8, seed=1, constant_cols=[5], window=30, stride=15, n_bins=3),
    dict(n_rows=3000, n_sensors=21, seed=2, constant_cols=[0, 20], window=16, stride=16, n_bins=6),
    dict(n_rows=300, n_sensors=4, seed=3, constant_cols=[], window=7, stride=3, n_bins=5),
    dict(n_rows=64, n_sensors=3, seed=4, constant_cols=[], window=1, stride=1, n_bins=2),
    dict(n_rows=40, n_sensors=3, seed=7, constant_cols=[1], window=4, stride=2, n_bins=3),   # estimates from < 5 samples
    dict(n_rows=20, n_sensors=2, seed=5, constant_cols=[], window=30, stride=15, n_bins=3),   # no window fits
    dict(n_rows=2000, n_sensors=6, seed=6, constant_cols=[], window=64, stride=100, n_bins=8),
    dict(n_rows=5000, n_sensors=8, seed=8, constant_cols=[], window=256, stride=7, n_bins=3),
]


HEAD = 6   # windows whose edges are stored in full; the rest are pinned by a SHA-256


def values_sha(v):
    return hashlib.sha256(np.ascontiguousarray(v, dtype="<f8").tobytes()).hexdigest()


def main():
    sys.dont_write_bytecode = True
    sys.modules.setdefault("pandas", types.ModuleType("pandas"))
    sys.path.insert(0, os.path.join(REF, "code", "pipeline"))
    import online_discretize as od
    orig_edges = od.OnlineBinner.edges
    orig_defaults = od.OnlineBinner.__init__.__defaults__
    out = []
    for c in CASES:
        vals, _ = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
        cols = [f"s{i}" for i in range(c["n_sensors"])]
        frame = _Frame({name: vals[:, i] for i, name in enumerate(cols)})
        seen = []

        def rec(self, min_gap=None):
            e = orig_edges(self, min_gap)
            seen.append([float(x).hex() for x in e])
            return e
        od.OnlineBinner.edges = rec
        od.OnlineBinner.__init__.__defaults__ = (c["n_bins"],)
        try:
            res = od.run_file(frame, cols, c["window"], c["stride"])
        finally:
            od.OnlineBinner.edges = orig_edges
            od.OnlineBinner.__init__.__defaults__ = orig_defaults
        items = [[i * c["n_bins"] + int(online[name]) for i, name in enumerate(cols)] for _, _, online in res]
        starts = [int(s) for _, s, _ in res]
        S = c["n_sensors"]
        edges = [seen[w * S:(w + 1) * S] for w in range(len(res))]
        assert len(seen) == len(res) * S
        flat = np.array([[[float.fromhex(x) for x in e] for e in w] for w in edges], dtype="<f8")
        out.append(dict(case=c, values_sha256=values_sha(vals), starts=starts, edges_head=edges[:HEAD],
                        edges_sha256=hashlib.sha256(flat.tobytes()).hexdigest(), items=items))
        print(f"case seed={c['seed']}: {len(items)} windows", flush=True)
    with open(os.path.join(HERE, "online_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_online_golden.py", "cases": out}, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
