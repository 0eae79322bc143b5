"""GPU transactionisation (sgfim_transactionize) against the reference's own
fit_bins / window_transactions outputs (golden) and the numpy oracle."""
import json
import os

import numpy as np
import pytest

from oracle import transact
from sgfim import datagen
from sgfim.engine import SgfimError

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "transact_golden.json")))["cases"]


@pytest.mark.parametrize("case", GOLD, ids=[f"seed{c['case']['seed']}" for c in GOLD])
def test_transactionize_matches_reference(engine, case):
    c = case["case"]
    vals, anom = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
    items, labels, edges = engine.transactionize(vals, c["window"], c["stride"], c["n_bins"], anomaly=anom)
    assert [[float(x).hex() for x in e] for e in edges] == case["edges"]
    assert items.tolist() == case["items"] and labels.tolist() == case["labels"]


def test_transactionize_large_matches_oracle_and_loads(engine):
    vals, anom = datagen.sensor_stream(200_000, 21, 9, constant_cols=(7,))
    items, labels, edges = engine.transactionize(vals, 30, 15, 6, anomaly=anom, load=True)
    want_edges = transact.fit_bins(vals, 6)
    assert all(np.array_equal(a, b) for a, b in zip(edges, want_edges))
    w_items, w_labels = transact.window_items(vals, want_edges, 30, 15, anom, 6)
    assert np.array_equal(items, w_items) and np.array_equal(labels, w_labels)
    info = engine.info()
    assert info["n_txn"] == len(items)
    counts = np.bincount(items.ravel(), minlength=126)
    assert np.array_equal(engine.item_counts(126), counts)


def test_transactionize_rejects_bad_input(engine):
    vals, _ = datagen.sensor_stream(100, 3, 0)
    vals[50, 1] = np.nan
    with pytest.raises(SgfimError):
        engine.transactionize(vals, 10, 5, 3)
    with pytest.raises(SgfimError):
        engine.transactionize(np.ones((400, 2)), 300, 5, 3)    # window > 256


def test_stream_to_windows_pipeline(engine):
    """Sensor stream -> transactions on the GPU -> device ring -> batched window
    mining: every window equals the oracle run on the oracle's own
    transactionisation of the same stream."""
    import oracle
    from sgfim.service import Ring
    vals, anom = datagen.sensor_stream(60_000, 21, 21, constant_cols=(4,))
    items, labels, edges = engine.transactionize(vals, 30, 15, 6, anomaly=anom)
    w_items, _ = transact.window_items(vals, transact.fit_bins(vals, 6), 30, 15, anom, 6)
    assert np.array_equal(items, w_items)
    rp, it = datagen.txns_to_csr(items)
    ring = Ring(126, 1 << 13)
    try:
        ring.append(rp, it)
        n = len(items)
        starts, lens = [0, 100, n - 3000, n - 500], [n, 2500, 3000, 500]
        thrs = [max(1, int(np.ceil(0.03 * L))) for L in lens]
        res = ring.mine_windows(engine, starts, lens, thrs)
        for w, (s, L, t) in enumerate(zip(starts, lens, thrs)):
            srp, sit = datagen.txns_to_csr(w_items[s:s + L])
            bm, _ = oracle.build_bitmaps(srp, sit, 126)
            ref, _ = oracle.mine_fast(bm, L, t)
            assert res.as_dict(w) == {frozenset(x): c for x, c in ref}, w
    finally:
        ring.close()
