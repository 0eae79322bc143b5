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


# ---------------------------------------------------------------- online (P²) form

ON_GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "online_golden.json")))["cases"]


@pytest.mark.parametrize("full", [False, True], ids=["fixed-estimate-exit", "full-recurrence"])
@pytest.mark.parametrize("case", ON_GOLD, ids=[f"seed{c['case']['seed']}" for c in ON_GOLD])
def test_online_matches_reference(engine, case, full):
    """sgfim_transactionize_online reproduces the reference run_file's items
    and every window's P² edges bit for bit, with and without the early exit."""
    import hashlib
    c = case["case"]
    vals, anom = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
    items, labels, edges = engine.transactionize_online(vals, c["window"], c["stride"], c["n_bins"], anomaly=anom,
                                                        full_recurrence=full)
    assert items.tolist() == case["items"]
    head = case["edges_head"]
    assert [[[float(x).hex() for x in e] for e in w] for w in edges[:len(head)]] == head
    flat = np.ascontiguousarray(edges, dtype="<f8")
    assert hashlib.sha256(flat.tobytes()).hexdigest() == case["edges_sha256"]
    n_win = len(case["items"])
    assert labels.tolist() == [int(anom[w * c["stride"]:w * c["stride"] + c["window"]].max()) for w in range(n_win)]


@pytest.mark.parametrize("full", [False, True], ids=["fixed-estimate-exit", "full-recurrence"])
@pytest.mark.parametrize("shape", [(200_000, 21, 30, 15, 3), (100_000, 16, 64, 8, 6), (50_000, 5, 5, 1, 2)])
def test_online_large_matches_oracle(engine, shape, full):
    """Long streams against the C restatement: edges of every window bit for
    bit, items, labels; TX_LOAD makes the items the dataset."""
    import oracle
    n, S, window, stride, n_bins = shape
    vals, anom = datagen.sensor_stream(n, S, 31 + S, constant_cols=(1,))
    items, labels, edges = engine.transactionize_online(vals, window, stride, n_bins, anomaly=anom, load=True,
                                                        full_recurrence=full)
    w_edges, w_items, w_labels = oracle.online_bins(vals, window, stride, n_bins, anom)
    assert np.array_equal(edges.view(np.int64), w_edges.view(np.int64))
    assert np.array_equal(items, w_items) and np.array_equal(labels, w_labels)
    assert engine.info()["n_txn"] == len(items)
    assert np.array_equal(engine.item_counts(S * n_bins), np.bincount(items.ravel(), minlength=S * n_bins))


def test_online_edge_cases(engine):
    vals, _ = datagen.sensor_stream(20, 2, 5)
    items, labels, edges = engine.transactionize_online(vals, 30, 15, 3)     # no window fits
    assert items.shape == (0, 2) and labels.shape == (0,) and edges.shape[0] == 0
    items, labels, edges = engine.transactionize_online(np.zeros((0, 3)), 30, 15, 3)
    assert items.shape == (0, 3)
    const = np.full((500, 3), 2.5)                                            # zero spread: span = 1e-9
    items, _, edges = engine.transactionize_online(const, 10, 5, 3)
    w_edges, w_items, _ = __import__("oracle").online_bins(const, 10, 5, 3)
    assert np.array_equal(edges.view(np.int64), w_edges.view(np.int64)) and np.array_equal(items, w_items)
    bad = vals.copy()
    bad[3, 1] = np.nan
    with pytest.raises(SgfimError):
        engine.transactionize_online(np.vstack([bad] * 5), 10, 5, 3)
    for window, stride, n_bins in ((0, 1, 3), (5, 0, 3), (5, 1, 1), (5, 1, 65), (300, 1, 3)):
        with pytest.raises(SgfimError):
            engine.transactionize_online(np.ones((400, 2)), window, stride, n_bins)


def test_online_run_file_and_report(engine):
    """The reference-shaped host calls: run_file's [(win_idx, start, {col:
    bin})] and the online-vs-offline agreement report, against the oracles."""
    from oracle import online
    from sgfim import online as son
    cols = [f"s{i}" for i in range(8)]
    frames = []
    for seed in (40, 41, 42):
        vals, _ = datagen.sensor_stream(3000 + 500 * (seed - 40), 8, seed)
        frames.append({c: vals[:, i] for i, c in enumerate(cols)})
    res = son.run_file(engine, frames[0], cols, 30, 15)
    v0 = np.column_stack([frames[0][c] for c in cols])
    _, want, _ = online.online_items(v0, 30, 15, 3)
    assert [r[1] for r in res] == [15 * w for w in range(len(want))]
    assert [[r[2][c] for c in cols] for r in res] == [[int(x) - 3 * i for i, x in enumerate(row)] for row in want]
    report = son.online_vs_offline(engine, frames, cols, 30, 15)
    seg = {k: [] for k in range(5)}
    for f in frames:
        v = np.column_stack([f[c] for c in cols])
        _, on, _ = online.online_items(v, 30, 15, 3)
        off, _ = transact.window_items(v, transact.fit_bins(v, 3), 30, 15, None, 3)
        for w in range(len(on)):
            seg[min(4, w * 5 // len(on))].append(float(np.count_nonzero(on[w] == off[w])) / 8)
    assert report == {son.segment_key(i): {"files": 3, "windows": len(v), "item_agreement": round(float(np.mean(v)), 4)}
                      for i, v in seg.items()}


@pytest.mark.parametrize("lanes", [1, 3, 32, 0])
def test_online_chain_packing(engine, lanes):
    """Any number of estimator chains per warp gives the same bits: 300
    sensors x 4 estimators = 1,200 chains, partial last warp (full recurrence,
    so that every chain steps through the whole stream)."""
    import oracle
    vals, anom = datagen.sensor_stream(3_000, 300, 77, constant_cols=(0, 299))
    items, labels, edges = engine.transactionize_online(vals, 20, 7, 5, anomaly=anom, lanes=lanes,
                                                        full_recurrence=True)
    w_edges, w_items, w_labels = oracle.online_bins(vals, 20, 7, 5, anom)
    assert np.array_equal(edges.view(np.int64), w_edges.view(np.int64))
    assert np.array_equal(items, w_items) and np.array_equal(labels, w_labels)


@pytest.mark.parametrize("n_bins", [2, 4, 6])
def test_online_half_quantile_streams(engine, n_bins):
    """The estimator at q = 1/2 keeps stepping while no sample has fallen
    between its markers 1 and 3: streams that stay in the outer cells for a
    long stretch (and ones whose first samples tie) against the C restatement."""
    import oracle
    rng = np.random.default_rng(n_bins)
    cols = []
    # distinct first samples, then a long run in the outer cells, then noise
    head = [0.0, 1.0, 2.0, 3.0, 5.0]
    outer = np.where(np.arange(4000) % 2 == 0, 10.0, -10.0)
    cols.append(np.concatenate([head, outer, rng.normal(2.0, 2.0, 2000)]))
    # tied first samples (markers 1..3 equal), then outer run
    cols.append(np.concatenate([[0.0, 1.0, 1.0, 1.0, 5.0], outer, rng.normal(1.0, 1.0, 2000)]))
    # markers 1 and 2 tied, 3 above
    cols.append(np.concatenate([[0.0, 1.0, 1.0, 4.0, 5.0], outer, rng.normal(3.0, 1.0, 2000)]))
    # ordinary noise
    cols.append(rng.normal(0.0, 1.0, 6005))
    vals = np.column_stack(cols)
    for window, stride in ((30, 15), (3, 2), (7, 7)):
        for full in (False, True):
            items, _, edges = engine.transactionize_online(vals, window, stride, n_bins, full_recurrence=full)
            w_edges, w_items, _ = oracle.online_bins(vals, window, stride, n_bins)
            assert np.array_equal(edges.view(np.int64), w_edges.view(np.int64)), (window, stride, full)
            assert np.array_equal(items, w_items)
