"""GPU miner parity: exact MFI sets and supports against the reference's own
outputs (golden fixtures) and against the CPU oracle at larger sizes."""
import json
import os

import numpy as np
import pytest

import oracle
from sgfim import datagen, results
from sgfim.engine import thresh_from

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mfi_golden.json")))["cases"]


def rows_of(case):
    g = case["gen"]
    if g["kind"] == "regime":
        r = datagen.regime_txns(g["n"], g["sensors"], g["bins"], g["regimes"], g["alpha"], seed=g["seed"])
        return [list(map(int, x)) for x in r]
    return [list(x) for x in g["rows"]]


def canon_dict(d):
    return sorted(([sorted(s), c] for s, c in d.items()), key=lambda t: (t[0], t[1]))


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_mine_matches_reference_golden(engine, case):
    rows = rows_of(case)
    engine.load_csr(*datagen.txns_to_csr(rows))
    kw = {"min_count": case["min_count"]} if "min_count" in case else {"min_sup": case["min_sup"]}
    res = engine.mine(thresh_from(len(rows), **kw))
    assert canon_dict(res.as_dict()) == case["mfis"]


@pytest.mark.parametrize("n,sensors,bins,regimes,alpha,frac,seed", [
    (100_000, 20, 8, 32, 0.2, 0.01, 0),     # anytime-2m shape, 20 sensors, 1% floor
    (50_000, 80, 8, 32, 0.2, 0.08, 1),      # the full 640-item anytime-2m shape, 8% floor
    (20_000, 21, 6, 8, 0.3, 0.03, 2),       # window shape
])
def test_mine_matches_oracle_larger(engine, n, sensors, bins, regimes, alpha, frac, seed):
    rows = datagen.regime_txns(n, sensors, bins, regimes, alpha, seed=seed)
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    thr = int(np.ceil(frac * n))
    got = engine.mine(thr).as_dict()
    bm, _ = oracle.build_bitmaps(rp, it, sensors * bins)
    ref, _ = oracle.mine_fast(bm, n, thr)
    assert got == {frozenset(s): c for s, c in ref}


def test_mine_result_properties(engine):
    """Size-independent checks on a 400,000-transaction, 640-item run: every
    reported set is frequent with the exact support, none contains another, and
    no single-item extension of a sample is frequent."""
    n = 400_000
    rows = datagen.regime_txns(n, 80, 8, 32, 0.2, seed=5)
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    thr = int(0.06 * n)
    res = engine.mine(thr)
    sets = res.sets()
    assert len(sets) > 100
    cp = np.zeros(len(sets) + 1, np.uint64)
    cp[1:] = np.cumsum([len(s) for s, _ in sets])
    ci = np.array([x for s, _ in sets for x in s], np.uint32)
    assert np.array_equal(engine.support_batch(cp, ci), np.array([c for _, c in sets], np.uint32))
    fs = [frozenset(s) for s, _ in sets]
    by_item = {}
    for i, s in enumerate(fs):
        for x in s:
            by_item.setdefault(x, set()).add(i)
    for i, s in enumerate(fs):
        sup = set.intersection(*(by_item[x] for x in s))
        assert sup == {i}, "a reported set is contained in another"
    rng = np.random.default_rng(0)
    sample = rng.choice(len(sets), min(200, len(sets)), replace=False)
    ext_ptr, ext_items = [0], []
    for i in sample:
        s = list(sets[i][0])
        for e in range(640):
            if e not in s:
                ext_items.extend(s + [e])
                ext_ptr.append(len(ext_items))
    ext = engine.support_batch(np.array(ext_ptr, np.uint64), np.array(ext_items, np.uint32))
    assert (ext < thr).all()


def test_root_rules_match_engine_semantics(engine):
    rows = datagen.regime_txns(3000, 6, 5, 3, 0.4, seed=3)
    rows1 = [[x + 1 for x in r] for r in rows.tolist()]
    engine.load_csr(*datagen.txns_to_csr(rows1))
    cnt = oracle.item_counts(rows1)
    order = oracle.freq_order(cnt)
    for k in (1, 4, 9, 17, 25):
        thr = int(cnt[order[k - 1]])
        got = engine.mine(thr, roots=[int(x) for x in order[:k]]).as_dict()
        want = oracle.anyfim_stages(rows1, k)[k]
        assert got == want, k
    for rel in (0.05, 0.1, 0.2):
        thr = max(1, int(np.ceil(len(rows1) * rel)))
        root_min = int(np.floor(len(rows1) * rel))
        while root_min / len(rows1) <= rel:
            root_min += 1
        got = engine.mine(thr, root_min_count=root_min).as_dict()
        assert got == oracle.tensorfim_mfis(rows1, rel), rel


def test_anytime_checkpoints(engine):
    rows = datagen.regime_txns(60_000, 40, 8, 32, 0.2, seed=8)
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    thr = int(0.02 * 60_000)
    res, recs = engine.mine_anytime(thr, [0.0, 0.05, 0.2, 1e6])
    final = res.as_dict()
    assert len(recs) == 4
    counts = [r["n_emitted"] for r in recs]
    assert counts == sorted(counts)
    emitted = {frozenset(s): c for s, c in recs[-1]["sets"]}
    assert set(final) <= set(emitted)
    assert all(emitted[s] == c for s, c in final.items())
    assert res.emit_time_s.max() <= res.elapsed_s + 1e-6
    bm, _ = oracle.build_bitmaps(rp, it, 320)
    ref, _ = oracle.mine_fast(bm, 60_000, thr)
    assert final == {frozenset(s): c for s, c in ref}


def test_orders_give_identical_sets_and_traces(engine):
    """Extension orders change the tree and the emission order, never the final
    set; traces label the nodes on the path to every final MFI."""
    rows = datagen.regime_txns(40_000, 30, 8, 32, 0.2, seed=13)
    engine.load_rows(rows)
    thr = int(0.03 * 40_000)
    base = engine.mine(thr, record_trace=True)
    assert base.trace_features.shape[1] == 8 and len(base.trace_labels) == len(base.trace_features)
    assert 0 < base.trace_labels.mean() < 1
    desc = engine.mine(thr, order="support_desc")
    assert desc.as_dict() == base.as_dict()
    # a scorer with random weights still gives the exact set
    rng = np.random.default_rng(0)
    engine.load_scorer(rng.normal(0, .3, (128, 8)), np.zeros(128), rng.normal(0, .1, (128, 128)), np.zeros(128),
                       rng.normal(0, .1, 128), np.zeros(1))
    learned = engine.mine(thr, order="learned")
    assert learned.as_dict() == base.as_dict()


def test_cancel_from_checkpoint(engine):
    from sgfim.engine import SgfimError
    rows = datagen.regime_txns(30_000, 30, 8, 32, 0.2, seed=9)
    engine.load_rows(rows)
    with pytest.raises(SgfimError) as ei:
        engine.mine_anytime(int(0.02 * 30_000), [0.0], callback=lambda t, e, s: True)
    assert ei.value.code == -7


def test_cli_shims_results_files(tmp_path):
    """The shims, run as the pipeline runs the engines, write result files whose
    sets are the oracle's TensorFIM and AnyFIM answers."""
    rows = datagen.regime_txns(4000, 8, 5, 4, 0.3, seed=12)
    rows1 = [[x + 1 for x in r] for r in rows.tolist()]
    fimi = str(tmp_path / "d.txt")
    datagen.write_fimi_ids(fimi, rows, one_based=True)
    r = results.run_shim("tensorfim", fimi, 0.03)
    assert r is not None and r.computation_s is not None and r.total_s is not None
    assert r.sets == oracle.tensorfim_mfis(rows1, 0.03)
    a = results.run_shim("anyfim", fimi, 12)
    assert a is not None
    want = oracle.anyfim_stages(rows1, 12)
    assert {k: dict(v) for k, v in a.stages.items()} == want
    assert a.arrays["MFIsNumPerStage"] == [len(want[k]) for k in range(1, 13)]
    assert len(a.arrays["runtimePerStage(s)"]) == 12


@pytest.mark.parametrize("projection", [True, False])
@pytest.mark.parametrize("n,sensors,bins,regimes,alpha,frac,seed", [
    (100_000, 20, 8, 32, 0.2, 0.01, 0),
    (50_000, 80, 8, 32, 0.2, 0.08, 1),
    (20_000, 21, 6, 8, 0.3, 0.03, 2),
    (3_000, 6, 4, 3, 0.3, 0.05, 3),
])
def test_projected_root_subtrees_match_oracle(projection, n, sensors, bins, regimes, alpha, frac, seed):
    """Every root subtree searched on its root item's projected database (forced
    here at sizes that would not project by default) gives the oracle's set, in
    every frontier order and with few mask slots (head-row queries on the
    projection)."""
    from sgfim.engine import Engine
    rows = datagen.regime_txns(n, sensors, bins, regimes, alpha, seed=seed)
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, sensors * bins)
    thr = int(np.ceil(frac * n))
    ref, _ = oracle.mine_fast(bm, n, thr)
    want = {frozenset(s): c for s, c in ref}
    for budget, wave in ((0, 0), (1 << 20, 5)):
        with Engine(projection=projection, hbm_budget=budget, wave_nodes=wave) as eng:
            eng.load_csr(rp, it)
            for order in ("support", "support_desc"):
                assert eng.mine(thr, order=order).as_dict() == want, (budget, wave, order)


def test_projection_default_on_large_data_equals_whole_database():
    """At 400,000 x 640 the miner projects by default; the search on the whole
    database gives the same set.  (The number of nodes may differ: HUT tests a
    node against the candidates emitted before its wave, and projected waves
    group nodes differently.)"""
    from sgfim.engine import Engine
    rows = datagen.regime_txns(400_000, 80, 8, 32, 0.2, seed=5)
    thr = int(np.ceil(0.05 * len(rows)))
    out = {}
    for projection in (None, False):
        with Engine(projection=projection) as eng:
            eng.load_rows(rows)
            res = eng.mine(thr)
            out[projection] = res.as_dict()
    assert out[None] == out[False] and len(out[None]) > 1000


@pytest.mark.parametrize("wave_nodes,floor", [(1, 0.08), (7, 0.05), (64, 0.02), (0, 0.02)])
def test_mine_exact_under_mask_arena_pressure(wave_nodes, floor):
    """A 1 MiB budget leaves the miner ~100 tidset-mask slots, so most nodes
    run without a mask (head-row queries) and masks are rebuilt at every wave
    start; small waves stage many copies back to back.  Results must equal the
    oracle's on window-shaped data at several seeds."""
    from sgfim.engine import Engine
    eng = Engine(hbm_budget=1 << 20, wave_nodes=wave_nodes)
    try:
        for seed in range(3):
            n = 20_000 + 3_331 * seed
            rows = datagen.regime_txns(n, 21, 6, 8, 0.3, seed=40 + seed)
            rp, it = datagen.txns_to_csr(rows)
            eng.load_csr(rp, it)
            thr = int(np.ceil(floor * n))
            got = eng.mine(thr).as_dict()
            bm, _ = oracle.build_bitmaps(rp, it, 126)
            ref, _ = oracle.mine_fast(bm, n, thr)
            assert got == {frozenset(s): c for s, c in ref}, (wave_nodes, seed)
    finally:
        eng.close()
