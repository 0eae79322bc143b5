"""The CPU oracle against outputs of the reference itself (tests/golden/).

mfi_golden.json holds mine_mfi (code/pipeline/skab_spike.py:84-135) and
mine_mfi_cpuvec (code/pipeline/exp_e6_cpuvec.py:59-107) outputs produced by
tests/golden/make_golden.py; the oracle must reproduce them exactly.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from sgfim import datagen

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mfi_golden.json")))["cases"]


def rows_of(case):
    g = case["gen"]
    if g["kind"] == "regime":
        r = datagen.regime_txns(g["n"], g["sensors"], g["bins"], g["regimes"], g["alpha"], seed=g["seed"])
        return [list(map(int, x)) for x in r]
    return [list(x) for x in g["rows"]]


def bitmaps_of(rows):
    d = max((x for r in rows for x in r), default=-1) + 1
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, max(d, 1))
    return bm


def canon(res):
    return sorted(([sorted(s), c] for s, c in res), key=lambda t: (t[0], t[1]))


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_generator_reproduces_golden_input(case):
    rows = rows_of(case)
    text = "\n".join(" ".join(str(x) for x in r) for r in rows) + "\n"
    assert hashlib.sha256(text.encode()).hexdigest() == case["fimi_sha256_zero_based"]


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_oracle_mine_mfi_matches_reference(case):
    rows = rows_of(case)
    bm = bitmaps_of(rows)
    kw = {"min_count": case["min_count"]} if "min_count" in case else {"min_sup": case["min_sup"]}
    res, _ = oracle.mine_mfi(bm, len(rows), **kw)
    assert canon(res) == case["mfis"]


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_oracle_fast_miner_matches_reference(case):
    rows = rows_of(case)
    bm = bitmaps_of(rows)
    kw = {"min_count": case["min_count"]} if "min_count" in case else {"min_sup": case["min_sup"]}
    thr = oracle.thresh_from(len(rows), **kw)
    res, _ = oracle.mine_fast(bm, len(rows), thr)
    assert canon(res) == case["mfis"]


@pytest.mark.parametrize("case", [c for c in GOLD if "cpuvec_sets_one_based" in c],
                         ids=[c["name"] for c in GOLD if "cpuvec_sets_one_based" in c])
def test_reference_cpu_baseline_agrees(case):
    """The numpy CPU baseline's MFI sets equal mine_mfi's (both reference outputs)."""
    ref = sorted(sorted(x + 1 for x in s) for s, _ in case["mfis"])
    assert sorted(case["cpuvec_sets_one_based"]) == ref


def test_node_cap_raises_like_reference():
    case = next(c for c in GOLD if c["name"] == "mfi-small-seed0")
    rows = rows_of(case)
    bm = bitmaps_of(rows)
    with pytest.raises(RuntimeError):
        oracle.mine_mfi(bm, len(rows), min_count=200, node_cap=100)


# ------------------------------------------------------------------ counting KATs
def test_support_and_cooccurrence_kat():
    # bmma_bench's correctness gate shape scaled down: N bits, d items, sparse seeded bits
    N, d = 4096, 24
    w32 = N // 32
    bits, _ = oracle.bmma_bench_bits(w32 * d, 0x9E3779B97F4A7C15)
    bm32 = bits.reshape(d, w32)
    bm = bm32.view(np.uint64).reshape(d, w32 // 2)
    dense = np.unpackbits(bm32.view(np.uint8), axis=1, bitorder="little").astype(np.int64)
    co = oracle.cooccurrence(bm)
    assert np.array_equal(co, dense @ dense.T)
    cp, ci = datagen.walk_candidates(300, d, 1, 8, seed=5)
    sup = oracle.support_batch(bm, cp, ci)
    for c in range(300):
        items = ci[cp[c]:cp[c + 1]]
        assert sup[c] == int(np.all(dense[items] == 1, axis=0).sum())


def test_build_bitmaps_counts():
    rows = [[0, 3], [3], [], [1, 2, 3], [0, 0, 3]]
    rp, it = datagen.txns_to_csr(rows)
    bm, cnt = oracle.build_bitmaps(rp, it, 4)
    assert cnt.tolist() == [2, 1, 1, 4]
    assert bm.shape == (4, 1)
    assert int(bm[3, 0]) == 0b11011


# ------------------------------------------------------------------ engine semantics
def _engine_characterisation(bm, n, thr, roots):
    """{M in MFI(thr) : max(M) in roots} -- the set the engines' DFS reports."""
    res, _ = oracle.mine_fast(bm, n, thr)
    rs = set(int(r) for r in roots)
    return {frozenset(s): c for s, c in res if max(s) in rs}


@pytest.mark.parametrize("seed,thr,nroots", [(1, 40, 5), (2, 25, 12), (3, 60, 40), (4, 30, 1)])
def test_engine_dfs_equals_root_restricted_mfi(seed, thr, nroots):
    rows = datagen.regime_txns(1500, 6, 5, 3, 0.4, seed=seed)
    rp, it = datagen.txns_to_csr(rows)
    bm, cnt = oracle.build_bitmaps(rp, it, 30)
    order = oracle.freq_order(cnt)
    roots = [int(x) for x in order[:nroots] if cnt[x] >= thr]
    got = {frozenset(s): c for s, c in oracle.mine_engine(bm, thr, np.array(roots, np.uint32))}
    assert got == _engine_characterisation(bm, len(rows), thr, roots)


def test_anyfim_stage_equals_mine_mfi_without_ties():
    """exp_e4_anytime.py:120-136: each stage pool equals mine_mfi at the stage's
    count threshold (the identity holds when the k-th count is not tied)."""
    rows = datagen.regime_txns(2000, 5, 4, 3, 0.5, seed=9)
    rows1 = [[x + 1 for x in r] for r in rows.tolist()]
    stages = oracle.anyfim_stages(rows1, 12)
    cnt = oracle.item_counts(rows1)
    srt = sorted(cnt.tolist(), reverse=True)
    rp, it = datagen.txns_to_csr(rows1)
    bm, _ = oracle.build_bitmaps(rp, it, len(cnt))
    checked = 0
    for k, pool in stages.items():
        if srt[k - 1] == srt[k]:
            continue
        ref, _ = oracle.mine_mfi(bm, len(rows1), min_count=srt[k - 1])
        assert pool == {frozenset(s): c for s, c in ref}
        checked += 1
    assert checked >= 8


def test_tensorfim_strict_root_rule():
    """kernel_bmma.cu:1199: an item whose count equals n*thr exactly is frequent
    but not a root, so MFIs whose highest id is that item are not reported."""
    rows = [[1, 2], [1, 2], [1, 3], [3], [2, 3], [1], [4], [4], [4], [4]]
    got = oracle.tensorfim_mfis(rows, 0.4)  # n*thr = 4: items 1 (4) and 4 (4) tie at the threshold
    assert got == {}
    got = oracle.tensorfim_mfis(rows, 0.35)  # thr 3.5 -> counts >= 4 frequent, roots count/n > .35
    assert got == {frozenset({1}): 4, frozenset({4}): 4}


TX_GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "transact_golden.json")))["cases"]


@pytest.mark.parametrize("case", TX_GOLD, ids=[f"seed{c['case']['seed']}" for c in TX_GOLD])
def test_transact_oracle_matches_reference(case):
    """The numpy restatement of fit_bins / window_transactions reproduces the
    reference's own outputs (edges bit for bit, items, labels)."""
    import hashlib
    from oracle import transact
    from sgfim import datagen
    c = case["case"]
    vals, anom = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
    assert hashlib.sha256(np.ascontiguousarray(vals, dtype="<f8").tobytes()).hexdigest() == case["values_sha256"]
    edges = transact.fit_bins(vals, c["n_bins"])
    assert [[float(x).hex() for x in e] for e in edges] == case["edges"]
    items, labels = transact.window_items(vals, edges, c["window"], c["stride"], anom, c["n_bins"])
    assert items.tolist() == case["items"] and labels.tolist() == case["labels"]


ON_GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "online_golden.json")))["cases"]


def _online_check(case, edges, items):
    import hashlib
    c = case["case"]
    assert items.tolist() == case["items"]
    assert [[[float(x).hex() for x in e] for e in w] for w in edges[:len(case["edges_head"])]] == case["edges_head"]
    flat = np.ascontiguousarray(edges, dtype="<f8").reshape(len(case["items"]), c["n_sensors"], c["n_bins"] + 1)
    assert hashlib.sha256(flat.tobytes()).hexdigest() == case["edges_sha256"]


@pytest.mark.parametrize("case", ON_GOLD, ids=[f"seed{c['case']['seed']}" for c in ON_GOLD])
def test_online_oracles_match_reference(case):
    """Both restatements of the online discretiser (pure Python, and C in
    liboracle.so) reproduce the reference run_file's items and every window's
    edges bit for bit."""
    import hashlib
    from oracle import online, oracle
    from sgfim import datagen
    c = case["case"]
    vals, anom = datagen.sensor_stream(c["n_rows"], c["n_sensors"], c["seed"], constant_cols=c["constant_cols"])
    assert hashlib.sha256(np.ascontiguousarray(vals, dtype="<f8").tobytes()).hexdigest() == case["values_sha256"]
    n_win = len(case["items"])
    assert case["starts"] == [w * c["stride"] for w in range(n_win)]
    e1, i1, l1 = online.online_items(vals, c["window"], c["stride"], c["n_bins"], anom)
    _online_check(case, e1, i1)
    e2, i2, l2 = oracle.online_bins(vals, c["window"], c["stride"], c["n_bins"], anom)
    _online_check(case, e2, i2)
    assert l1.tolist() == l2.tolist()


def test_planted_kat_generator_small():
    """batch_proto.cu:195-231 restated: patterns of 2..6 distinct sorted items,
    frequencies in [0.2%, 1.5%], every pattern's support near its frequency."""
    bm, pats, freq, minsup = oracle.planted_kat(1 << 18)
    assert bm.shape == (512, (1 << 18) // 64) and len(pats) == 80 and minsup == int((1 << 18) * 0.15 / 100.0)
    assert all(2 <= len(p) <= 6 and list(p) == sorted(set(p)) for p in pats)
    assert ((freq >= 0.002) & (freq <= 0.015)).all()
    cp = np.cumsum([0] + [len(p) for p in pats]).astype(np.uint64)
    ci = np.array([x for p in pats for x in p], np.uint32)
    sup = oracle.support_batch(bm, cp, ci)
    assert (sup >= (freq * (1 << 18) * 0.7).astype(np.int64)).all()
