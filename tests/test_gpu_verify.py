"""sgfim_frequent_extensions against the oracle, and the checks of a mined set
that do not go through the miner's search (full maximality, greedy maximal
walks) on a 400,000-transaction instance of the 640-item anytime family."""
import numpy as np
import pytest

import oracle
from sgfim import datagen
from sgfim.engine import Engine
from sgfim.verify import check_mfi_set, greedy_walks

pytestmark = pytest.mark.gpu


def _oracle_extensions(bm, n_ids, sets, thr):
    out = np.zeros((len(sets), (n_ids + 63) // 64), np.uint64)
    for s, items in enumerate(sets):
        ext = [e for e in range(n_ids) if e not in set(items)]
        cp = np.arange(len(ext) + 1, dtype=np.uint64) * (len(items) + 1)
        ci = np.array([x for e in ext for x in list(items) + [e]], np.uint32)
        sup = oracle.support_batch(bm, cp, ci) if ext else np.zeros(0, np.uint32)
        for e, c in zip(ext, sup):
            if c >= max(1, thr):
                out[s, e >> 6] |= np.uint64(1) << np.uint64(e & 63)
    return out


@pytest.mark.parametrize("thr", [0, 1, 300, 2500])
def test_frequent_extensions_match_oracle(thr):
    rows = datagen.regime_txns(9_000, 10, 7, 4, 0.3, seed=21)   # 70 items, ids 0..69
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, 70)
    rng = np.random.default_rng(thr)
    sets = [[], [3], [3, 3], [69, 0], [200], [5, 200]]          # empty, duplicate, unknown id
    sets += [sorted(rng.choice(70, rng.integers(1, 6), replace=False).tolist()) for _ in range(60)]
    cp = np.zeros(len(sets) + 1, np.uint64)
    cp[1:] = np.cumsum([len(s) for s in sets])
    ci = np.array([x for s in sets for x in s], np.uint32)
    with Engine() as eng:
        eng.load_csr(rp, it)
        got = eng.frequent_extensions(cp, ci, thr)
    assert np.array_equal(got, _oracle_extensions(bm, 70, sets, thr))


def test_mfi_set_checks_on_400k_instance():
    rows = datagen.regime_txns(400_000, 80, 8, 32, 0.2, seed=3)
    thr = int(np.ceil(0.05 * len(rows)))
    with Engine() as eng:
        eng.load_rows(rows)
        res = eng.mine(thr)
        rep = check_mfi_set(eng, res, thr, walks=100_000, seed=1)
        assert len(res) > 1000
        assert rep["supports_recount_equal"] and rep["all_frequent"] and rep["antichain"]
        assert rep["maximal_all"] and rep["maximal_checked"] == len(res)
        assert rep["walks_all_found"] and rep["walks_distinct_sets"] > 100
