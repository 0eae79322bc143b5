"""The CPU oracle miner in both extension orders: the canonical one (each
node's extensions in ascending support) and the reference's plain order (one
global order of descending item support, kernel_bitmap.cu:276-283,
exp_e6_cpuvec.py:65-69).  The MFI set does not depend on the order -- it
equals the reference miner's restatement -- but the tree does: on the
anytime-2m family the plain order searches more nodes.  This is the sequential
counterpart of the GPU miner's extension orders (tests/test_gpu_mining.py runs
them against this oracle)."""
import numpy as np
import pytest

import oracle
from sgfim import datagen


def _sets(res):
    return {frozenset(s): c for s, c in res}


@pytest.mark.parametrize("n,sensors,bins,regimes,alpha,frac,seed", [
    (3_000, 6, 4, 3, 0.3, 0.05, 3),
    (8_000, 21, 6, 8, 0.3, 0.03, 2),
    (5_000, 10, 5, 4, 0.3, 0.02, 7),
])
def test_orders_equal_reference_miner(n, sensors, bins, regimes, alpha, frac, seed):
    rows = datagen.regime_txns(n, sensors, bins, regimes, alpha, seed=seed)
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, sensors * bins)
    thr = int(np.ceil(frac * n))
    asc, _ = oracle.mine_fast(bm, n, thr, order="support")
    desc, _ = oracle.mine_fast(bm, n, thr, order="support_desc")
    ref, _ = oracle.mine_mfi(bm, n, min_count=thr)
    assert _sets(asc) == _sets(desc) == _sets(ref)


def test_plain_order_searches_more_nodes_on_anytime_family():
    """20,000-transaction streams of the anytime-2m family (80 sensors x 8
    bins, 32 regimes) at a 6% floor: identical sets, and the plain order's tree
    is larger on every seed."""
    for seed in (5010, 5011, 5012):
        rows = datagen.regime_txns(20_000, 80, 8, 32, 0.2, seed=seed)
        rp, it = datagen.txns_to_csr(rows)
        bm, _ = oracle.build_bitmaps(rp, it, 640)
        thr = int(np.ceil(0.06 * 20_000))
        asc, n_asc = oracle.mine_fast(bm, 20_000, thr, order="support")
        desc, n_desc = oracle.mine_fast(bm, 20_000, thr, order="support_desc")
        assert _sets(asc) == _sets(desc)
        assert n_desc > n_asc, (seed, n_asc, n_desc)


def test_static_order_that_knows_the_answer_is_close_to_ascending():
    """A bound on what any one global order can gain: items ordered by how many
    final MFIs hold them (knowledge no search has up front) search within 10% of
    the canonical order's nodes (0.94-1.03x on these seeds), with the same set."""
    for seed in (5010, 5011, 5012):
        rows = datagen.regime_txns(20_000, 80, 8, 32, 0.2, seed=seed)
        rp, it = datagen.txns_to_csr(rows)
        bm, _ = oracle.build_bitmaps(rp, it, 640)
        thr = int(np.ceil(0.06 * 20_000))
        asc, n_asc = oracle.mine_fast(bm, 20_000, thr, order="support")
        held = np.zeros(640)
        for s, _ in asc:
            held[list(s)] += 1
        keyed, n_key = oracle.mine_fast(bm, 20_000, thr, order="key", key=held)
        assert _sets(keyed) == _sets(asc)
        assert 0.9 < n_key / n_asc < 1.1, (seed, n_asc, n_key)
