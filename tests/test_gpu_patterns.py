"""Pattern-fault scoring (pattern_fault_analysis, code/pipeline/skab_spike.py:139-163):
GPU label-item supports equal the reference's set-loop counts, and the table
equals a restatement of the reference's arithmetic and ordering."""
import numpy as np
import pytest

from sgfim import datagen
from sgfim.patterns import pattern_fault_analysis, pattern_fault_counts

pytestmark = pytest.mark.gpu


def _reference_table(mfis, transactions, txn_anom):
    """The reference function's arithmetic, with pandas' stable two-key sort
    written as a stable Python sort."""
    anom_idx = set(np.where(txn_anom == 1)[0])
    norm_idx = set(np.where(txn_anom == 0)[0])
    n_anom = max(1, len(anom_idx))
    n_norm = max(1, len(norm_idx))
    base_rate = len(anom_idx) / (len(anom_idx) + len(norm_idx) + 1e-9)
    rows = []
    for pattern, _ in mfis:
        pset = set(pattern)
        hit_anom = sum(1 for i in anom_idx if pset <= set(transactions[i]))
        hit_norm = sum(1 for i in norm_idx if pset <= set(transactions[i]))
        sup_anom = hit_anom / n_anom
        sup_norm = hit_norm / n_norm
        lift = (sup_anom + 1e-9) / (sup_norm + 1e-9)
        rows.append({"pattern": " ∧ ".join(str(x) for x in pattern), "len": len(pattern),
                     "sup_anom": round(sup_anom, 3), "sup_norm": round(sup_norm, 3), "lift": round(lift, 2)})
    rows = sorted(rows, key=lambda d: (-d["lift"], -d["sup_anom"]))
    for r, d in enumerate(rows):
        d["pct_of_anom_covered_rank"] = r + 1
    return rows, base_rate


@pytest.mark.parametrize("seed,frac_anom", [(0, 0.1), (1, 0.0), (2, 1.0)])
def test_pattern_fault_analysis_matches_reference(engine, seed, frac_anom):
    rows = datagen.regime_txns(3000, 8, 5, 4, 0.3, seed=seed)
    rng = np.random.default_rng(seed)
    anom = (rng.random(len(rows)) < frac_anom).astype(int)
    engine.load_csr(*datagen.txns_to_csr(rows))
    mfis = engine.mine(60).sets()
    assert len(mfis) > 10
    txns = [list(map(int, r)) for r in rows]
    got, base = pattern_fault_analysis(engine, mfis, rows, anom)
    want, base_w = _reference_table(mfis, txns, anom)
    assert base == base_w
    assert got == want
    ha, hn = pattern_fault_counts(engine, [p for p, _ in mfis], rows, anom)
    for (p, c), a, b in zip(mfis, ha, hn):
        assert a + b == c      # label items split every support exactly
