"""Autotuner: every plan it sweeps gives identical supports / co-occurrences,
the winner is applied and cached."""
import json

import numpy as np
import pytest

import oracle
from sgfim import datagen

pytestmark = pytest.mark.gpu


def test_autotune_support_and_cooc(engine, tmp_path):
    torch = pytest.importorskip("torch")
    from sgfim.autotune import Autotuner
    n_txn, d = 32 * 1024, 200
    bm = datagen.correlated_bitmaps(n_txn, d, 8, 0.02, 0.3, seed=4)
    cp, ci = datagen.walk_candidates(20_000, d, 2, 10, seed=5)
    dev = torch.device("cuda:0")
    w = bm.shape[1]
    tb = torch.from_numpy(bm.view(np.int64)).to(dev)
    tp = torch.from_numpy(cp.view(np.int64)).to(dev)
    ti = torch.from_numpy(ci.view(np.int32)).to(dev)
    out = torch.zeros(len(cp) - 1, dtype=torch.int32, device=dev)
    cache = str(tmp_path / "tune.json")
    try:
        tuner = Autotuner(engine, cache)
        best, ms = tuner.tune_support(tb, d, w, w, tp, ti, len(cp) - 1, out)
        assert len(ms) >= 4 and best[0] in ("staged", "staged4", "sorted", "stream")
        assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle.support_batch(bm, cp, ci))
        co = torch.zeros(d * d, dtype=torch.int32, device=dev)
        kind, cms = tuner.tune_cooc(tb, d, w, w, co)
        assert kind in cms and len(cms) == 4
        assert np.array_equal(co.cpu().numpy().view(np.uint32).reshape(d, d), oracle.cooccurrence(bm))
        saved = json.load(open(cache))
        assert len(saved) == 2
        # a second tuner reads the cache instead of sweeping
        again = Autotuner(engine, cache)
        assert tuple(again.tune_support(tb, d, w, w, tp, ti, len(cp) - 1, out)[0]) == tuple(best)
    finally:
        engine.set_support_plan("auto")
