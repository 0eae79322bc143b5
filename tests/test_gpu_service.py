"""Device-resident ring (append / evict / window extraction) and the
sliding-window service: every window's MFI set equals the oracle's on the same
slice of the stream (bit-exact)."""
import numpy as np
import pytest

import oracle
from sgfim import datagen

pytestmark = pytest.mark.gpu


def _oracle_mfis(rows, thr, d=126):
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, d)
    res, _ = oracle.mine_fast(bm, len(rows), thr)
    return {frozenset(s): c for s, c in res}


def test_ring_windows_match_slices(engine):
    from sgfim.service import Ring
    rows = datagen.regime_txns(30_000, 21, 6, 8, 0.3, seed=1)
    rp, it = datagen.txns_to_csr(rows)
    ring = Ring(126, 4096)
    assert ring.capacity == 4096
    rng = np.random.default_rng(0)
    pos = 0
    checked = 0
    try:
        while pos < len(rows):
            n = int(rng.integers(1, 700))
            b = min(len(rows), pos + n)
            ring.append(rp[pos:b + 1] - rp[pos], it[int(rp[pos]):int(rp[b])])
            pos = b
            assert ring.head == pos
            if pos > 3000 and rng.random() < 0.2:
                length = int(rng.integers(1, 4000))
                start = pos - length - int(rng.integers(0, 4096 - length))
                engine_rows = rows[start:start + length]
                ring.window_load(engine, start, length)
                cp, ci = datagen.walk_candidates(300, 126, 1, 4, seed=checked)
                got = engine.support_batch(cp, ci)
                wrp, wit = datagen.txns_to_csr(engine_rows)
                bm, _ = oracle.build_bitmaps(wrp, wit, 126)
                assert np.array_equal(got, oracle.support_batch(bm, cp, ci)), (start, length)
                thr = max(1, int(np.ceil(0.05 * length)))
                assert engine.mine(thr).as_dict() == _oracle_mfis(engine_rows, thr)
                checked += 1
        assert checked >= 5
        # an evicted window is refused
        from sgfim.engine import SgfimError
        with pytest.raises(SgfimError):
            ring.window_load(engine, 0, 100)
    finally:
        ring.close()


def test_service_windows_exact():
    from sgfim.service import WindowService, make_requests
    rows = datagen.regime_txns(200_000, 21, 6, 8, 0.3, seed=7)
    reqs = make_requests(48, 400.0, 512, 8192, seed=3)
    svc = WindowService(workers=4, hbm_budget=2 << 30, ring_txn=1 << 16, keep_results=True)
    try:
        rep = svc.run(rows, reqs, stream_rate=20_000.0, floor_frac=0.05, warm_txn=8192)
    finally:
        svc.close()
    assert rep["windows"] == 48 and rep["errors"] == 0
    for rq in rep["requests"]:
        length = min(rq.length, rq.end)
        thr = max(1, int(np.ceil(0.05 * length)))
        assert rq.result == _oracle_mfis(rows[rq.end - length:rq.end], thr), rq.idx
