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


@pytest.mark.parametrize("mode,schedulers", [("batched", 1), ("batched", 3), ("workers", 1)])
def test_service_windows_exact(mode, schedulers):
    """Every window of a replayed request stream equals the oracle's MFIs: one
    batch scheduler, three concurrent batch schedulers sharing the ring, and the
    per-window workers."""
    from sgfim.service import WindowService, make_requests
    rows = datagen.regime_txns(200_000, 21, 6, 8, 0.3, seed=7)
    reqs = make_requests(48, 400.0, 512, 8192, seed=3)
    svc = WindowService(workers=4, hbm_budget=2 << 30, ring_txn=1 << 16, keep_results=True, mode=mode,
                        schedulers=schedulers)
    try:
        rep = svc.run(rows, reqs, stream_rate=20_000.0, floor_frac=0.05, warm_txn=8192)
    finally:
        svc.close()
    assert rep["windows"] == 48 and rep["errors"] == 0 and rep["mode"] == mode
    if mode == "batched":
        assert rep["batched_windows"] == 48
    for rq in rep["requests"]:
        length = min(rq.length, rq.end)
        thr = max(1, int(np.ceil(0.05 * length)))
        assert rq.result.as_dict() == _oracle_mfis(rows[rq.end - length:rq.end], thr), rq.idx


@pytest.mark.parametrize("horizontal", [False, True], ids=["vertical", "horizontal"])
def test_ring_mine_windows_batched(horizontal):
    """One batched launch over windows of every size class, including the
    empty window, floors above the window length and floor 1, with the ring
    wrapped: each window's MFIs equal the oracle's, and the kernel (not the
    wave miner) mined them."""
    from sgfim.engine import Engine
    from sgfim.service import Ring
    rows = datagen.regime_txns(300_000, 21, 6, 8, 0.3, seed=11)
    rp, it = datagen.txns_to_csr(rows)
    ring = Ring(126, 1 << 17)
    engine = Engine(windows_horizontal=horizontal)
    try:
        ring.append(rp, it)            # wraps: the ring keeps the newest 131,072
        head = ring.head
        rng = np.random.default_rng(5)
        lens = [0, 1, 7, 64, 65, 512, 513, 4096, 20_000, 65_536, 100_000]
        lens += [int(np.exp(rng.uniform(np.log(512), np.log(65536)))) for _ in range(40)]
        starts, thrs = [], []
        for i, L in enumerate(lens):
            starts.append(head - L - int(rng.integers(0, (1 << 17) - L + 1)))
            thrs.append(max(1, int(np.ceil(0.02 * L))))
        thrs[1] = 1
        thrs[3] = 1000          # above the window length
        thrs[5] = 1             # every distinct maximal transaction
        # split windows (>= 4,096 transactions) at denser floors and a floor above the length
        for L, thr in ((8192, 164), (8192, 82), (5000, 10 ** 6), (4096, 1)):
            lens.append(L)
            starts.append(head - L - int(rng.integers(0, (1 << 17) - L + 1)))
            thrs.append(thr)
        res = ring.mine_windows(engine, starts, lens, thrs)
        assert len(res) == len(lens) and (res.status == 0).all()
        assert res.batched.all() and res.launches >= 1 and res.kernel_ms > 0
        for w, (s, L, thr) in enumerate(zip(starts, lens, thrs)):
            assert res.as_dict(w) == _oracle_mfis(rows[s:s + L], thr), (w, s, L, thr)
        # the same windows through the wave miner agree
        for w in (4, 7, 9):
            ring.window_load(engine, starts[w], lens[w])
            assert engine.mine(thrs[w]).as_dict() == res.as_dict(w)
        # a window no longer in the ring is refused
        from sgfim.engine import SgfimError
        with pytest.raises(SgfimError):
            ring.mine_windows(engine, [0], [10], [1])
    finally:
        ring.close()
        engine.close()


def test_appends_wait_for_windows_being_mined(engine):
    """Appends from another thread that would overwrite windows of a running
    batch wait for it; every window still matches the oracle."""
    import threading
    import time
    from sgfim.service import Ring
    rows = datagen.regime_txns(400_000, 21, 6, 8, 0.3, seed=13)
    rp, it = datagen.txns_to_csr(rows)
    cap = 1 << 16
    ring = Ring(126, cap)
    try:
        ring.append(rp[:cap + 1], it[:int(rp[cap])])
        lens = [4096] * 24 + [cap - 100]
        starts = [i * 2000 for i in range(24)] + [50]
        thrs = [max(1, int(np.ceil(0.02 * L))) for L in lens]
        out = {}

        def miner():
            out["res"] = ring.mine_windows(engine, starts, lens, thrs)

        m = threading.Thread(target=miner)
        m.start()
        time.sleep(0.05)      # the call registers its windows first thing
        # ten batches, the first of which already overwrites the oldest windows
        for k in range(10):
            a, b = cap + k * 10_000, cap + (k + 1) * 10_000
            ring.append(rp[a:b + 1] - rp[a], it[int(rp[a]):int(rp[b])])
        out["head"] = ring.head
        m.join()
        res = out["res"]
        assert out["head"] == cap + 100_000 and (res.status == 0).all()
        for w, (s, L, thr) in enumerate(zip(starts, lens, thrs)):
            assert res.as_dict(w) == _oracle_mfis(rows[s:s + L], thr), w
    finally:
        ring.close()


def test_mine_windows_wide_ring_uses_wave_miner(engine):
    """A ring of more than 128 items has no item masks: every window goes to
    the wave miner, and the results come back as 4-word masks, equal to the
    oracle's."""
    from sgfim.service import Ring, masks_to_sets
    rows = datagen.regime_txns(12_000, 25, 8, 6, 0.3, seed=21)   # 200 items
    rp, it = datagen.txns_to_csr(rows)
    ring = Ring(200, 1 << 14)
    try:
        ring.append(rp, it)
        starts, lens = [0, 5000, 11_000], [4000, 7000, 1000]
        thrs = [max(1, int(np.ceil(0.04 * L))) for L in lens]
        res = ring.mine_windows(engine, starts, lens, thrs)
        assert res.mask_words == 4 and not res.batched.any() and (res.status == 0).all()
        for w, (s, L, t) in enumerate(zip(starts, lens, thrs)):
            assert res.as_dict(w) == _oracle_mfis(rows[s:s + L], t, d=200), w
        assert masks_to_sets(np.array([[1, 0, 0, 1 << 3]], np.uint64)) == [(0, 195)]
    finally:
        ring.close()


def test_ring_mine_windows_many_windows_filter_layout():
    """More split windows than two per SM: the cross-subtree filter runs 256-thread
    CTAs (1,024-thread ones below that count); every window still equals the oracle."""
    from sgfim.engine import Engine
    from sgfim.service import Ring
    rows = datagen.regime_txns(40_000, 21, 6, 8, 0.3, seed=23)
    rp, it = datagen.txns_to_csr(rows)
    ring = Ring(126, 1 << 16)
    engine = Engine()
    try:
        ring.append(rp, it)
        rng = np.random.default_rng(8)
        lens = [int(x) for x in rng.integers(64, 1500, 420)]
        starts = [int(rng.integers(0, len(rows) - L)) for L in lens]
        thrs = [max(1, int(np.ceil(0.04 * L))) for L in lens]
        res = ring.mine_windows(engine, starts, lens, thrs)
        assert (res.status == 0).all() and res.batched.all()
        for w, (s, L, thr) in enumerate(zip(starts, lens, thrs)):
            assert res.as_dict(w) == _oracle_mfis(rows[s:s + L], thr), (w, s, L, thr)
    finally:
        ring.close()
        engine.close()
