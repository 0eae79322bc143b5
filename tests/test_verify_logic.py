"""The MFI-set checks of sgfim.verify on the CPU: the oracle stands in for the
GPU handle, and the mistakes are planted in the oracle's own result."""
import numpy as np

import oracle
from sgfim import datagen
from sgfim.verify import check_mfi_set


class OracleEngine:
    """The calls sgfim.verify makes, answered by the CPU oracle."""

    def __init__(self, bm=None, n_ids=0):
        self.bm, self.n_ids = bm, n_ids

    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass

    def load_csr(self, rp, it):
        self.n_ids = int(it.max()) + 1 if len(it) else 0
        self.bm, _ = oracle.build_bitmaps(rp, it, self.n_ids)

    def info(self):
        return {"n_ids": self.n_ids}

    def support_batch(self, cp, ci):
        return oracle.support_batch(self.bm, cp, ci, n_threads=2)

    def frequent_extensions(self, sp, si, thr):
        out = np.zeros((len(sp) - 1, (self.n_ids + 63) // 64), np.uint64)
        for s in range(len(sp) - 1):
            items = [int(x) for x in si[int(sp[s]):int(sp[s + 1])]]
            ext = [e for e in range(self.n_ids) if e not in items]
            cp = np.arange(len(ext) + 1, dtype=np.uint64) * (len(items) + 1)
            ci = np.array([x for e in ext for x in items + [e]], np.uint32)
            sup = oracle.support_batch(self.bm, cp, ci, n_threads=2)
            for e, c in zip(ext, sup):
                if c >= max(1, thr):
                    out[s, e >> 6] |= np.uint64(1) << np.uint64(e & 63)
        return out


class _Res:
    def __init__(self, sets):
        self.ptr = np.zeros(len(sets) + 1, np.uint64)
        self.ptr[1:] = np.cumsum([len(s) for s, _ in sets])
        self.items = np.array([x for s, _ in sets for x in sorted(s)], np.uint32)
        self.support = np.array([c for _, c in sets], np.uint32)


def _case():
    rows = datagen.regime_txns(3_000, 6, 4, 3, 0.3, seed=2)
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, 24)
    thr = 150
    mfis, _ = oracle.mine_fast(bm, len(rows), thr)
    return OracleEngine(bm, 24), [(tuple(s), c) for s, c in mfis], thr


def test_checks_pass_on_the_exact_set():
    eng, mfis, thr = _case()
    rep = check_mfi_set(eng, _Res(mfis), thr, walks=400, seed=0, engine_factory=OracleEngine)
    assert rep["supports_recount_equal"] and rep["antichain"] and rep["maximal_all"] and rep["walks_all_found"]


def test_checks_catch_planted_mistakes():
    eng, mfis, thr = _case()
    # a non-maximal set in place of an MFI: maximality fails, and so does the antichain when both stay
    big = max(range(len(mfis)), key=lambda i: len(mfis[i][0]))
    s, _ = mfis[big]
    sub = tuple(s[:-1])
    cp = np.array([0, len(sub)], np.uint64)
    sub_sup = int(eng.support_batch(cp, np.array(sub, np.uint32))[0])
    bad = mfis[:big] + [(sub, sub_sup)] + mfis[big + 1:]
    rep = check_mfi_set(eng, _Res(bad), thr, walks=0, engine_factory=OracleEngine)
    assert not rep["maximal_all"] and rep["not_maximal"] == 1
    rep = check_mfi_set(eng, _Res(mfis + [(sub, sub_sup)]), thr, walks=0, engine_factory=OracleEngine)
    assert not rep["antichain"]
    # a wrong support
    wrong = [(s, c + (i == 0)) for i, (s, c) in enumerate(mfis)]
    assert not check_mfi_set(eng, _Res(wrong), thr, walks=0, engine_factory=OracleEngine)["supports_recount_equal"]
    # a missing MFI: enough walks land on it
    rep = check_mfi_set(eng, _Res(mfis[1:]), thr, walks=4000, seed=1, engine_factory=OracleEngine)
    assert rep["maximal_all"] and rep["walks_missing"] > 0 and not rep["walks_all_found"]
