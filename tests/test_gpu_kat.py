"""The reference's own known-answer data sets, at their own sizes, through the
GPU engine: the planted-pattern set of batch_proto.cu (8,388,608 transactions
x 512 items, 80 planted patterns, minsup 0.15%) and the seeded sparse bits of
bmma_bench.cu's correctness gate."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def planted():
    return oracle.planted_kat()


def test_planted_patterns_mined_exactly(engine, planted):
    """batch_proto.cu:376-408's checks on the MFI engine: every planted pattern
    whose exact support reaches minsup is inside a reported MFI and none that
    misses it is (recall, no false positives); the MFI set equals the exact
    oracle's, every reported support recounted."""
    bm, pats, freq, minsup = planted
    n_tx = bm.shape[1] * 64
    engine.load_bitmaps(bm, n_tx)
    res = engine.mine(minsup)
    got = res.as_dict()
    want, _ = oracle.mine_fast(bm, n_tx, minsup)
    assert got == {frozenset(s): c for s, c in want}
    cp = np.cumsum([0] + [len(p) for p in pats]).astype(np.uint64)
    ci = np.array([x for p in pats for x in p], np.uint32)
    sup = oracle.support_batch(bm, cp, ci)
    assert np.array_equal(engine.support_batch(cp, ci), sup)
    mfis = list(got)
    for p, s in zip(pats, sup):
        inside = any(frozenset(p) <= m for m in mfis)
        assert inside == (s >= minsup), (p, int(s), minsup)
    # downward closure of what was reported: every MFI's supports recounted exactly
    mp = np.cumsum([0] + [len(m) for m in mfis]).astype(np.uint64)
    mi = np.array([x for m in mfis for x in sorted(m)], np.uint32)
    assert np.array_equal(oracle.support_batch(bm, mp, mi), np.array([got[m] for m in mfis], np.uint32))


@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["auto", "popc", "bmma", "tcgen05"])
def test_bmma_bench_bits_cooccurrence(engine, kind):
    """bmma_bench.cu:196-207's seeded sparse bits (two xorshift streams, ~12.5%
    density): every co-occurrence kernel equals the exact integer product."""
    torch = pytest.importorskip("torch")
    N, d = 1 << 16, 64
    w32 = N // 32
    bits, _ = oracle.bmma_bench_bits(w32 * d, 0x9E3779B97F4A7C15)
    bm = bits.reshape(d, w32).view(np.uint64).reshape(d, w32 // 2)
    dense = np.unpackbits(bits.reshape(d, w32).view(np.uint8), axis=1, bitorder="little").astype(np.int64)
    want = dense @ dense.T
    dev = torch.device("cuda:0")
    tb = torch.from_numpy(np.ascontiguousarray(bm).view(np.int64)).to(dev)
    out = torch.zeros(d * d, dtype=torch.int32, device=dev)
    engine.cooccurrence_device(tb.data_ptr(), d, w32 // 2, w32 // 2, out.data_ptr(), kind,
                               torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32).reshape(d, d).astype(np.int64)
    assert np.array_equal(got, want)
