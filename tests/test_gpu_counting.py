"""GPU parity of the counting kernels (support batches, co-occurrence) against
the CPU oracle.  All counts are integers: the bar is bit-exact equality."""
import numpy as np
import pytest

import oracle
from sgfim import datagen

pytestmark = pytest.mark.gpu


def _bitmaps(n_txn, d, seed, lo=0.02, hi=0.3):
    return datagen.correlated_bitmaps(n_txn, d, 8, lo, hi, seed=seed)


@pytest.mark.parametrize("n_txn,d,n_cand,kmin,kmax", [
    (64 * 1024, 256, 20000, 3, 8),      # staged kernel, several CTAs
    (4096, 40, 3000, 1, 8),             # single-chunk bitmaps, k=1..8
    (64 * 1000 + 64, 300, 5000, 2, 6),  # odd word count, d not a multiple of 256
    (128 * 64, 1024, 9000, 3, 8),       # four TMA boxes
    (8192 + 64, 1792, 40000, 1, 8),     # the widest lane layout (seven boxes)
    (8192, 1800, 3000, 2, 9),           # too wide for the lane layout: another kernel
])
def test_support_batch_matches_oracle(engine, n_txn, d, n_cand, kmin, kmax):
    bm = _bitmaps(n_txn, d, seed=n_txn + d)
    engine.load_bitmaps(bm, n_txn)
    cp, ci = datagen.walk_candidates(n_cand, d, kmin, kmax, seed=d)
    got = engine.support_batch(cp, ci)
    ref = oracle.support_batch(bm, cp, ci)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("kernel", ["lane", "lane_tm", "sorted", "staged", "staged4", "stream"])
@pytest.mark.parametrize("d", [1024, 300])
def test_support_kernels_agree(engine, kernel, d):
    """Every kernel plan gives the oracle's supports (k = 0..12, unknown ids included)."""
    n_txn = 32 * 1024 + 64
    bm = _bitmaps(n_txn, d, seed=d + 5)
    engine.load_bitmaps(bm, n_txn)
    cp, ci = datagen.walk_candidates(12000, d, 1, 12, seed=11)
    # prepend an empty candidate and one with an unknown id
    cp = np.concatenate([[0, 0, 2], cp + 2]).astype(np.uint64)
    ci = np.concatenate([[3, d + 7], ci]).astype(np.uint32)
    try:
        for cpc, waves in [(0, 0), (777, 0), (0, 5)]:
            engine.set_support_plan(kernel, cpc, waves)
            got = engine.support_batch(cp, ci)
            want = oracle.support_batch(bm, cp[2:] - 2, ci[2:])
            assert got[0] == n_txn and got[1] == 0
            assert np.array_equal(got[2:], want), (kernel, cpc, waves)
    finally:
        engine.set_support_plan("auto")


def test_support_batch_edge_candidates(engine):
    n_txn, d = 8192, 50
    bm = _bitmaps(n_txn, d, seed=1)
    engine.load_bitmaps(bm, n_txn)
    sets = [[], [3], list(range(0, 12)),          # empty, single, k > 8 (streaming path)
            [5, 5, 5], [49], [10, 60], [70],       # repeated id, last row, unknown ids -> 0
            list(range(20, 40)), [1, 2, 3, 4, 5, 6, 7, 8]]
    cp = np.zeros(len(sets) + 1, np.uint64)
    cp[1:] = np.cumsum([len(s) for s in sets])
    ci = np.array([x for s in sets for x in s], np.uint32)
    got = engine.support_batch(cp, ci)
    dense = np.unpackbits(bm.view(np.uint8), axis=1, bitorder="little")[:, :n_txn].astype(bool)
    for i, s in enumerate(sets):
        if not s:
            want = n_txn
        elif any(x >= d for x in s):
            want = 0
        else:
            want = int(np.all(dense[s], axis=0).sum())
        assert got[i] == want, (i, s)


def test_support_batch_bad_csr_and_sparse_ids(engine):
    """A decreasing cand_ptr is refused (checked on the device) and the handle
    stays usable; after a CSR load (sparse original ids) candidates map through
    the device remap: absent ids give 0."""
    from sgfim.engine import SgfimError
    bm = _bitmaps(4096, 20, seed=4)
    engine.load_bitmaps(bm, 4096)
    with pytest.raises(SgfimError):
        engine.support_batch(np.array([0, 3, 2, 4], np.uint64), np.array([1, 2, 3, 4], np.uint32))
    assert engine.support_batch(np.array([0, 1], np.uint64), np.array([3], np.uint32))[0] == \
        oracle.support_batch(bm, np.array([0, 1], np.uint64), np.array([3], np.uint32))[0]
    rows = [[5, 100, 7], [100, 7], [5], [900, 5, 7], [7]]
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    sets = [[5], [7, 100], [5, 7], [900], [6], [1000], [5, 7, 900], []]
    cp = np.zeros(len(sets) + 1, np.uint64)
    cp[1:] = np.cumsum([len(x) for x in sets])
    ci = np.array([x for x in sets for x in x], np.uint32)
    want = [sum(1 for r in rows if set(x) <= set(r)) for x in sets]
    assert engine.support_batch(cp, ci).tolist() == want


def test_support_batch_device_pointer_api(engine):
    torch = pytest.importorskip("torch")
    n_txn, d = 32 * 1024, 128
    bm = _bitmaps(n_txn, d, seed=7)
    cp, ci = datagen.walk_candidates(7000, d, 3, 8, seed=8)
    dev = torch.device("cuda:0")
    tb = torch.from_numpy(bm.view(np.int64)).to(dev)
    tp = torch.from_numpy(cp.view(np.int64)).to(dev)
    ti = torch.from_numpy(ci.view(np.int32)).to(dev)
    out = torch.zeros(len(cp) - 1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    engine.support_batch_device(tb.data_ptr(), d, bm.shape[1], bm.shape[1], tp.data_ptr(), ti.data_ptr(),
                                len(cp) - 1, out.data_ptr(), stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, oracle.support_batch(bm, cp, ci))


def test_support_full_size_sample(engine):
    """The 1,048,576 x 1,024 workload: 200,000 candidates on the GPU, a seeded
    sample of 2,000 re-counted by the oracle, plus size-independent checks."""
    n_txn, d = 1 << 20, 1024
    bm = datagen.correlated_bitmaps(n_txn, d, 16, 0.02, 0.2, seed=0)
    engine.load_bitmaps(bm, n_txn)
    cp, ci = datagen.walk_candidates(200_000, d, 3, 8, seed=1)
    got = engine.support_batch(cp, ci)
    rng = np.random.default_rng(2)
    idx = np.sort(rng.choice(len(got), 2000, replace=False))
    sp = np.zeros(len(idx) + 1, np.uint64)
    sp[1:] = np.cumsum(np.diff(cp)[idx])
    si = np.concatenate([ci[cp[i]:cp[i + 1]] for i in idx])
    assert np.array_equal(got[idx], oracle.support_batch(bm, sp, si))
    # anti-monotonicity: dropping the last item never lowers the support
    k = np.diff(cp).astype(np.int64)
    pp = np.zeros(len(k) + 1, np.uint64)
    pp[1:] = np.cumsum(k - 1)
    keep = np.ones(len(ci), bool)
    keep[(cp[1:] - 1).astype(np.int64)] = False
    parent = engine.support_batch(pp, ci[keep])
    assert (parent >= got).all()


@pytest.mark.parametrize("kind", [1, 2, 3, 4])
@pytest.mark.parametrize("n_txn,d", [(4096, 24), (65536 + 64, 300), (1 << 16, 256), (100_032, 130), (200_064, 700)])
def test_cooccurrence_matches_oracle(engine, kind, n_txn, d):
    torch = pytest.importorskip("torch")
    bm = _bitmaps(n_txn, d, seed=d + kind)
    dev = torch.device("cuda:0")
    w = bm.shape[1]
    stride = w + (w & 1)
    host = np.zeros((d, stride), np.uint64)
    host[:, :w] = bm
    tb = torch.from_numpy(host.view(np.int64)).to(dev)
    out = torch.zeros(d * d, dtype=torch.int32, device=dev)
    engine.cooccurrence_device(tb.data_ptr(), d, w, stride, out.data_ptr(), kind,
                               torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32).reshape(d, d)
    assert np.array_equal(got, oracle.cooccurrence(bm))


def test_cooccurrence_host_api(engine):
    rows = datagen.regime_txns(5000, 8, 5, 4, 0.3, seed=3)
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    got = engine.cooccurrence()
    bm, _ = oracle.build_bitmaps(rp, it, 40)
    present = np.nonzero(oracle.cooccurrence(bm).diagonal())[0]
    assert np.array_equal(got, oracle.cooccurrence(bm)[np.ix_(present, present)])


def test_transpose_and_counts(engine):
    rows = [[5, 1, 9], [], [9], [1, 1, 5], [7]] * 300
    rp, it = datagen.txns_to_csr(rows)
    engine.load_csr(rp, it)
    info = engine.info()
    assert info["n_txn"] == 1500 and info["n_present"] == 4 and info["id_min"] == 1 and info["id_max"] == 9
    # occurrence counts count a duplicated id twice (kernel_bitmap.cu:269-275); supports do not
    assert engine.item_counts(10).tolist() == [0, 900, 0, 0, 0, 600, 0, 300, 0, 600]
    cp = np.array([0, 1, 2, 3, 5], np.uint64)
    ci = np.array([1, 9, 7, 1, 5], np.uint32)
    assert engine.support_batch(cp, ci).tolist() == [600, 600, 300, 600]
