"""Seeded synthetic workloads for the MFI mining engine.

The reference measures its engines on sensor datasets (SKAB, C-MAPSS, AI4I, HAI,
CWRU) that are transactionised by ``window_transactions``
(code/pipeline/skab_spike.py:61-80): every transaction holds exactly one
``sensor=bin`` state item per sensor.  Those datasets are not shipped with the
reference, so every workload here is generated from a seeded latent-regime
mixture with the same shape:

* ``regime_txns``      one item per sensor per transaction; the regime of each
                       transaction is drawn from Dirichlet(alpha_regime)
                       weights and each (regime, sensor) has its own
                       Dirichlet(alpha_bin) bin distribution.
* ``correlated_bitmaps`` vertical bitmaps for the support-counting kernels:
                       per-item marginal density log-uniform in [lo, hi],
                       correlated through latent regimes.
* ``walk_candidates``  candidate itemsets of size k ~ U{kmin..kmax} grown by a
                       random walk over item pairs that co-occur.

Item ids returned by the generators are 0-based dense ids; FIMI files written
from them are 1-based (``write_fimi`` in code/pipeline/engine_adapter.py:37
numbers items from 1).

All randomness comes from ``numpy.random.default_rng(seed)`` (PCG64), whose
streams are identical on x86-64 and aarch64, so the same seed yields the same
workload on every machine.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "regime_txns", "txns_to_csr", "csr_to_bitmaps", "correlated_bitmaps",
    "walk_candidates", "write_fimi_ids", "CONFIGS",
]

# Named workloads (sizes, alphas, floors).  Every one is generated from a seed.
CONFIGS = {
    # 20,000 txns, 8 sensors x 5 bins, 4 regimes, floor 200 (1%)
    "mfi-small": dict(n_txn=20_000, n_sensors=8, n_bins=5, n_regimes=4,
                      alpha_bin=0.3, alpha_regime=1.0, floor=200),
    # 1,048,576 txns x 1,024 items, 16 regimes, density log-U[2%,20%];
    # 1,000,000 candidates of size 3..8
    "support-1m": dict(n_txn=1 << 20, d=1024, n_regimes=16, dens_lo=0.02,
                       dens_hi=0.20, n_cand=1_000_000, kmin=3, kmax=8),
    # 2,000,000 txns, 80 sensors x 8 bins, 32 regimes, alpha 0.2, floor 0.5%
    "anytime-2m": dict(n_txn=2_000_000, n_sensors=80, n_bins=8, n_regimes=32,
                       alpha_bin=0.2, alpha_regime=1.0, floor_frac=0.005),
    # sliding-window service: 21 sensors x 6 bins, 8 regimes, floor 2%
    "windows-4096": dict(n_req=4096, len_lo=512, len_hi=65_536, n_sensors=21,
                         n_bins=6, n_regimes=8, alpha_bin=0.3,
                         alpha_regime=1.0, floor_frac=0.02, rate_hz=2000.0),
}


def _regime_tables(rng, n_sensors, n_bins, n_regimes, alpha_bin, alpha_regime):
    w = rng.dirichlet(np.full(n_regimes, float(alpha_regime)))
    p = rng.dirichlet(np.full(n_bins, float(alpha_bin)),
                      size=(n_regimes, n_sensors))          # [R, S, B]
    cdf = np.cumsum(p, axis=2)
    cdf[:, :, -1] = 1.0                                     # guard rounding
    return w, p, cdf


def regime_txns(n_txn, n_sensors, n_bins, n_regimes, alpha_bin,
                alpha_regime=1.0, seed=0, chunk=1 << 16, return_model=False):
    """Transactions with exactly one item per sensor.

    Returns an ``int32`` array ``[n_txn, n_sensors]`` whose entry ``(t, s)`` is
    the dense item id ``s * n_bins + bin``; rows are ascending because sensors
    own disjoint id ranges.
    """
    rng = np.random.default_rng(seed)
    w, p, cdf = _regime_tables(rng, n_sensors, n_bins, n_regimes,
                               alpha_bin, alpha_regime)
    out = np.empty((n_txn, n_sensors), dtype=np.int32)
    base = (np.arange(n_sensors, dtype=np.int32) * n_bins)[None, :]
    for t0 in range(0, n_txn, chunk):
        t1 = min(n_txn, t0 + chunk)
        z = rng.choice(n_regimes, size=t1 - t0, p=w)
        u = rng.random((t1 - t0, n_sensors))
        c = cdf[z]                                          # [n, S, B]
        b = (u[:, :, None] >= c[:, :, :-1]).sum(axis=2, dtype=np.int32)
        out[t0:t1] = base + b
    if return_model:
        return out, dict(w=w, p=p)
    return out


def txns_to_csr(rows):
    """Dense ``[n, width]`` rows or a list of id lists -> (row_ptr u64, items u32)."""
    if isinstance(rows, np.ndarray) and rows.ndim == 2:
        n, width = rows.shape
        row_ptr = np.arange(n + 1, dtype=np.uint64) * np.uint64(width)
        return row_ptr, np.ascontiguousarray(rows, dtype=np.uint32).reshape(-1)
    lens = np.fromiter((len(r) for r in rows), dtype=np.uint64, count=len(rows))
    row_ptr = np.zeros(len(rows) + 1, dtype=np.uint64)
    np.cumsum(lens, out=row_ptr[1:])
    items = np.fromiter((x for r in rows for x in r), dtype=np.uint32,
                        count=int(row_ptr[-1]))
    return row_ptr, items


def csr_to_bitmaps(row_ptr, items, d, n_words=None):
    """Vertical bitmaps ``uint64[d, n_words]``: bit ``t & 63`` of word ``t >> 6``
    of row ``e`` is set when transaction ``t`` holds item ``e``
    (code/engine_tensorfim/code/engine/src/kernel_bitmap.cu:374-379)."""
    n = len(row_ptr) - 1
    if n_words is None:
        n_words = (n + 63) // 64
    bm = np.zeros((d, n_words), dtype=np.uint64)
    lens = np.diff(row_ptr.astype(np.int64))
    t = np.repeat(np.arange(n, dtype=np.int64), lens)
    it = items.astype(np.int64)
    np.bitwise_or.at(bm, (it, t >> 6), np.left_shift(np.uint64(1), (t & 63).astype(np.uint64)))
    return bm


def correlated_bitmaps(n_txn, d, n_regimes, dens_lo, dens_hi, seed=0,
                       chunk=1 << 16, return_model=False):
    """Vertical bitmaps with log-uniform marginals correlated through regimes.

    Each transaction draws a regime ``r`` (Dirichlet(1) weights); item ``j`` is
    present with probability ``m_j * a[r, j] / sum_r w_r a[r, j]`` where
    ``m_j`` ~ log-U[dens_lo, dens_hi] is the target marginal and ``a`` are
    Exp(1) regime scales, so the marginal density of item ``j`` is ``m_j``
    (up to clipping at 1).
    """
    assert n_txn % 64 == 0 and chunk % 64 == 0
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(n_regimes))
    m = np.exp(rng.uniform(np.log(dens_lo), np.log(dens_hi), size=d))
    a = rng.exponential(1.0, size=(n_regimes, d))
    p = np.minimum(1.0, m[None, :] * a / (w @ a)[None, :]).astype(np.float32)
    n_words = n_txn // 64
    bm = np.empty((d, n_words), dtype=np.uint64)
    for t0 in range(0, n_txn, chunk):
        t1 = min(n_txn, t0 + chunk)
        z = rng.choice(n_regimes, size=t1 - t0, p=w)
        u = rng.random((t1 - t0, d), dtype=np.float32)
        bits = np.ascontiguousarray((u < p[z]).T)            # [d, n]
        packed = np.ascontiguousarray(np.packbits(bits, axis=1, bitorder="little"))
        bm[:, t0 // 64:t1 // 64] = packed.view("<u8")
    if return_model:
        return bm, dict(w=w, p=p, m=m)
    return bm


def walk_candidates(n_cand, d, kmin, kmax, seed=0, pair_ok=None):
    """Candidate itemsets grown by a random walk over co-occurring pairs.

    The first item is uniform; each further item is uniform over the items that
    co-occur with the previously added item (``pair_ok[last, j]``) and are not
    yet in the set.  Returns CSR ``(cand_ptr u64, cand_items u32)`` with items
    sorted ascending inside each candidate.
    """
    rng = np.random.default_rng(seed)
    if pair_ok is None:
        pair_ok = np.ones((d, d), dtype=bool)
    pair_ok = pair_ok.copy()
    np.fill_diagonal(pair_ok, False)
    k = rng.integers(kmin, kmax + 1, size=n_cand)
    sets = np.full((n_cand, kmax), -1, dtype=np.int64)
    sets[:, 0] = rng.integers(0, d, size=n_cand)
    for pos in range(1, kmax):
        need = np.nonzero(k > pos)[0]
        last = sets[need, pos - 1]
        pick = np.full(len(need), -1, dtype=np.int64)
        todo = np.arange(len(need))
        for _ in range(64):
            if len(todo) == 0:
                break
            c = rng.integers(0, d, size=len(todo))
            ok = pair_ok[last[todo], c]
            ok &= ~(sets[need[todo], :pos] == c[:, None]).any(axis=1)
            pick[todo[ok]] = c[ok]
            todo = todo[~ok]
        if len(todo):
            raise RuntimeError("random walk stuck: pair graph too sparse")
        sets[need, pos] = pick
    sets = np.sort(np.where(sets < 0, np.iinfo(np.int64).max, sets), axis=1)
    cand_ptr = np.zeros(n_cand + 1, dtype=np.uint64)
    np.cumsum(k, out=cand_ptr[1:])
    mask = np.arange(kmax)[None, :] < k[:, None]
    cand_items = sets[mask].astype(np.uint32)
    return cand_ptr, cand_items


def write_fimi_ids(path, rows, one_based=True):
    """Write transactions as a FIMI file: one line per transaction, ascending
    space-separated ids (the layout ``write_fimi`` produces,
    code/pipeline/engine_adapter.py:37-56)."""
    off = 1 if one_based else 0
    with open(path, "w", encoding="utf-8") as f:
        if isinstance(rows, np.ndarray):
            for r in rows:
                f.write(" ".join(map(str, (np.sort(r) + off).tolist())))
                f.write("\n")
        else:
            for r in rows:
                f.write(" ".join(str(x + off) for x in sorted(set(r))))
                f.write("\n")


def sensor_stream(n_rows, n_sensors, seed, constant_cols=(), anomaly_rate_permille=50):
    """Seeded synthetic sensor stream in thousandths (ties, as in CSV input):
    per-sensor integer random-walk level, regime shifts, a triangle wave and
    noise, built from integer draws only so every platform produces the same
    doubles; listed columns are constant.  Returns (values [n, S] float64,
    anomaly [n] int32)."""
    rng = np.random.default_rng(seed)
    t = np.arange(n_rows, dtype=np.int64)
    vals = np.empty((n_rows, n_sensors), dtype=np.float64)
    regime = np.cumsum(rng.integers(0, 500, n_rows) == 0) % 4
    for c in range(n_sensors):
        level = np.cumsum(rng.integers(-20, 21, n_rows))
        shift = rng.integers(-1500, 1501, 4)[regime]
        period = int(rng.integers(50, 400))
        tri = np.abs((t % period) - period // 2) * 8
        noise = rng.integers(-300, 301, n_rows)
        vals[:, c] = (level + shift + tri + noise) / 1000.0
    for c in constant_cols:
        vals[:, c] = 1.25
    anom = (rng.integers(0, 1000, n_rows) < anomaly_rate_permille).astype(np.int32)
    return vals, anom
