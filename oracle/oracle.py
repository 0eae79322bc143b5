"""ctypes front end of the C oracle plus the reference's threshold and root rules.

TEST INFRASTRUCTURE: used by tests, the smoke check and bench.py's CPU baseline
only.  Every function cites the reference code it restates (paths relative to
the reference project root).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

__all__ = [
    "build", "lib", "build_bitmaps", "support_batch", "cooccurrence",
    "mine_mfi", "mine_fast", "mine_engine", "thresh_from", "tensorfim_mfis",
    "anyfim_stages", "item_counts", "freq_order", "parse_fimi", "online_bins", "planted_kat",
    "bmma_bench_bits",
]


class _Mfis(C.Structure):
    _fields_ = [("n", C.c_uint64), ("ptr", C.POINTER(C.c_uint64)),
                ("items", C.POINTER(C.c_uint32)), ("support", C.POINTER(C.c_uint32)),
                ("nodes", C.c_uint64)]


_lib = None


def build(force=False):
    """Compile liboracle.so with gcc (the recipe lives in oracle/Makefile)."""
    srcs = ("mfi_oracle.c", "online_oracle.c", "kat_oracle.c", "Makefile")
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, s)) for s in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u64p, u32p = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)
        L.orc_build_bitmaps.argtypes = [u64p, u32p, C.c_uint64, C.c_uint32, C.c_uint64, u64p, u32p]
        L.orc_support_batch.argtypes = [u64p, C.c_uint32, C.c_uint64, u64p, u32p, C.c_uint64, u32p, C.c_int]
        L.orc_cooccurrence.argtypes = [u64p, C.c_uint32, C.c_uint64, u32p, C.c_int]
        L.orc_mine_dfs.argtypes = [u64p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(_Mfis)]
        L.orc_mine_fast.argtypes = [u64p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(_Mfis)]
        L.orc_mine_fast_order.argtypes = [u64p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(_Mfis)]
        L.orc_mine_engine.argtypes = [u64p, C.c_uint32, C.c_uint64, C.c_uint32, u32p, C.c_uint32, C.c_uint64, C.POINTER(_Mfis)]
        L.orc_free.argtypes = [C.POINTER(_Mfis)]
        L.orc_online_bins.argtypes = [C.POINTER(C.c_double), C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                      C.c_uint32, C.c_int, C.POINTER(C.c_double), u32p]
        L.orc_online_bins.restype = C.c_int64
        L.orc_planted_kat.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, u32p, u32p, u32p,
                                      C.POINTER(C.c_double)]
        L.orc_planted_kat.restype = C.c_int
        for f in ("orc_mine_dfs", "orc_mine_fast", "orc_mine_fast_order", "orc_mine_engine"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def build_bitmaps(row_ptr, items, d, n_words=None):
    """kernel_bitmap.cu:374-379 -- returns (bitmaps u64[d, W], counts u32[d])."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.uint64)
    items = np.ascontiguousarray(items, dtype=np.uint32)
    n = len(row_ptr) - 1
    W = (n + 63) // 64 if n_words is None else n_words
    bm = np.zeros((d, max(W, 1)), dtype=np.uint64)
    cnt = np.zeros(d, dtype=np.uint32)
    lib().orc_build_bitmaps(_p(row_ptr, C.c_uint64), _p(items, C.c_uint32), n, d, W,
                            _p(bm, C.c_uint64), _p(cnt, C.c_uint32))
    return bm[:, :W] if W else bm[:, :0], cnt


def support_batch(bm, cand_ptr, cand_items, n_threads=None):
    """kernel_bitmap.cu:390-408 per candidate: popcount of the AND of its bitmaps."""
    bm = np.ascontiguousarray(bm, dtype=np.uint64)
    cand_ptr = np.ascontiguousarray(cand_ptr, dtype=np.uint64)
    cand_items = np.ascontiguousarray(cand_items, dtype=np.uint32)
    n = len(cand_ptr) - 1
    out = np.zeros(n, dtype=np.uint32)
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    lib().orc_support_batch(_p(bm, C.c_uint64), bm.shape[0], bm.shape[1], _p(cand_ptr, C.c_uint64),
                            _p(cand_items, C.c_uint32), n, _p(out, C.c_uint32), int(n_threads))
    return out


def cooccurrence(bm, n_threads=None):
    """bmma_bench.cu:180-191 with A = B = item bitmaps: C[i][j] = popc(bv_i & bv_j)."""
    bm = np.ascontiguousarray(bm, dtype=np.uint64)
    d = bm.shape[0]
    out = np.zeros((d, d), dtype=np.uint32)
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    lib().orc_cooccurrence(_p(bm, C.c_uint64), d, bm.shape[1], _p(out, C.c_uint32), int(n_threads))
    return out


def _collect(m):
    n = int(m.n)
    res = []
    if n:
        ptr = np.ctypeslib.as_array(m.ptr, shape=(n + 1,)).copy()
        items = np.ctypeslib.as_array(m.items, shape=(int(ptr[-1]) or 1,)).copy()
        sup = np.ctypeslib.as_array(m.support, shape=(n,)).copy()
        for i in range(n):
            res.append((tuple(int(x) for x in items[ptr[i]:ptr[i + 1]]), int(sup[i])))
    lib().orc_free(C.byref(m))
    return res


def thresh_from(n, min_sup=0.05, min_count=None):
    """skab_spike.py:99-100: max(1, int(min_count)) or max(1, ceil(min_sup * n))."""
    if min_count is not None:
        return max(1, int(min_count))
    return max(1, int(np.ceil(min_sup * n)))


def mine_mfi(bm, n_txn, min_sup=0.05, min_count=None, node_cap=0):
    """skab_spike.py:84-135 over bitmaps; returns ([(items, support)], nodes).

    ``node_cap`` reproduces the reference's search-tree limit
    (skab_spike.py:109-116, 200,000 there); 0 means no limit.  Exceeding the
    cap raises ``RuntimeError`` as the reference does.
    """
    bm = np.ascontiguousarray(bm, dtype=np.uint64)
    thr = thresh_from(n_txn, min_sup, min_count)
    m = _Mfis()
    rc = lib().orc_mine_dfs(_p(bm, C.c_uint64), bm.shape[0], bm.shape[1], n_txn, thr,
                            node_cap, C.byref(m))
    nodes = int(m.nodes)
    if rc == 1:
        lib().orc_free(C.byref(m))
        raise RuntimeError(f"search tree exceeds node cap {node_cap}")
    if rc < 0:
        raise MemoryError("oracle allocation failed")
    return _collect(m), nodes


def mine_fast(bm, n_txn, thr, node_cap=0, order="support", key=None):
    """Pruned exact MFI miner (PEP/HUT/FHUT, projection): [(items, support)], nodes.
    ``order``: "support" (each node's extensions in ascending support),
    "support_desc" (the reference's global descending-support order) or "key"
    (one global order of ascending ``key[item]``); the set is the same, the
    number of nodes is not."""
    bm = np.ascontiguousarray(bm, dtype=np.uint64)
    m = _Mfis()
    code = {"support": 0, "support_desc": 1, "key": 2}[order]
    kv = np.ascontiguousarray(key if key is not None else np.zeros(bm.shape[0]), dtype=np.float64)
    if len(kv) < bm.shape[0]:
        raise ValueError("key needs one value per bitmap row")
    rc = lib().orc_mine_fast_order(_p(bm, C.c_uint64), bm.shape[0], bm.shape[1], n_txn, max(1, int(thr)),
                                   node_cap, code, _p(kv, C.c_double), C.byref(m))
    nodes = int(m.nodes)
    if rc == 1:
        lib().orc_free(C.byref(m))
        raise RuntimeError(f"search tree exceeds node cap {node_cap}")
    if rc < 0:
        raise MemoryError("oracle allocation failed")
    return _collect(m), nodes


def mine_engine(bm, thr, roots, node_cap=0):
    """The engines' task-stack DFS (kernel_bitmap.cu:841-894,
    AnytimeMining/kernel.cu:850-899) from the given dense root items."""
    bm = np.ascontiguousarray(bm, dtype=np.uint64)
    roots = np.ascontiguousarray(roots, dtype=np.uint32)
    m = _Mfis()
    rc = lib().orc_mine_engine(_p(bm, C.c_uint64), bm.shape[0], bm.shape[1], int(thr),
                               _p(roots, C.c_uint32), len(roots), node_cap, C.byref(m))
    if rc == 1:
        lib().orc_free(C.byref(m))
        raise RuntimeError(f"search tree exceeds node cap {node_cap}")
    if rc < 0:
        raise MemoryError("oracle allocation failed")
    return _collect(m)


# ---------------------------------------------------------------- engine rules
def online_bins(values, window=30, stride=15, n_bins=3, anomaly=None, n_threads=None):
    """code/pipeline/online_discretize.py:22-128 (run_file over every sensor) in C
    -> (edges [n_win, S, n_bins+1], items [n_win, S] sensor * n_bins + bin,
    labels [n_win] = the window's max flag)."""
    values = np.ascontiguousarray(values, dtype=np.float64)
    n, S = values.shape
    n_win = (n - window) // stride + 1 if n >= window else 0
    edges = np.zeros((max(n_win, 1), S, n_bins + 1), np.float64)
    items = np.zeros((max(n_win, 1), S), np.uint32)
    got = lib().orc_online_bins(_p(values, C.c_double), n, S, window, stride, n_bins,
                                n_threads or os.cpu_count() or 1, _p(edges, C.c_double), _p(items, C.c_uint32))
    if got < 0:
        raise ValueError("orc_online_bins: bad arguments")
    assert got == n_win
    labels = np.zeros(n_win, np.int64)
    if anomaly is not None:
        for w in range(n_win):
            labels[w] = int(np.max(anomaly[w * stride:w * stride + window]))
    return edges[:n_win], items[:n_win].astype(np.int64), labels


def bmma_bench_bits(words, seed):
    """bmma_bench.cu:196-207 fill_random_bits restated: two xorshift streams
    ANDed, folded with the upper half (~12.5% density) -> (uint32 words, state)."""
    m = (1 << 64) - 1
    s = seed
    s2 = (seed * 0x2545F4914F6CDD1D + 0x123456789) & m
    out = np.empty(words, dtype=np.uint32)
    for w in range(words):
        s ^= (s << 13) & m
        s ^= s >> 7
        s ^= (s << 17) & m
        s2 ^= (s2 << 13) & m
        s2 ^= s2 >> 7
        s2 ^= (s2 << 17) & m
        out[w] = (s & s2 & 0xFFFFFFFF) & (s >> 32)
    return out, s


def planted_kat(n_tx=1 << 23, d=512, n_pat=80, maxpat=6):
    """batch_proto.cu:45-51,193-231: the reference's planted-pattern data set
    -> (bitmaps uint64 [d, n_tx/64], patterns [tuple of items], frequencies,
    minsup = (int)(n_tx * 0.15 / 100))."""
    W32 = n_tx // 32
    bits = np.zeros(d * W32, dtype=np.uint32)
    ptr = np.zeros(n_pat + 1, dtype=np.uint32)
    items = np.zeros(n_pat * maxpat, dtype=np.uint32)
    freq = np.zeros(n_pat, dtype=np.float64)
    rc = lib().orc_planted_kat(n_tx, d, n_pat, maxpat, _p(bits, C.c_uint32), _p(ptr, C.c_uint32),
                               _p(items, C.c_uint32), _p(freq, C.c_double))
    if rc != 0:
        raise ValueError("orc_planted_kat: bad arguments")
    pats = [tuple(int(x) for x in items[ptr[p]:ptr[p + 1]]) for p in range(n_pat)]
    bm = bits.view(np.uint64).reshape(d, W32 // 2)
    return bm, pats, freq, int(n_tx * 0.15 / 100.0)


def parse_fimi(path):
    """kernel_bitmap.cu:205-233 byte scan: one transaction per '\\n' (empty lines
    kept as empty transactions), non-negative integers are items, a '-' and the
    digits after it are dropped, any other byte separates; a last line without
    '\\n' still counts when it holds an item."""
    data = open(path, "rb").read()
    rows, row = [], []
    i, n = 0, len(data)
    while i < n:
        c = data[i]
        if c == 0x0A:
            rows.append(row); row = []; i += 1; continue
        if 0x30 <= c <= 0x39:
            v = 0
            while i < n and 0x30 <= data[i] <= 0x39:
                v = v * 10 + (data[i] - 0x30); i += 1
            row.append(v); continue
        if c == 0x2D:
            i += 1
            while i < n and 0x30 <= data[i] <= 0x39:
                i += 1
            continue
        i += 1
    if row:
        rows.append(row)
    return rows


def item_counts(rows):
    """kernel_bitmap.cu:269-275: occurrences per id 0..itemIDmax (duplicates count)."""
    mx = max((x for r in rows for x in r), default=0)
    cnt = np.zeros(mx + 1, dtype=np.int64)
    for r in rows:
        for x in r:
            cnt[x] += 1
    return cnt


def freq_order(cnt):
    """kernel_bitmap.cu:276-283: ids by count descending, stable (ties ascending id)."""
    return np.argsort(-np.asarray(cnt), kind="stable")


def _dense_bitmaps(rows, keep_ids):
    """Bitmaps over the kept original ids (dense order = ascending original id)."""
    o2d = {int(x): i for i, x in enumerate(keep_ids)}
    rp = [0]
    items = []
    for r in rows:
        for x in r:
            if x in o2d:
                items.append(o2d[x])
        rp.append(len(items))
    bm, _ = build_bitmaps(np.array(rp, np.uint64), np.array(items, np.uint32), len(keep_ids))
    return bm


def tensorfim_mfis(rows, rel_thr):
    """MFIs the TensorFIM engines report for ``<fimi> <rel_thr>``.

    kernel_bitmap.cu:809 and kernel_bmma.cu:1189: frequencyThreshold =
    transNum * supportThreshold (double), extensions need count >= it;
    roots are the first dimensionReduced items of the frequency order, where
    dimensionReduced counts ids with count / transNum > supportThreshold
    (strict, kernel_bitmap.cu:817; kernel_bmma.cu:1199); item id 0 is never
    a candidate (kernel_bitmap.cu:354-356).  Returns {frozenset(orig ids): freq}.
    """
    n = len(rows)
    cnt = item_counts(rows)
    thr_d = n * float(rel_thr)
    thr = max(0, math.ceil(thr_d))
    keep = [i for i in range(1, len(cnt)) if cnt[i] >= thr_d]
    if not keep:
        return {}
    dim_red = int(sum(1 for v in cnt if float(v) / n > rel_thr))
    dense_cnt = np.array([cnt[i] for i in keep])
    order = freq_order(dense_cnt)
    roots = order[:min(dim_red, len(keep))]
    bm = _dense_bitmaps(rows, keep)
    res = mine_engine(bm, max(thr, 1), roots)
    return {frozenset(keep[i] for i in s): f for s, f in res}


def anyfim_stages(rows, upto_stage):
    """Per-stage MFI pools of the anytime engine (AnytimeMining/kernel.cu:844-899).

    Stage k uses threshold = count of the k-th item of the frequency order over
    all ids 0..itemIDmax (:846), roots = the first k ids of that order (:850-859),
    survivors = ids >= 1 with count >= the (upto_stage+1)-th count (:336-342).
    Returns {k: {frozenset(orig ids): freq}}.
    """
    cnt = item_counts(rows)
    order = freq_order(cnt)
    sorted_cnt = cnt[order]
    final_thr = sorted_cnt[upto_stage] if upto_stage < len(sorted_cnt) else 0
    keep = [i for i in range(1, len(cnt)) if cnt[i] >= final_thr]
    o2d = {x: i for i, x in enumerate(keep)}
    bm = _dense_bitmaps(rows, keep)
    out = {}
    for k in range(1, upto_stage + 1):
        thr = int(sorted_cnt[k - 1])
        roots = [o2d[int(x)] for x in order[:k] if int(x) in o2d]
        res = mine_engine(bm, thr, np.array(roots, np.uint32)) if roots else []
        out[k] = {frozenset(keep[i] for i in s): f for s, f in res}
    return out
