"""Python front end of the sgfim engine (a thin layer over the C ABI).

``Engine`` keeps one handle: bitmaps stay resident on the GPU between calls.
Methods map one-to-one onto include/sgfim.h; item ids are original ids.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _lib as L

__all__ = ["Engine", "SgfimError", "MineResult"]


class SgfimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sgfim error {code}: {msg}")
        self.code = code


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class MineResult:
    """MFIs as (tuple of original ids ascending, support), plus run statistics."""

    def __init__(self, res_ptr):
        r = res_ptr.contents
        n = int(r.n_sets)
        ptr = np.ctypeslib.as_array(r.set_ptr, shape=(n + 1,)).copy() if n else np.zeros(1, np.uint64)
        tot = int(ptr[-1])
        self.items = np.ctypeslib.as_array(r.items, shape=(tot,)).copy() if tot else np.zeros(0, np.uint32)
        self.support = np.ctypeslib.as_array(r.support, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        self.emit_time_s = np.ctypeslib.as_array(r.emit_time_s, shape=(n,)).copy() if n else np.zeros(0)
        self.emit_node = np.ctypeslib.as_array(r.emit_node, shape=(n,)).copy() if n else np.zeros(0, np.uint64)
        self.ptr = ptr
        self.n_txn = int(r.n_txn)
        self.min_count = int(r.min_count)
        self.elapsed_s = float(r.elapsed_s)
        self.nodes = int(r.nodes)
        self.waves = int(r.waves)
        self.kernel_launches = int(r.kernel_launches)
        self.candidates = int(r.candidates)
        self.phase_s = dict(zip(("counts", "pool", "fhut", "final_filter", "scoring", "other", "expand", "assemble"),
                                (float(x) for x in r.phase_s)))
        tn, td = int(r.trace_n), int(r.trace_dim)
        if tn:
            self.trace_features = np.ctypeslib.as_array(r.trace_features, shape=(tn * td,)).reshape(tn, td).copy()
            self.trace_labels = np.ctypeslib.as_array(r.trace_labels, shape=(tn,)).copy()
        else:
            self.trace_features = np.zeros((0, td or L.TRACE_DIM), np.float32)
            self.trace_labels = np.zeros(0, np.uint8)

    def coverage_curve(self, emit_times=None):
        """Sorted emission times of the final MFIs: coverage(t) = fraction emitted by t."""
        t = np.sort(self.emit_time_s if emit_times is None else emit_times)
        return t

    def time_to_coverage(self, frac):
        """Seconds until ``frac`` of the final MFIs had been emitted."""
        t = np.sort(self.emit_time_s)
        if len(t) == 0:
            return 0.0
        k = max(1, int(math.ceil(frac * len(t))))
        return float(t[k - 1])

    def nodes_to_coverage(self, frac):
        """Search nodes expanded until ``frac`` of the final MFIs had been emitted."""
        t = np.sort(self.emit_node)
        if len(t) == 0:
            return 0
        k = max(1, int(math.ceil(frac * len(t))))
        return int(t[k - 1])

    def __len__(self):
        return len(self.support)

    def sets(self):
        p, it = self.ptr, self.items
        return [(tuple(int(x) for x in it[p[i]:p[i + 1]]), int(self.support[i])) for i in range(len(self))]

    def as_dict(self):
        return {frozenset(s): c for s, c in self.sets()}


class Engine:
    def __init__(self, device=0, hbm_budget=0, wave_nodes=0, verbose=False, phase_timers=False,
                 ignore_id0=False, blocking_sync=False, windows_horizontal=False, wait_limit_us=0, projection=None):
        """projection: None = the miner decides by size, True = always project root
        subtrees, False = never (see SGFIM_F_PROJECT / SGFIM_F_NO_PROJECTION)."""
        self._L = L.load()
        flags = (L.F_VERBOSE if verbose else 0) | (L.F_PHASE_TIMERS if phase_timers else 0) | \
            (L.F_IGNORE_ID0 if ignore_id0 else 0) | (L.F_BLOCKING_SYNC if blocking_sync else 0) | \
            (L.F_WINDOWS_HORIZONTAL if windows_horizontal else 0) | \
            (L.F_PROJECT if projection is True else L.F_NO_PROJECTION if projection is False else 0)
        cfg = L.Config(device, hbm_budget, wave_nodes, flags, None, wait_limit_us)
        h = C.c_void_p()
        rc = self._L.sgfim_open(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise SgfimError(rc, "sgfim_open failed (no CUDA device?)")
        self._h = h
        self._keep = []

    # ------------------------------------------------------------ plumbing
    def _check(self, rc):
        if rc != 0:
            msg = self._L.sgfim_last_error(self._h)
            raise SgfimError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sgfim_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def device_status(self, stream=0):
        """sgfim_device_status: 0, or SGFIM_EDEVICE when a device-pointer call since the
        last check gave up on a bounded wait (the error word is cleared)."""
        return int(self._L.sgfim_device_status(self._h, C.c_void_p(stream)))

    def selftest_wait(self):
        """sgfim_selftest_wait: a kernel whose wait can never complete; returns the
        call's code (SGFIM_EDEVICE when the bound works)."""
        return int(self._L.sgfim_selftest_wait(self._h))

    # ------------------------------------------------------------ loading
    def load_fimi(self, path):
        self._check(self._L.sgfim_load_fimi(self._h, os.fsencode(path)))
        return self

    def load_csr(self, row_ptr, items):
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        items = np.ascontiguousarray(items, dtype=np.uint32)
        if len(items) == 0:
            items = np.zeros(1, np.uint32)
        self._check(self._L.sgfim_load_csr(self._h, _p(row_ptr, C.c_uint64), _p(items, C.c_uint32),
                                           len(row_ptr) - 1))
        return self

    def load_rows(self, rows):
        from .datagen import txns_to_csr
        return self.load_csr(*txns_to_csr(rows))

    def transactionize(self, values, window=30, stride=15, n_bins=3, anomaly=None, load=False):
        """Sensor stream [n_rows, n_sensors] -> (items [n_windows, n_sensors]
        dense ids, labels [n_windows], edges: list of per-sensor arrays) on the
        GPU (sgfim_transactionize); ``load=True`` also makes the transactions
        this handle's dataset."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        if values.ndim != 2:
            raise ValueError("values must be [n_rows, n_sensors]")
        n, S = values.shape
        an = None
        if anomaly is not None:
            an = np.ascontiguousarray(anomaly, dtype=np.int32)
            if an.shape != (n,):
                raise ValueError("one anomaly flag per row")
        n_win = (n - window) // stride + 1 if n >= window else 0
        edges = np.zeros(S * (n_bins + 1), np.float64)
        n_edges = np.zeros(S, np.uint32)
        items = np.zeros(max(1, n_win * S), np.uint32)
        labels = np.zeros(max(1, n_win), np.int32)
        nw = C.c_uint64(0)
        rc = self._L.sgfim_transactionize(self._h, _p(values, C.c_double), n, S,
                                          an.ctypes.data_as(C.POINTER(C.c_int32)) if an is not None else None,
                                          window, stride, n_bins, L.TX_LOAD if load else 0, _p(edges, C.c_double),
                                          _p(n_edges, C.c_uint32), _p(items, C.c_uint32),
                                          labels.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(nw))
        self._check(rc)
        assert nw.value == n_win
        e = [edges[s * (n_bins + 1):s * (n_bins + 1) + int(n_edges[s])].copy() for s in range(S)]
        return items[:n_win * S].reshape(n_win, S).astype(np.int64), labels[:n_win].astype(np.int64), e

    def transactionize_online(self, values, window=30, stride=15, n_bins=3, anomaly=None, load=False,
                              with_edges=True, lanes=0, full_recurrence=False):
        """Online form (P² edges per window, sgfim_transactionize_online):
        -> (items [n_windows, n_sensors] dense ids, labels [n_windows], edges
        [n_windows, n_sensors, n_bins+1] or None without ``with_edges``).
        ``lanes``: estimator chains per warp (0 = automatic);
        ``full_recurrence``: step every estimator through the whole stream
        instead of stopping once its estimate can no longer change."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        if values.ndim != 2:
            raise ValueError("values must be [n_rows, n_sensors]")
        n, S = values.shape
        an = None
        if anomaly is not None:
            an = np.ascontiguousarray(anomaly, dtype=np.int32)
            if an.shape != (n,):
                raise ValueError("one anomaly flag per row")
        n_win = (n - window) // stride + 1 if n >= window and window >= 1 and stride >= 1 else 0
        edges = np.zeros((max(1, n_win), S, max(n_bins, 0) + 1), np.float64) if with_edges else None
        items = np.zeros(max(1, n_win * S), np.uint32)
        labels = np.zeros(max(1, n_win), np.int32)
        nw = C.c_uint64(0)
        rc = self._L.sgfim_transactionize_online(
            self._h, _p(values, C.c_double), n, S,
            an.ctypes.data_as(C.POINTER(C.c_int32)) if an is not None else None, window, stride, n_bins,
            (L.TX_LOAD if load else 0) | (L.TX_P2_FULL if full_recurrence else 0) | ((int(lanes) & 63) << 8),
            _p(edges, C.c_double) if with_edges else None,
            _p(items, C.c_uint32),
            labels.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(nw))
        self._check(rc)
        assert nw.value == n_win
        return (items[:n_win * S].reshape(n_win, S).astype(np.int64), labels[:n_win].astype(np.int64),
                edges[:n_win] if with_edges else None)

    def load_bitmaps(self, bm, n_txn):
        bm = np.ascontiguousarray(bm, dtype=np.uint64)
        d, w = bm.shape
        self._check(self._L.sgfim_load_bitmaps(self._h, _p(bm, C.c_uint64), d, int(n_txn), w))
        return self

    def info(self):
        i = L.DatasetInfo()
        self._check(self._L.sgfim_dataset_info_get(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in L.DatasetInfo._fields_}

    def item_counts(self, n=None):
        if n is None:
            n = self.info()["n_ids"]
        out = np.zeros(max(n, 1), dtype=np.uint32)
        self._check(self._L.sgfim_item_counts(self._h, _p(out, C.c_uint32), n))
        return out[:n]

    # ------------------------------------------------------------ counting
    def support_batch(self, cand_ptr, cand_items, out=None):
        """Supports of the CSR candidates (original ids).  ``out``: an optional
        uint32 array of at least n_cand entries to write into (e.g. pinned host
        memory, so that the device-to-host copy runs at full speed)."""
        cand_ptr = np.ascontiguousarray(cand_ptr, dtype=np.uint64)
        cand_items = np.ascontiguousarray(cand_items, dtype=np.uint32)
        if len(cand_items) == 0:
            cand_items = np.zeros(1, np.uint32)
        n = len(cand_ptr) - 1
        if out is None:
            out = np.zeros(max(n, 1), dtype=np.uint32)
        elif out.dtype != np.uint32 or not out.flags.c_contiguous or len(out) < max(n, 1):
            raise ValueError("out must be a contiguous uint32 array of n_cand entries")
        self._check(self._L.sgfim_support_batch(self._h, _p(cand_ptr, C.c_uint64), _p(cand_items, C.c_uint32),
                                                n, _p(out, C.c_uint32)))
        return out[:n]

    def support_batch_device(self, bm_ptr, d, n_words, row_stride, cand_ptr_ptr, cand_items_ptr, n_cand,
                             out_ptr, stream=0):
        self._check(self._L.sgfim_support_batch_device(self._h, bm_ptr, d, n_words, row_stride, cand_ptr_ptr,
                                                       cand_items_ptr, n_cand, out_ptr, stream or None))

    KERNELS = {"auto": 0, "staged": 1, "sorted": 2, "stream": 3, "staged4": 4, "lane": 5, "lane_tm": 6}

    def set_support_plan(self, kernel="auto", cands_per_cta=0, waves=0):
        """Choose the support-batch kernel and its CTA sizing (see sgfim_support_plan_set)."""
        self._check(self._L.sgfim_support_plan_set(self._h, self.KERNELS[kernel], int(cands_per_cta), int(waves)))

    def frequent_extensions(self, set_ptr, set_items, min_count):
        """sgfim_frequent_extensions: uint64 masks [n_sets, ceil(n_ids / 64)]; bit id is set
        when set + {id} is frequent.  An all-zero row means the set is maximal."""
        sp = np.ascontiguousarray(set_ptr, dtype=np.uint64)
        si = np.ascontiguousarray(set_items, dtype=np.uint32)
        if len(si) == 0:
            si = np.zeros(1, np.uint32)
        n = len(sp) - 1
        mw = max(1, (self.info()["n_ids"] + 63) // 64)
        out = np.zeros((max(n, 0), mw), np.uint64)
        if n > 0:
            self._check(self._L.sgfim_frequent_extensions(self._h, _p(sp, C.c_uint64), _p(si, C.c_uint32), n,
                                                          int(min_count), _p(out, C.c_uint64), mw))
        return out

    def phase_stats(self, reset=True):
        """Summed CUDA-event phase times of support-batch calls (needs phase_timers=True)."""
        s = L.PhaseStats()
        self._check(self._L.sgfim_phase_stats_get(self._h, C.byref(s), 1 if reset else 0))
        return {k: getattr(s, k) for k, _ in L.PhaseStats._fields_}

    def cooccurrence(self):
        """d x d co-occurrence of the bitmap rows (d = info()['rows'])."""
        d = self.info()["rows"]
        out = np.zeros((max(d, 1), max(d, 1)), dtype=np.uint32)
        self._check(self._L.sgfim_cooccurrence(self._h, _p(out, C.c_uint32), d))
        return out[:d, :d]

    def cooccurrence_device(self, bm_ptr, d, n_words, row_stride, out_ptr, kind=L.COOC_AUTO, stream=0):
        self._check(self._L.sgfim_cooccurrence_device(self._h, bm_ptr, d, n_words, row_stride, out_ptr, kind,
                                                      stream or None))

    # ------------------------------------------------------------ mining
    ORDERS = {"support": L.ORDER_SUPPORT, "learned": L.ORDER_LEARNED, "support_desc": L.ORDER_SUPPORT_DESC}

    def _params(self, min_count, roots=None, root_min_count=None, order="support", time_limit_s=0.0,
                node_limit=0, record_trace=False):
        p = L.MineParams()
        p.min_count = int(min_count)
        p.root_rule = L.ROOTS_ALL
        if roots is not None:
            r = np.ascontiguousarray(roots, dtype=np.uint32)
            if len(r) == 0:
                r = np.zeros(1, np.uint32)
                p.n_roots = 0
            else:
                p.n_roots = len(r)
            self._keep.append(r)
            p.roots = _p(r, C.c_uint32)
            p.root_rule = L.ROOTS_LIST
        elif root_min_count is not None:
            p.root_rule = L.ROOTS_MINCOUNT
            p.root_min_count = int(root_min_count)
        p.order = self.ORDERS[order]
        p.time_limit_s = float(time_limit_s)
        p.node_limit = int(node_limit)
        p.record_trace = 1 if record_trace else 0
        return p

    def mine(self, min_count, **kw):
        """Exact MFIs at absolute threshold ``min_count`` (see sgfim_mine)."""
        p = self._params(min_count, **kw)
        res = C.POINTER(L.Result)()
        rc = self._L.sgfim_mine(self._h, C.byref(p), C.byref(res))
        self._keep.clear()
        self._check(rc)
        try:
            return MineResult(res)
        finally:
            self._L.sgfim_result_free(res)

    def mine_anytime(self, min_count, checkpoints, callback=None, materialize=True, records=None, **kw):
        """Mine with wall-clock checkpoints.  ``callback(t_s, elapsed_s, sets)``
        receives the emitted candidates as a list of (ids tuple, support);
        returning True stops the search.  ``materialize=False`` keeps only the
        counts in the records (no per-set Python objects).  ``records`` (a list)
        receives the checkpoint records as they happen, so they survive a time or
        node limit.  Returns (result, records)."""
        p = self._params(min_count, **kw)
        cks = np.ascontiguousarray(checkpoints, dtype=np.float64)
        if records is None:
            records = []

        def _cb(user, ckp):
            ck = ckp.contents
            n = int(ck.n_emitted)
            sets = None
            if materialize:
                ptr = np.ctypeslib.as_array(ck.set_ptr, shape=(n + 1,)) if n else np.zeros(1, np.uint64)
                tot = int(ptr[-1])
                it = np.ctypeslib.as_array(ck.items, shape=(tot,)) if tot else np.zeros(0, np.uint32)
                sp = np.ctypeslib.as_array(ck.support, shape=(n,)) if n else np.zeros(0, np.uint32)
                sets = [(tuple(int(x) for x in it[ptr[i]:ptr[i + 1]]), int(sp[i])) for i in range(n)]
            records.append({"t_s": ck.t_s, "elapsed_s": ck.elapsed_s, "n_emitted": n, "nodes": int(ck.nodes),
                            "sets": sets})
            if callback is not None:
                return 1 if callback(ck.t_s, ck.elapsed_s, sets) else 0
            return 0

        cb = L.CKPT_CB(_cb)
        res = C.POINTER(L.Result)()
        rc = self._L.sgfim_mine_anytime(self._h, C.byref(p), _p(cks, C.c_double) if len(cks) else None,
                                        len(cks), cb, None, C.byref(res))
        self._keep.clear()
        self._check(rc)
        try:
            return MineResult(res), records
        finally:
            self._L.sgfim_result_free(res)

    # ------------------------------------------------------------ scoring
    def mlp_forward(self, X, n, in_dim, hidden, W1, b1, W2, b2, w3, b3, Z1, Z2, P, stream=0):
        """Device pointers (ints); see sgfim_mlp_forward."""
        self._check(self._L.sgfim_mlp_forward(self._h, X, n, in_dim, hidden, W1, b1, W2, b2, w3, b3,
                                              Z1 or None, Z2 or None, P, stream or None))

    def mlp_backward(self, X, n, in_dim, hidden, W2, w3, Z1, Z2, P, Y, WT, scale, dW1, db1, dW2, db2, dw3, db3,
                     loss, stream=0):
        self._check(self._L.sgfim_mlp_backward(self._h, X, n, in_dim, hidden, W2, w3, Z1, Z2, P, Y, WT or None,
                                               scale, dW1, db1, dW2, db2, dw3, db3, loss, stream or None))

    def adam_step(self, param, grad, m, v, param_bf16, n, lr, beta1, beta2, eps, step, weight_decay, stream=0):
        self._check(self._L.sgfim_adam_step(self._h, param, grad, m, v, param_bf16 or None, n, lr, beta1, beta2,
                                            eps, step, weight_decay, stream or None))

    def load_scorer(self, w1, b1, w2, b2, w3, b3):
        """Weights as float arrays (converted to bf16 here, round-to-nearest-even)."""
        from .mlp import to_bf16_bits
        ws = [np.ascontiguousarray(to_bf16_bits(w)) for w in (w1, w2, w3)]
        bs = [np.ascontiguousarray(b, dtype=np.float32) for b in (b1, b2, b3)]
        hidden, in_dim = w1.shape
        self._check(self._L.sgfim_load_scorer(self._h, in_dim, hidden,
                                              _p(ws[0], C.c_uint16), _p(bs[0], C.c_float),
                                              _p(ws[1], C.c_uint16), _p(bs[1], C.c_float),
                                              _p(ws[2], C.c_uint16), _p(bs[2], C.c_float)))


def thresh_from(n, min_sup=0.05, min_count=None):
    """The reference's threshold rule (code/pipeline/skab_spike.py:99-100)."""
    if min_count is not None:
        return max(1, int(min_count))
    return max(1, int(math.ceil(float(np.float64(min_sup) * n))))
