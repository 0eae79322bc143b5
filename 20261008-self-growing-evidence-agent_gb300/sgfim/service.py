"""Sliding-window MFI mining service on one GPU.

Workload "windows-4096": a stream of transactions (21 sensors x 6 bins = 126
items, one item per sensor per transaction, 8-regime mixture) arrives at
``stream_rate`` transactions/s and is appended into a device-resident bitmap
ring (sgfim_ring_*; appends evict the oldest transactions).  Requests arrive
as a Poisson process; request i asks for the MFIs of the newest L_i
transactions at its arrival, L_i log-uniform in [512, 65,536], at floor
ceil(2% * L_i).  Worker threads, each owning an engine handle (its own CUDA
stream and reused device workspace), take requests in arrival order; a request
is admitted when its device-memory estimate fits the service's HBM budget.
Latency = completion - arrival.  Reports p50/p99 latency and windows/s.

The reference has no service (it transactionises windows on the host,
code/pipeline/skab_spike.py:61-80, and starts one engine process per file).
"""
from __future__ import annotations

import ctypes as C
import heapq
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import datagen
from .engine import Engine, SgfimError

WORKLOAD = dict(n_req=4096, len_lo=512, len_hi=65536, n_sensors=21, n_bins=6, n_regimes=8, alpha_bin=0.3,
                floor_frac=0.02, rate_hz=2000.0, stream_rate=100_000.0, ring_txn=1 << 22)


class Ring:
    """Python handle of sgfim_ring (device-resident transaction ring)."""

    def __init__(self, n_items, capacity_txn, device=0):
        self._L = L.load()
        r = C.c_void_p()
        rc = self._L.sgfim_ring_open(device, n_items, capacity_txn, C.byref(r))
        if rc != 0:
            raise SgfimError(rc, "sgfim_ring_open failed")
        self._r = r

    @property
    def head(self):
        return int(self._L.sgfim_ring_head(self._r))

    @property
    def capacity(self):
        return int(self._L.sgfim_ring_capacity(self._r))

    def append(self, row_ptr, items):
        row_ptr = np.ascontiguousarray(row_ptr, np.uint64)
        items = np.ascontiguousarray(items, np.uint32)
        if len(items) == 0:
            items = np.zeros(1, np.uint32)
        rc = self._L.sgfim_ring_append(self._r, row_ptr.ctypes.data_as(L.u64p), items.ctypes.data_as(L.u32p),
                                       len(row_ptr) - 1)
        if rc != 0:
            raise SgfimError(rc, "sgfim_ring_append failed")

    def window_load(self, eng, start, length):
        rc = self._L.sgfim_ring_window_load(self._r, eng.handle, int(start), int(length))
        eng._check(rc)

    def mine_windows(self, eng, starts, lens, min_counts):
        """MFIs of many windows in one batched launch (sgfim_ring_mine_windows)."""
        starts = np.ascontiguousarray(starts, np.uint64)
        lens = np.ascontiguousarray(lens, np.uint64)
        mc = np.ascontiguousarray(min_counts, np.uint32)
        n = len(starts)
        if not (len(lens) == n and len(mc) == n):
            raise ValueError("starts, lens and min_counts must have the same length")
        if n == 0:
            starts, lens, mc = np.zeros(1, np.uint64), np.zeros(1, np.uint64), np.zeros(1, np.uint32)
        res = C.POINTER(L.WindowsResult)()
        rc = self._L.sgfim_ring_mine_windows(self._r, eng.handle, starts.ctypes.data_as(L.u64p),
                                             lens.ctypes.data_as(L.u64p), mc.ctypes.data_as(L.u32p), n,
                                             C.byref(res))
        eng._check(rc)
        return WindowsMined(res, self._L)

    def close(self):
        if getattr(self, "_r", None):
            self._L.sgfim_ring_close(self._r)
            self._r = None


def masks_to_sets(masks):
    """[k, words] uint64 item masks -> list of ascending item-id tuples."""
    masks = np.ascontiguousarray(masks, np.uint64)
    if len(masks) == 0:
        return []
    bits = np.unpackbits(masks.view(np.uint8).reshape(len(masks), -1), axis=1, bitorder="little")
    rows, cols = np.nonzero(bits)
    cuts = np.searchsorted(rows, np.arange(1, len(masks)))
    return [tuple(int(x) for x in c) for c in np.split(cols, cuts)]


class WindowsMined:
    """Per-window MFIs of sgfim_ring_mine_windows.  The masks and supports are
    numpy views of the library's result arrays (no copy); the result is freed
    when this object is."""

    def __init__(self, res_ptr, lib):
        self._res, self._L = res_ptr, lib
        r = res_ptr.contents
        n = int(r.n_windows)
        self.mask_words = int(r.mask_words)
        self.offset = np.ctypeslib.as_array(r.offset, shape=(n + 1,)).copy()
        tot = int(self.offset[-1])
        self.masks = (self._view(r.masks, C.c_uint64, tot * self.mask_words, np.uint64).reshape(tot, self.mask_words)
                      if tot else np.zeros((0, self.mask_words), np.uint64))
        self.support = self._view(r.support, C.c_uint32, tot, np.uint32) if tot else np.zeros(0, np.uint32)
        self.status = np.ctypeslib.as_array(r.status, shape=(n,)).copy() if n else np.zeros(0, np.int32)
        self.nodes = np.ctypeslib.as_array(r.nodes, shape=(n,)).copy() if n else np.zeros(0, np.uint64)
        self.batched = np.ctypeslib.as_array(r.batched, shape=(n,)).copy() if n else np.zeros(0, np.uint8)
        self.elapsed_s = float(r.elapsed_s)
        self.kernel_ms = float(r.kernel_ms)
        self.launches = int(r.launches)
        self.warps = int(r.warps)
        self.tasks = int(r.tasks)
        self.task_kernel_ms = float(r.task_kernel_ms)
        self.task_ms_max = float(r.task_ms_max)
        self.task_ms_sum = float(r.task_ms_sum)

    def _view(self, ptr, ctype, count, dtype):
        # the buffer object references this result, so the views keep it (and its memory) alive
        buf = (ctype * count).from_address(C.addressof(ptr.contents))
        buf._owner = self
        return np.frombuffer(buf, dtype=dtype)

    def __del__(self):
        if getattr(self, "_res", None) is not None:
            self._L.sgfim_windows_result_free(self._res)
            self._res = None

    def __len__(self):
        return len(self.status)

    def count(self, w):
        return int(self.offset[w + 1] - self.offset[w])

    def sets(self, w):
        a, b = int(self.offset[w]), int(self.offset[w + 1])
        return list(zip(masks_to_sets(self.masks[a:b]), (int(x) for x in self.support[a:b])))

    def as_dict(self, w):
        return {frozenset(s): c for s, c in self.sets(w)}


@dataclass(order=True)
class Request:
    arrival: float
    idx: int = field(compare=False)
    length: int = field(compare=False)
    end: int = field(compare=False, default=0)       # stream position of the window end
    start_s: float = field(compare=False, default=0.0)
    done_s: float = field(compare=False, default=0.0)
    n_mfis: int = field(compare=False, default=0)
    mine_s: float = field(compare=False, default=0.0)
    nodes: int = field(compare=False, default=0)
    error: str = field(compare=False, default="")
    result: object = field(compare=False, default=None)


def make_requests(n, rate_hz, len_lo, len_hi, seed):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n)
    arrival = np.cumsum(gaps)
    lengths = np.exp(rng.uniform(np.log(len_lo), np.log(len_hi), n)).astype(np.int64)
    return [Request(float(a), i, int(L_)) for i, (a, L_) in enumerate(zip(arrival, lengths))]


def window_bytes(length, n_items=126):
    """Device-memory estimate of one window's mining: bitmap + mask arena + pool."""
    words = ((length + 63) // 64 + 1) & ~1
    slots = max(4096, n_items * 64)          # the miner's mask-arena sizing
    return (n_items + slots) * words * 8 + n_items * 1026 * 8


class WindowView:
    """One window of a WindowsMined batch, with the MineResult accessors."""

    def __init__(self, batch, w):
        self.batch, self.w = batch, w

    def __len__(self):
        return self.batch.count(self.w)

    def sets(self):
        return self.batch.sets(self.w)

    def as_dict(self):
        return self.batch.as_dict(self.w)


class WindowService:
    """mode "batched": `schedulers` threads (one by default), each with its own
    handle; a free scheduler hands every queued request to one
    sgfim_ring_mine_windows call (a warp per root subtree of every window; the
    handle's HBM budget bounds the per-warp workspaces and the output arena), so
    with two a new batch starts while the previous one is still on the GPU.  mode
    "workers": `workers` threads, each with its own handle, mine one window at
    a time with the wave miner, admitted by a per-window memory estimate."""

    def __init__(self, workers=8, hbm_budget=8 << 30, device=0, ring_txn=WORKLOAD["ring_txn"], n_items=126,
                 keep_results=False, mode="batched", max_batch=8192, schedulers=1):
        if mode not in ("batched", "workers"):
            raise ValueError("mode must be 'batched' or 'workers'")
        if schedulers < 1:
            raise ValueError("schedulers must be >= 1")
        self.mode = mode
        self.max_batch = max_batch
        self.ring = Ring(n_items, ring_txn, device)
        if mode == "batched":
            self.engines = [Engine(device=device, hbm_budget=hbm_budget, blocking_sync=True)
                            for _ in range(schedulers)]
        else:
            self.engines = [Engine(device=device, blocking_sync=True) for _ in range(workers)]
        self.budget = hbm_budget
        self.n_items = n_items
        self.keep = keep_results
        self._cv = threading.Condition()
        self._in_use = 0
        self._queue = []
        self._closed = False

    def close(self):
        for e in self.engines:
            e.close()
        self.ring.close()

    # ------------------------------------------------------------ admission
    def _admit(self, need):
        with self._cv:
            while self._in_use + need > self.budget and self._in_use > 0:
                self._cv.wait()
            self._in_use += need

    def _release(self, need):
        with self._cv:
            self._in_use -= need
            self._cv.notify_all()

    # ------------------------------------------------------------ run
    def run(self, stream_rows, requests, stream_rate, floor_frac, warm_txn=None):
        """Replay the stream and the requests in real time; returns the report."""
        rp_all, it_all = datagen.txns_to_csr(stream_rows)
        total = len(rp_all) - 1
        warm = warm_txn if warm_txn is not None else WORKLOAD["len_hi"]
        self.ring.append(rp_all[:warm + 1], it_all[:int(rp_all[warm])])
        appended = warm
        t0 = time.perf_counter()
        lock = threading.Lock()
        work = []          # heap of admitted-to-queue requests by arrival
        done = []
        stop = threading.Event()

        def produce_until(pos):
            nonlocal appended
            with lock:
                if pos > appended:
                    a, b = appended, min(pos, total)
                    if b > a:
                        self.ring.append(rp_all[a:b + 1] - rp_all[a], it_all[int(rp_all[a]):int(rp_all[b])])
                        appended = b

        def stream_pos(t):
            return min(total, warm + int(stream_rate * t))

        def dispatcher():
            for rq in requests:
                now = time.perf_counter() - t0
                if rq.arrival > now:
                    time.sleep(rq.arrival - now)
                rq.end = stream_pos(rq.arrival)
                produce_until(rq.end)
                with self._cv:
                    heapq.heappush(work, rq)
                    self._cv.notify_all()
            stop.set()
            with self._cv:
                self._cv.notify_all()

        def worker(eng):
            while True:
                with self._cv:
                    while not work and not stop.is_set():
                        self._cv.wait()
                    if not work:
                        return
                    rq = heapq.heappop(work)
                need = window_bytes(rq.length, self.n_items)
                self._admit(need)
                try:
                    rq.start_s = time.perf_counter() - t0
                    length = min(rq.length, rq.end)
                    self.ring.window_load(eng, rq.end - length, length)
                    thr = max(1, int(np.ceil(floor_frac * length)))
                    res = eng.mine(thr)
                    rq.n_mfis = len(res)
                    rq.mine_s = res.elapsed_s
                    rq.nodes = res.nodes
                    if self.keep:
                        rq.result = res   # numpy arrays; converted to Python sets after the run
                except SgfimError as e:
                    rq.error = str(e)
                finally:
                    self._release(need)
                rq.done_s = time.perf_counter() - t0
                with lock:
                    done.append(rq)

        batches = []

        def scheduler(eng):
            while True:
                with self._cv:
                    while not work and not stop.is_set():
                        self._cv.wait()
                    if not work:
                        return
                    batch = [heapq.heappop(work) for _ in range(min(len(work), self.max_batch))]
                t_start = time.perf_counter() - t0
                lens = [min(rq.length, rq.end) for rq in batch]
                starts = [rq.end - L_ for rq, L_ in zip(batch, lens)]
                thrs = [max(1, int(np.ceil(floor_frac * L_))) for L_ in lens]
                for rq in batch:
                    rq.start_s = t_start
                try:
                    res = self.ring.mine_windows(eng, starts, lens, thrs)
                    for i, rq in enumerate(batch):
                        rq.n_mfis = res.count(i)
                        rq.nodes = int(res.nodes[i])
                        rq.mine_s = res.elapsed_s
                        if res.status[i] != 0:
                            rq.error = f"sgfim error {int(res.status[i])}"
                        elif self.keep:
                            rq.result = WindowView(res, i)
                    batches.append({"windows": len(batch), "kernel_ms": res.kernel_ms, "call_s": res.elapsed_s,
                                    "batched": int(res.batched.sum()), "launches": res.launches})
                except SgfimError as e:
                    for rq in batch:
                        rq.error = str(e)
                t_done = time.perf_counter() - t0
                for rq in batch:
                    rq.done_s = t_done
                with lock:
                    done.extend(batch)

        target = scheduler if self.mode == "batched" else worker
        threads = [threading.Thread(target=target, args=(e,), daemon=True) for e in self.engines]
        for t in threads:
            t.start()
        disp = threading.Thread(target=dispatcher, daemon=True)
        disp.start()
        disp.join()
        for t in threads:
            t.join()
        wall = time.perf_counter() - t0
        lat = np.array([r.done_s - r.arrival for r in done])
        errors = [r for r in done if r.error]
        first, last = min(r.arrival for r in requests), max(r.done_s for r in done)
        mine = np.array([r.mine_s for r in done if not r.error] or [0.0])
        queue = np.array([r.start_s - r.arrival for r in done])
        extra = {}
        if batches:
            extra = {"batches": len(batches), "batch_windows_mean": float(np.mean([b["windows"] for b in batches])),
                     "kernel_ms_total": float(sum(b["kernel_ms"] for b in batches)),
                     "call_s_total": float(sum(b["call_s"] for b in batches)),
                     "batched_windows": int(sum(b["batched"] for b in batches))}
        return {"mode": self.mode, **extra, "windows": len(done), "errors": len(errors), "wall_s": wall,
                "mine_ms_p50": float(np.percentile(mine, 50) * 1e3), "mine_ms_p99": float(np.percentile(mine, 99) * 1e3),
                "mine_s_total": float(mine.sum()), "queue_ms_p50": float(np.percentile(queue, 50) * 1e3),
                "nodes_total": int(sum(r.nodes for r in done)),
                "windows_per_s": len(done) / max(last - first, 1e-9),
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "max_ms": float(lat.max() * 1e3),
                "mfis_total": int(sum(r.n_mfis for r in done)), "requests": done}


def stream_rows_for(n_req=WORKLOAD["n_req"], rate_hz=WORKLOAD["rate_hz"], stream_rate=WORKLOAD["stream_rate"],
                    seed=0):
    duration = n_req / rate_hz * 1.5 + 1.0
    n = WORKLOAD["len_hi"] + int(stream_rate * duration)
    return datagen.regime_txns(n, WORKLOAD["n_sensors"], WORKLOAD["n_bins"], WORKLOAD["n_regimes"],
                               WORKLOAD["alpha_bin"], seed=seed)


def saturate(rows, reqs, repeat, horizontal=False, hbm_budget=32 << 30, out=""):
    """Every request's window (as the service would cut it) in one batched call."""
    import json
    rp, it = datagen.txns_to_csr(rows)
    eng = Engine(hbm_budget=hbm_budget, windows_horizontal=horizontal)
    ring = Ring(126, WORKLOAD["ring_txn"])
    try:
        ring.append(rp, it)
        total, warm = len(rows), WORKLOAD["len_hi"]
        ends = np.array([min(total, warm + int(WORKLOAD["stream_rate"] * rq.arrival)) for rq in reqs], np.int64)
        lens = np.minimum(np.array([rq.length for rq in reqs], np.int64), ends)
        thrs = np.maximum(1, np.ceil(WORKLOAD["floor_frac"] * lens)).astype(np.int64)
        reps = []
        for _ in range(repeat):
            t = time.perf_counter()
            res = ring.mine_windows(eng, ends - lens, lens, thrs)
            dt = time.perf_counter() - t
            reps.append({"call_s": dt, "kernel_ms": res.kernel_ms, "task_kernel_ms": res.task_kernel_ms,
                         "task_ms_max": res.task_ms_max, "warps": res.warps, "tasks": res.tasks,
                         "warp_busy_ms": res.task_ms_sum / max(1, res.warps), "launches": res.launches,
                         "batched": int(res.batched.sum()), "nodes": int(res.nodes.sum()),
                         "mfis": int(res.offset[-1]), "windows_per_s": len(reqs) / dt,
                         "windows_per_s_kernels": len(reqs) / (res.kernel_ms / 1e3)})
            del res
        report = {"workload": "windows-4096 (all windows in one call)", "windows": len(reqs),
                  "mode": "horizontal" if horizontal else "vertical", "runs": reps}
        print(json.dumps(report))
        if out:
            with open(out, "w") as f:
                json.dump(report, f, indent=1)
        return report
    finally:
        ring.close()
        eng.close()


def run_workload(n_requests=WORKLOAD["n_req"], rate=WORKLOAD["rate_hz"], mode="batched", schedulers=2, workers=16,
                 hbm_budget_gb=32.0, keep_results=False):
    """The windows-4096 workload in real time (a warm-up pass first).  Returns
    (report, completed requests, stream rows)."""
    rows = stream_rows_for(n_requests, rate_hz=rate)
    reqs = make_requests(n_requests, rate, WORKLOAD["len_lo"], WORKLOAD["len_hi"], seed=1)
    svc = WindowService(workers=workers, hbm_budget=int(hbm_budget_gb * (1 << 30)), keep_results=keep_results,
                        mode=mode, schedulers=schedulers)
    try:
        # warm-up pass on a handful of requests (first-use allocations of every handle)
        warm = make_requests(2 * workers, 4000.0, WORKLOAD["len_lo"], WORKLOAD["len_hi"], seed=99)
        svc.run(rows, warm, WORKLOAD["stream_rate"], WORKLOAD["floor_frac"])
        svc.ring.close()
        svc.ring = Ring(126, WORKLOAD["ring_txn"])
        rep = svc.run(rows, reqs, WORKLOAD["stream_rate"], WORKLOAD["floor_frac"])
    finally:
        svc.close()
    done = rep.pop("requests")
    errs = {}
    for rq in done:
        if rq.error:
            errs[rq.error] = errs.get(rq.error, 0) + 1
    report = {"workload": "windows-4096", "requests": n_requests, "rate_hz": rate,
              "workers": workers if mode == "workers" else schedulers,
              "hbm_budget_gb": hbm_budget_gb, **rep, "error_kinds": errs,
              "config": {k: WORKLOAD[k] for k in WORKLOAD}}
    return report, done, rows


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="sliding-window MFI service, workload windows-4096")
    ap.add_argument("--requests", type=int, default=WORKLOAD["n_req"])
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--mode", choices=("batched", "workers"), default="batched")
    ap.add_argument("--schedulers", type=int, default=2,
                    help="batched mode: concurrent batches (a handle and a thread each); measured at "
                         "2,000 req/s: 1 -> p50 36.9 / p99 56.2 ms, 2 -> 32.9 / 52.5 ms, 3 -> 35.5 / 59.3 ms")
    ap.add_argument("--hbm-budget-gb", type=float, default=32.0)
    ap.add_argument("--out", default="")
    ap.add_argument("--saturate", type=int, default=0, metavar="REPEAT",
                    help="instead of the timed service, mine every request's window in one "
                         "sgfim_ring_mine_windows call, REPEAT times (capacity of the batched miner)")
    ap.add_argument("--horizontal", action="store_true", help="batched miner on horizontal masks")
    ap.add_argument("--rate", type=float, default=WORKLOAD["rate_hz"],
                    help="Poisson arrival rate of the requests (req/s); the workload's is 2,000")
    a = ap.parse_args(argv)
    if a.saturate:
        rows = stream_rows_for(a.requests, rate_hz=a.rate)
        reqs = make_requests(a.requests, a.rate, WORKLOAD["len_lo"], WORKLOAD["len_hi"], seed=1)
        return saturate(rows, reqs, a.saturate, a.horizontal, int(a.hbm_budget_gb * (1 << 30)), a.out)
    report, _, _ = run_workload(a.requests, a.rate, a.mode, a.schedulers, a.workers, a.hbm_budget_gb)
    print(json.dumps(report))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
    return report


if __name__ == "__main__":
    main()
