#!/usr/bin/env python
"""Benchmark of the batched support-counting path, plus the mining workloads.

Workload "support-1m" (the default line): 1,048,576 transactions x 1,024 items
as vertical bitmaps (per-item density log-uniform in [2%, 20%], correlated
through 16 latent regimes) and 1,000,000 candidate itemsets of size
k ~ U{3..8} grown by random walks over co-occurring item pairs; a step counts
the exact support of every candidate.  The data are synthetic and seeded (the
reference's datasets are not shipped).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload support-1m|anytime-2m|windows-4096|learned-order|transact-1m]

Prints one JSON line (rank 0).  ``value`` is supports/s with inputs resident
in HBM (CUDA events on the launching stream, L2 flushed by a 512 MiB write
before every step); ``e2e`` is the same metric through the C ABI with pinned
host buffers (bitmaps and candidates copied in, supports copied out, every
step).  ``roofline`` relates the counting kernel's algorithmic bytes (k * N / 8
per candidate, all read from shared memory once TMA has staged a chunk) to the
shared-memory bandwidth (SMs x 128 B/clk x the SM clock sampled during the
timed region); the HBM ratio and the DRAM traffic are kept beside it.
``cpu_baseline`` times the CPU oracle (a restatement of the reference's
counting loop, kernel_bitmap.cu:390-408) on every host core;
``cpu_baseline_numpy`` times the reference's numpy AND + byte-LUT popcount
(exp_e6_cpuvec.py:43,86) on one core.  ``configs`` carries the other
workloads' headline numbers (anytime-2m coverage, the windows-4096 service,
the learned frontier order), each also available as its own ``--workload``.

With N > 1 ranks the transactions are split (sgfim.sharding): every rank
keeps 1/N of each bitmap row, counts partial supports of the one shared
candidate set and an int32 sum all-reduce completes them.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from sgfim import datagen  # noqa: E402
from sgfim import sharding  # noqa: E402

WORKLOAD = dict(name="support-1m", n_txn=1 << 20, d=1024, n_regimes=16, dens_lo=0.02, dens_hi=0.20,
                n_cand=1_000_000, kmin=3, kmax=8)
METRIC = "supports/s (frac of HBM peak)"
UNIT = "supports/s"
SMEM_BYTES_PER_CLK = 128        # shared-memory bandwidth of one SM (32 banks x 4 B)
KERNEL_NAMES = {"auto": "k1_lane_tm_kernel", "lane_tm": "k1_lane_tm_kernel", "lane": "k1_lane_kernel",
                "sorted": "k1_sorted_kernel", "staged": "k1_staged_kernel", "staged4": "k1_staged4_kernel",
                "stream": "query_kernel"}
LEARNED_WEIGHTS = os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300", "sgfim", "data",
                               "scorer_weights.npz")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n-cand", type=int, default=WORKLOAD["n_cand"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cooc", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the anytime, service and learned-order keys")
    ap.add_argument("--kernel", choices=sorted(KERNEL_NAMES), default="auto")
    ap.add_argument("--workload", default="support-1m",
                    choices=["support-1m", "anytime-2m", "windows-4096", "learned-order", "transact-1m"])
    ap.add_argument("--floor", type=float, default=0.03, help="anytime-2m: support floor (fraction)")
    ap.add_argument("--verify", action="store_true",
                    help="anytime-2m: full maximality and greedy-walk completeness checks of the final set; "
                         "windows-4096: every window against the oracle")
    ap.add_argument("--check-budget-s", type=float, default=240.0)
    ap.add_argument("--cpu-budget-s", type=float, default=30.0)
    ap.add_argument("--walks", type=int, default=100_000)
    ap.add_argument("--checkpoints", default="1,2,5,10,30", help="anytime-2m: checkpoint times (s)")
    ap.add_argument("--time-limit", type=float, default=0.0, help="anytime-2m: stop the search after this many s")
    ap.add_argument("--node-limit", type=int, default=0, help="anytime-2m: stop the search after this many nodes")
    ap.add_argument("--seeds", type=int, default=3, help="learned-order: held-out seeds")
    return ap.parse_args()


def make_workload(rank, n_cand):
    bm, model = datagen.correlated_bitmaps(WORKLOAD["n_txn"], WORKLOAD["d"], WORKLOAD["n_regimes"],
                                           WORKLOAD["dens_lo"], WORKLOAD["dens_hi"], seed=0, return_model=True)
    p = model["p"].astype(np.float64)
    expected = WORKLOAD["n_txn"] * ((p.T * model["w"][None, :]) @ p)   # expected pair co-occurrence
    cp, ci = datagen.walk_candidates(n_cand, WORKLOAD["d"], WORKLOAD["kmin"], WORKLOAD["kmax"], seed=1 + rank,
                                     pair_ok=expected >= 1.0)
    return bm, cp, ci


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per launch of the counting kernel from the committed ncu summary
    (a one-pass capture of this workload: dram__bytes_read.sum + dram__bytes_write.sum)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_support-1m.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU arms (oracle = the checker / baseline)
def cpu_baseline(bm, cp, ci, budget_s=10.0):
    """The CPU oracle on the candidates (all of them when they fit the budget), every host core."""
    import oracle
    threads = os.cpu_count() or 1
    n0 = min(2000, len(cp) - 1)
    t = time.perf_counter()
    oracle.support_batch(bm, cp[:n0 + 1], ci[:int(cp[n0])], n_threads=threads)
    rate = n0 / max(time.perf_counter() - t, 1e-6)
    n = int(min(len(cp) - 1, max(n0, rate * budget_s)))
    t = time.perf_counter()
    sup = oracle.support_batch(bm, cp[:n + 1], ci[:int(cp[n])], n_threads=threads)
    dt = time.perf_counter() - t
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {n} of {len(cp) - 1} candidates ({dt:.1f} s, C oracle, {threads} threads)"}, sup, n


def cpu_baseline_numpy(bm, cp, ci, n=2000):
    """The reference's numpy counting (byte view of the bitmaps, AND, 256-entry
    popcount table, exp_e6_cpuvec.py:43,86) on the first ``n`` candidates, one core."""
    from oracle import numpy_lut
    t = time.perf_counter()
    sup = numpy_lut.supports(bm, cp[:n + 1], ci[:int(cp[n])])
    dt = time.perf_counter() - t
    return {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {n} of {len(cp) - 1} candidates, numpy AND + byte-LUT popcount, "
                      f"1 thread, {dt:.2f} s (rate extrapolated to the whole set)"}, sup


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU counting loop (kernel_bitmap.cu:390-408, as
    restated by the C oracle) on every host core, all candidates per timed step; rank 0 only."""
    if rank != 0:
        return
    import oracle
    bm, cp, ci = make_workload(0, args.n_cand)
    threads = os.cpu_count() or 1
    n = len(cp) - 1
    warm = min(n, 20_000)
    for _ in range(args.warmup):   # untimed: a slice warms the caches and the thread pool
        oracle.support_batch(bm, cp[:warm + 1], ci[:int(cp[warm])], n_threads=threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.support_batch(bm, cp, ci, n_threads=threads)
        times.append(time.perf_counter() - t)
    ms = 1000.0 * sum(times) / len(times)
    value = n / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD["name"], "n_txn": WORKLOAD["n_txn"], "items": WORKLOAD["d"],
                       "candidates": n, "k": "3..8", "l2": "host run"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"all {n} candidates per step, C oracle, {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- other workloads
TRANSACT_STREAMS = [(1_000_000, 8, 3), (1_000_000, 21, 6)]   # rows, sensors, bins; window 30, stride 15


def run_transact(args, rank):
    """--workload transact-1m: sgfim_transactionize and sgfim_transactionize_online
    on seeded 1M-row streams (host values in, items/edges out, every call
    timed whole), beside the C restatement of the online discretiser on every
    host core and on one.  Prints one JSON line per stream (rank 0)."""
    if rank != 0:
        return
    import oracle
    from sgfim.engine import Engine
    threads = os.cpu_count() or 1
    with Engine() as eng:
        for n, S, nb in TRANSACT_STREAMS:
            vals, anom = datagen.sensor_stream(n, S, 5)
            for _ in range(max(1, args.warmup)):
                eng.transactionize(vals[:100_000], 30, 15, nb, anomaly=anom[:100_000])
                eng.transactionize_online(vals[:20_000], 30, 15, nb, anomaly=anom[:20_000])
            t_off, t_on = [], []
            for _ in range(max(1, min(args.steps, 3))):
                t = time.perf_counter()
                eng.transactionize(vals, 30, 15, nb, anomaly=anom)
                t_off.append(time.perf_counter() - t)
                t = time.perf_counter()
                items, labels, edges = eng.transactionize_online(vals, 30, 15, nb, anomaly=anom)
                t_on.append(time.perf_counter() - t)
            t = time.perf_counter()
            w_edges, w_items, _ = oracle.online_bins(vals, 30, 15, nb, anom, n_threads=threads)
            c_all = time.perf_counter() - t
            t = time.perf_counter()
            oracle.online_bins(vals, 30, 15, nb, anom, n_threads=1)
            c_one = time.perf_counter() - t
            same = bool(np.array_equal(items, w_items) and np.array_equal(edges.view(np.int64), w_edges.view(np.int64)))
            on_s = min(t_on)
            line = {"metric": "rows/s (online P2 transactionisation)", "value": n / on_s, "unit": "rows/s",
                    "n_gpus": 1, "steps": len(t_on), "warmup": args.warmup, "ms_per_step": 1000 * on_s,
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic (seeded sensor stream)",
                    "config": {"workload": "transact-1m", "rows": n, "sensors": S, "bins": nb, "window": 30,
                               "stride": 15, "windows": int(items.shape[0])},
                    "offline_quantile_call_s": min(t_off), "online_call_s": on_s, "matches_c_oracle": same,
                    "cpu_baseline": {"value": n / c_all, "unit": "rows/s", "cores": threads, "kind": "port",
                                     "sample": f"whole stream, C restatement, {threads} threads ({c_all:.2f} s; "
                                               f"1 thread {c_one:.2f} s)"},
                    "e2e": {"value": n / on_s, "unit": "rows/s", "h2d_bytes_per_step": int(vals.nbytes + anom.nbytes),
                            "d2h_bytes_per_step": int(items.size * 4 + labels.size * 4 + edges.nbytes)},
                    "gpu_launches": 3}
            print(json.dumps(line), flush=True)


def anytime_report(floor=0.03, verify=False, walks=100_000, seed=0, checkpoints=(1, 2, 5, 10, 30), time_limit_s=0.0,
                   node_limit=0):
    """anytime-2m: coverage at the checkpoints, time to 50/90/95/100% and (with
    ``verify``) checks of the final set that do not reuse the miner's search:
    every support recounted, antichain, every single-item extension of every
    MFI counted (sgfim_frequent_extensions), greedy maximal walks that must all
    land in the set, and an oracle recount of a sample of supports."""
    from sgfim import anytime_run
    from sgfim.engine import Engine
    t0 = time.perf_counter()
    rows = anytime_run.workload_rows(seed=seed)
    t_gen = time.perf_counter() - t0
    with Engine() as eng:
        rep, res = anytime_run.run(eng, rows, floor, checkpoints, time_limit_s=time_limit_s, node_limit=node_limit)
        rep["gen_s"] = t_gen
        if verify and res is not None:
            from sgfim import verify as V
            rep["verify"] = V.check_mfi_set(eng, res, rep["min_count"], walks=walks, seed=seed)
            rep["verify"]["oracle_sample_supports_equal"] = _oracle_sample(rows, res, anytime_run.ITEMS)
    return rep


def _oracle_sample(rows, res, d, sample=2000, seed=0):
    import oracle
    cp, ci, sup = res.ptr.astype(np.uint64), res.items.astype(np.uint32), res.support
    if len(sup) == 0:
        return True
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, d)
    pick = np.sort(np.random.default_rng(seed).choice(len(sup), min(sample, len(sup)), replace=False))
    k = (cp[1:] - cp[:-1])[pick]
    sp = np.zeros(len(pick) + 1, np.uint64)
    sp[1:] = np.cumsum(k)
    si = np.concatenate([ci[cp[i]:cp[i + 1]] for i in pick])
    return bool(np.array_equal(oracle.support_batch(bm, sp, si), sup[pick]))


_ROWS = None


def _pool_init(rows):
    global _ROWS
    _ROWS = rows


def _check_window(args):
    """Oracle MFIs of one window (runs in a spawned worker process)."""
    import oracle
    end, length, thr = args
    rows = _ROWS[end - length:end]
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, 126)
    res, _ = oracle.mine_fast(bm, length, thr)
    return sorted((tuple(s), c) for s, c in res)


def _cpu_window(args):
    """The reference's miner restated (mine_mfi with its 200,000-node cap) on one window."""
    import oracle
    end, length, thr = args
    rows = _ROWS[end - length:end]
    rp, it = datagen.txns_to_csr(rows)
    bm, _ = oracle.build_bitmaps(rp, it, 126)
    t = time.perf_counter()
    try:
        oracle.mine_mfi(bm, length, min_count=thr, node_cap=200_000)
        ok = True
    except RuntimeError:
        ok = False
    return ok, time.perf_counter() - t


def windows_report(check=False, check_budget_s=240.0, cpu_budget_s=0.0):
    """windows-4096 at 2,000 req/s (sgfim.service), optionally with every window
    compared with the oracle and the reference's miner timed on the host cores."""
    import multiprocessing as mp
    from sgfim import service
    report, done, rows = service.run_workload(keep_results=check)
    ctx = mp.get_context("spawn")
    procs = os.cpu_count() or 1
    ff = service.WORKLOAD["floor_frac"]
    jobs = [(rq.end, min(rq.length, rq.end), max(1, int(np.ceil(ff * min(rq.length, rq.end))))) for rq in done]
    if check:
        t0 = time.perf_counter()
        checked = mism = 0
        with ctx.Pool(procs, initializer=_pool_init, initargs=(rows,)) as pool:
            for rq, ref in zip(done, pool.imap(_check_window, jobs, chunksize=4)):
                if rq.result is None:
                    continue
                got = sorted((tuple(sorted(s)), c) for s, c in rq.result.sets())
                checked += 1
                mism += got != ref
                if time.perf_counter() - t0 > check_budget_s:
                    pool.terminate()
                    break
        report["exact"] = {"checked": checked, "mismatches": mism}
    if cpu_budget_s > 0:
        t0 = time.perf_counter()
        n_ok = n_cap = 0
        with ctx.Pool(procs, initializer=_pool_init, initargs=(rows,)) as pool:
            for ok, _ in pool.imap(_cpu_window, jobs, chunksize=1):
                n_ok += ok
                n_cap += not ok
                if time.perf_counter() - t0 > cpu_budget_s:
                    pool.terminate()
                    break
        wall = time.perf_counter() - t0
        report["cpu_baseline"] = {"windows": n_ok + n_cap, "completed": n_ok, "node_cap_hit": n_cap,
                                  "windows_per_s": (n_ok + n_cap) / wall, "cores": procs, "kind": "port",
                                  "sample": f"first {n_ok + n_cap} windows in arrival order within "
                                            f"{cpu_budget_s:.0f} s, mine_mfi restated with its 200,000-node cap"}
    report.pop("config", None)
    return report


def learned_report(n_seeds=3):
    """Held-out streams of the anytime-2m family: time to 50/90/95% coverage with
    the learned order against support-descending, with the committed scorer."""
    if not os.path.exists(LEARNED_WEIGHTS):
        return {"unavailable": "no committed scorer weights"}
    from sgfim import learned_order
    return learned_order.evaluate_committed(LEARNED_WEIGHTS, n_seeds)


def run_single(args, rank):
    """--workload anytime-2m | windows-4096 | learned-order: one JSON line (rank 0)."""
    if rank != 0:
        return
    if args.workload == "anytime-2m":
        t0 = time.perf_counter()
        rep = anytime_report(args.floor, args.verify, args.walks,
                             checkpoints=[float(x) for x in args.checkpoints.split(",") if x],
                             time_limit_s=args.time_limit, node_limit=args.node_limit)
        rep["verify_s"] = time.perf_counter() - t0 - rep.get("gen_s", 0) - rep.get("load_s", 0) - rep.get("mine_s", 0)
        line = {"metric": "MFI coverage at wall-clock checkpoints",
                "value": rep["time_to"]["95%"] if rep.get("complete") else None,
                "unit": "s to 95% coverage", "higher_is_better": False, **rep}
    elif args.workload == "windows-4096":
        rep = windows_report(args.verify, args.check_budget_s, args.cpu_budget_s)
        line = {"metric": "windows/s and p50/p99 latency at 2,000 req/s", "value": rep["windows_per_s"],
                "unit": "windows/s", "higher_is_better": True, **rep}
    else:
        rep = learned_report(args.seeds)
        line = {"metric": "time to 95% coverage, learned / support-descending", "unit": "ratio",
                "higher_is_better": False, **rep}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- support-1m
def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "transact-1m":
        return run_transact(args, rank)
    if args.workload != "support-1m":
        return run_single(args, rank)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    from sgfim.engine import Engine

    # one shared candidate set; rank r keeps its slice of the transactions
    bm, cp, ci = make_workload(0, args.n_cand)
    n_cand = len(cp) - 1
    d, n_words = bm.shape
    w0, w1 = sharding.txn_shard(n_words, rank, world)
    bm_r = sharding.row_slice(bm, w0, w1) if world > 1 else bm
    wr = w1 - w0
    eng = Engine(device=local, phase_timers=True)
    eng.set_support_plan(args.kernel)
    t_bm = torch.from_numpy(bm_r.view(np.int64)).to(dev)
    t_cp = torch.from_numpy(cp.view(np.int64)).to(dev)
    t_ci = torch.from_numpy(ci.view(np.int32)).to(dev)
    t_out = torch.zeros(n_cand, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        eng.support_batch_device(t_bm.data_ptr(), d, wr, bm_r.shape[1], t_cp.data_ptr(), t_ci.data_ptr(), n_cand,
                                 t_out.data_ptr(), stream.cuda_stream)
        sharding.allreduce_counts(t_out, dist)

    for _ in range(args.warmup):
        flush.fill_(1)
        step()
    torch.cuda.synchronize()
    eng.phase_stats(reset=True)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for a, b in evs:
            flush.fill_(1)
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if dist:
        dist.barrier()
    assert eng.device_status(stream.cuda_stream) == 0, "a bounded device wait ran out"
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ps = eng.phase_stats(reset=True)
    ms = sum(step_ms) / len(step_ms)
    if dist:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    value = n_cand / (ms / 1000.0)   # the whole job counts the one candidate set
    clocks = clk.summary()

    # roofline of the counting kernel: algorithmic bytes of this rank's slice
    peaks, peak_src = measured_peaks()
    k = np.diff(cp).astype(np.int64)
    alg_bytes = float(k.sum()) * (wr * 64 / 8.0)
    count_ms = ps["count_ms"] / max(1, ps["calls"])
    achieved = alg_bytes / (count_ms / 1000.0) / 1e9
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clocks["sm_mhz"] or peaks.get("sm_max_mhz", 2070.0)
    smem_peak = n_sm * SMEM_BYTES_PER_CLK * sm_mhz * 1e6 / 1e9
    kname = KERNEL_NAMES[args.kernel]
    tr = ncu_traffic(kname.replace("_kernel", ""))
    traffic = tr["dram_bytes_per_launch"] if tr else None
    roofline = {"bound": "smem", "achieved": achieved, "peak": smem_peak, "unit": "GB/s", "frac": achieved / smem_peak,
                "traffic": traffic,
                "peak_source": f"{n_sm} SMs x {SMEM_BYTES_PER_CLK} B/clk x {sm_mhz:.0f} MHz "
                               f"({'median SM clock sampled in the timed region' if clocks['sm_mhz'] else 'max SM clock'})",
                "kernel": kname, "kernel_ms": count_ms, "alg_bytes_per_launch": alg_bytes,
                "hbm": {"peak_gbs": peaks["hbm_gbs"], "peak_source": peak_src,
                        "alg_bytes_over_hbm_peak": achieved / peaks["hbm_gbs"],
                        "dram_traffic_gbs": (traffic / (count_ms / 1000.0) / 1e9) if traffic else None,
                        "dram_frac": (traffic / (count_ms / 1000.0) / 1e9 / peaks["hbm_gbs"]) if traffic else None,
                        "note": "each staged chunk is read from shared memory by every candidate that holds one "
                                "of its rows; DRAM sees the bitmaps about once per CTA wave"}}

    # end to end through the host C ABI with pinned buffers (the rank's slice)
    e2e = None
    if args.e2e_steps > 0:
        pin_bm = torch.from_numpy(bm_r.view(np.int64)).pin_memory().numpy().view(np.uint64)
        pin_cp = torch.from_numpy(cp.view(np.int64)).pin_memory().numpy().view(np.uint64)
        pin_ci = torch.from_numpy(ci.view(np.int32)).pin_memory().numpy().view(np.uint32)
        pin_out = torch.zeros(n_cand, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
        host = Engine(device=local)
        e_times = []
        for s in range(1 + args.e2e_steps):
            t0 = time.perf_counter()
            host.load_bitmaps(pin_bm, wr * 64)
            sup = host.support_batch(pin_cp, pin_ci, out=pin_out)
            if dist:
                t_sup = torch.from_numpy(sup.view(np.int32)).to(dev)
                sharding.allreduce_counts(t_sup, dist)
                sup = t_sup.cpu().numpy().view(np.uint32)
            dt = time.perf_counter() - t0
            if s > 0:
                e_times.append(dt)
        host.close()
        e_ms = 1000.0 * sum(e_times) / len(e_times)
        if dist:
            tt = torch.tensor([e_ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e_ms = float(tt.item())
        gpu_sup = t_out.cpu().numpy().view(np.uint32)
        assert np.array_equal(sup, gpu_sup), "host and device entry points disagree"
        e2e = {"value": n_cand / (e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(bm_r.nbytes + cp.nbytes + ci.nbytes),
               "d2h_bytes_per_step": int(4 * n_cand), "ms_per_step": e_ms,
               "note": "sgfim_load_bitmaps + sgfim_support_batch per step, pinned host buffers"}

    # the 1,024 x 1,024 co-occurrence matrix of the same bitmaps (every kernel kind)
    cooc = {}
    if not args.no_cooc and world == 1:
        t_co = {k: torch.zeros(d * d, dtype=torch.int32, device=dev) for k in (1, 2, 3, 4)}
        for kind, name in ((1, "popc"), (2, "bmma_b1"), (3, "tcgen05_e4m3"), (4, "tcgen05_e4m3_256")):
            for _ in range(2):
                eng.cooccurrence_device(t_bm.data_ptr(), d, n_words, n_words, t_co[kind].data_ptr(), kind,
                                        stream.cuda_stream)
            times = []
            for _ in range(5):
                flush.fill_(1)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                eng.cooccurrence_device(t_bm.data_ptr(), d, n_words, n_words, t_co[kind].data_ptr(), kind,
                                        stream.cuda_stream)
                b.record(stream)
                torch.cuda.synchronize()
                times.append(a.elapsed_time(b))
            ms_c = statistics.median(times)
            bitops = float(d) * d * WORKLOAD["n_txn"]
            cooc[name] = {"ms": ms_c, "tbitops": bitops / (ms_c / 1000.0) / 1e12}
        cooc["kinds_agree"] = bool(all(torch.equal(t_co[1], t_co[k]) for k in (2, 3, 4)))

    cpu = cpu_np = None
    gpu_sup = t_out.cpu().numpy().view(np.uint32)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, sup_cpu, n_s = cpu_baseline(bm, cp, ci)
        cpu["sample_match"] = bool(np.array_equal(sup_cpu, gpu_sup[:n_s]))
        cpu_np, sup_np = cpu_baseline_numpy(bm, cp, ci)
        cpu_np["sample_match"] = bool(np.array_equal(sup_np, gpu_sup[:len(sup_np)]))
    eng.close()

    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        configs = {}
        for key, fn in (("anytime_2m", lambda: anytime_report(0.03)),
                        ("windows_4096", lambda: windows_report()),
                        ("learned_order", lambda: learned_report(args.seeds))):
            try:
                configs[key] = fn()
            except Exception as e:   # a failing side workload must not cost the headline line
                configs[key] = {"error": f"{type(e).__name__}: {e}"}
        aw = configs.get("anytime_2m", {})
        if "checkpoints" in aw:
            configs["anytime_2m"] = {k: aw[k] for k in ("floor", "min_count", "mfis", "nodes", "mine_s", "time_to",
                                                         "gen_s", "load_s")}
            configs["anytime_2m"]["coverage"] = {str(c["t_s"]): c["coverage"] for c in aw["checkpoints"]}
        lw = configs.get("learned_order", {})
        if "summary" in lw:
            configs["learned_order"] = {"n_txn": lw["n_txn"], "floor": lw["floor"], "summary": lw["summary"],
                                        "seeds": [r["seed"] for r in lw["runs"]]}
        ww = configs.get("windows_4096", {})
        if "p50_ms" in ww:
            configs["windows_4096"] = {k: ww[k] for k in ("requests", "rate_hz", "windows", "errors", "p50_ms",
                                                          "p99_ms", "windows_per_s", "wall_s", "mfis_total")}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "strong" if world > 1 else "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "n_txn": WORKLOAD["n_txn"], "items": WORKLOAD["d"],
                           "candidates": n_cand, "k": "3..8", "bitmap_bytes": int(bm.nbytes),
                           "l2": "flushed (512 MiB write) before every step",
                           "parallelism": (f"transaction split x{world}: 1/{world} of every bitmap row per rank, "
                                           f"int32 sum all-reduce of the supports" if world > 1 else "one GPU")},
                "roofline": roofline, "cpu_baseline": cpu, "cpu_baseline_numpy": cpu_np, "e2e": e2e,
                "cooccurrence_1024": cooc, "configs": configs,
                "gpu_launches": int(ps["launches"]), "clocks": clocks, "wall_s_timed": wall}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
