#!/usr/bin/env python
"""Benchmark of the batched support-counting path on one or more GPUs.

Workload "support-1m": 1,048,576 transactions x 1,024 items as vertical
bitmaps (per-item density log-uniform in [2%, 20%], correlated through 16
latent regimes) and 1,000,000 candidate itemsets of size k ~ U{3..8} grown by
random walks over co-occurring item pairs; a step counts the exact support of
every candidate.  The data are synthetic and seeded (the reference's datasets
are not shipped).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  ``value`` is supports/s with inputs resident
in HBM (CUDA events on the launching stream, L2 flushed by a 512 MiB write
before every step); ``e2e`` is the same metric through the C ABI with pinned
host buffers (bitmaps and candidates copied in, supports copied out, every
step); ``roofline`` relates the counting kernel's algorithmic bytes
(k * N / 8 per candidate) to the measured HBM copy bandwidth; ``cpu_baseline``
times the CPU oracle (a restatement of the reference's counting loop,
kernel_bitmap.cu:390-408) on a bounded sample with every host core.
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

WORKLOAD = dict(name="support-1m", n_txn=1 << 20, d=1024, n_regimes=16, dens_lo=0.02, dens_hi=0.20,
                n_cand=1_000_000, kmin=3, kmax=8)
METRIC = "supports/s (frac of HBM peak)"
UNIT = "supports/s"


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
    ap.add_argument("--kernel", choices=["auto", "lane", "sorted", "staged", "staged4", "stream"], default="auto")
    ap.add_argument("--workload", choices=["support-1m", "transact-1m"], default="support-1m",
                    help="transact-1m: the sensor-stream front end (quantile and online P2 "
                         "transactionisation of 1M-row streams) instead of the support bench")
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
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


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


def cpu_baseline(bm, cp, ci, budget_s=10.0):
    """The CPU oracle on a bounded sample of the candidates, every host core."""
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


def run_reference(args, rank, world):
    """--impl reference: the CPU counting loop on the host cores (rank 0 only)."""
    if rank != 0:
        return
    import oracle
    bm, cp, ci = make_workload(0, args.n_cand)
    threads = os.cpu_count() or 1
    n0 = min(2000, len(cp) - 1)
    t = time.perf_counter()
    oracle.support_batch(bm, cp[:n0 + 1], ci[:int(cp[n0])], n_threads=threads)
    rate = n0 / max(time.perf_counter() - t, 1e-6)
    per_step = int(min(len(cp) - 1, max(n0, rate * 1.0)))   # ~1 s of work per step
    times = []
    for s in range(args.warmup + args.steps):
        lo = (s * per_step) % max(1, (len(cp) - 1 - per_step))
        sp = cp[lo:lo + per_step + 1] - cp[lo]
        si = ci[int(cp[lo]):int(cp[lo + per_step])]
        t = time.perf_counter()
        oracle.support_batch(bm, sp, si, n_threads=threads)
        if s >= args.warmup:
            times.append(time.perf_counter() - t)
    ms = 1000.0 * sum(times) / len(times)
    value = per_step / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD["name"], "n_txn": WORKLOAD["n_txn"], "items": WORKLOAD["d"],
                       "candidates": len(cp) - 1, "k": "3..8", "step_sample": per_step,
                       "l2": "host run"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{per_step} candidates per step, C oracle, {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "transact-1m":
        return run_transact(args, rank)
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

    bm, cp, ci = make_workload(rank, args.n_cand)
    n_cand = len(cp) - 1
    d, w = bm.shape
    eng = Engine(device=local, phase_timers=True)
    eng.set_support_plan(args.kernel)
    t_bm = torch.from_numpy(bm.view(np.int64)).to(dev)
    t_cp = torch.from_numpy(cp.view(np.int64)).to(dev)
    t_ci = torch.from_numpy(ci.view(np.int32)).to(dev)
    t_out = torch.zeros(n_cand, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        eng.support_batch_device(t_bm.data_ptr(), d, w, w, t_cp.data_ptr(), t_ci.data_ptr(), n_cand,
                                 t_out.data_ptr(), stream.cuda_stream)

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
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ps = eng.phase_stats(reset=True)
    ms = sum(step_ms) / len(step_ms)
    if dist:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    value = world * n_cand / (ms / 1000.0)

    # roofline of the counting kernel
    k = np.diff(cp).astype(np.int64)
    alg_bytes = float(k.sum()) * (WORKLOAD["n_txn"] / 8.0)
    count_ms = ps["count_ms"] / max(1, ps["calls"])
    peaks, peak_src = measured_peaks()
    achieved = alg_bytes / (count_ms / 1000.0) / 1e9
    kname = {"auto": "k1_staged4_kernel", "sorted": "k1_sorted_kernel", "staged": "k1_staged_kernel",
             "staged4": "k1_staged4_kernel",
             "stream": "query_kernel"}[args.kernel]
    tr = ncu_traffic(kname.replace("_kernel", ""))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peak_src,
                "traffic": (tr["dram_bytes_per_launch"] if tr else None),
                "kernel": kname, "kernel_ms": count_ms, "alg_bytes_per_launch": alg_bytes}

    # end to end through the host C ABI with pinned buffers
    e2e = None
    if args.e2e_steps > 0:
        pin_bm = torch.from_numpy(bm.view(np.int64)).pin_memory().numpy().view(np.uint64)
        pin_cp = torch.from_numpy(cp.view(np.int64)).pin_memory().numpy().view(np.uint64)
        pin_ci = torch.from_numpy(ci.view(np.int32)).pin_memory().numpy().view(np.uint32)
        pin_out = torch.zeros(n_cand, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
        host = Engine(device=local)
        e_times = []
        for s in range(1 + args.e2e_steps):
            t0 = time.perf_counter()
            host.load_bitmaps(pin_bm, WORKLOAD["n_txn"])
            sup = host.support_batch(pin_cp, pin_ci, out=pin_out)
            dt = time.perf_counter() - t0
            if s > 0:
                e_times.append(dt)
        host.close()
        e_ms = 1000.0 * sum(e_times) / len(e_times)
        gpu_sup = t_out.cpu().numpy().view(np.uint32)
        assert np.array_equal(sup, gpu_sup), "host and device entry points disagree"
        e2e = {"value": n_cand / (e_ms / 1000.0) * world, "unit": UNIT,
               "h2d_bytes_per_step": int(bm.nbytes + cp.nbytes + ci.nbytes),
               "d2h_bytes_per_step": int(4 * n_cand), "ms_per_step": e_ms,
               "note": "sgfim_load_bitmaps + sgfim_support_batch per step, pinned host buffers"}

    # the 1,024 x 1,024 co-occurrence matrix of the same bitmaps (both kernel kinds)
    cooc = {}
    if not args.no_cooc:
        t_co = {k: torch.zeros(d * d, dtype=torch.int32, device=dev) for k in (1, 2, 3)}
        for kind, name in ((1, "popc"), (2, "bmma_b1"), (3, "tcgen05_e4m3")):
            for _ in range(2):
                eng.cooccurrence_device(t_bm.data_ptr(), d, w, w, t_co[kind].data_ptr(), kind, stream.cuda_stream)
            times = []
            for _ in range(5):
                flush.fill_(1)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                eng.cooccurrence_device(t_bm.data_ptr(), d, w, w, t_co[kind].data_ptr(), kind, stream.cuda_stream)
                b.record(stream)
                torch.cuda.synchronize()
                times.append(a.elapsed_time(b))
            ms_c = statistics.median(times)
            bitops = float(d) * d * WORKLOAD["n_txn"]
            cooc[name] = {"ms": ms_c, "tbitops": bitops / (ms_c / 1000.0) / 1e12}
        cooc["kinds_agree"] = bool(torch.equal(t_co[1], t_co[2]) and torch.equal(t_co[1], t_co[3]))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, sup_cpu, n_s = cpu_baseline(bm, cp, ci)
        cpu["sample_match"] = bool(np.array_equal(sup_cpu, t_out.cpu().numpy().view(np.uint32)[:n_s]))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD["name"], "n_txn": WORKLOAD["n_txn"], "items": WORKLOAD["d"],
                           "candidates_per_gpu": n_cand, "k": "3..8", "bitmap_bytes": int(bm.nbytes),
                           "l2": "flushed (512 MiB write) before every step",
                           "parallelism": f"candidate shards x{world}, no collective on the data path"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "cooccurrence_1024": cooc,
                "gpu_launches": int(ps["launches"]), "clocks": clk.summary(),
                "wall_s_timed": wall}
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
