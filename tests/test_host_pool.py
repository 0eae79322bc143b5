"""The miner's host thread pool (csrc/host_pool.h) on the CPU: a small C++
program built against the header runs thousands of jobs of random sizes and
chunkings, with pauses long enough for the threads to fall asleep between
some of them, and checks that every index of every job is visited exactly
once; pools of one thread run serially; pools are created and destroyed
repeatedly.  A hang (a lost wake-up) shows up as the subprocess timeout."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "20261008-self-growing-evidence-agent_gb300", "csrc")

PROGRAM = r"""
#include <atomic>
#include <chrono>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>
#include "host_pool.h"

static int check(sg::HostPool &pool, std::mt19937_64 &rng, int jobs, bool pauses) {
    std::vector<std::atomic<uint32_t>> hit(200000);
    for (int j = 0; j < jobs; ++j) {
        const uint64_t n = rng() % 200000, chunk = 1 + rng() % 5000;
        for (uint64_t i = 0; i < n; ++i) hit[i].store(0, std::memory_order_relaxed);
        std::atomic<uint64_t> sum{0};
        pool.run(n, chunk, [&](uint64_t lo, uint64_t hi) {
            uint64_t s = 0;
            for (uint64_t i = lo; i < hi; ++i) { hit[i].fetch_add(1, std::memory_order_relaxed); s += i; }
            sum.fetch_add(s, std::memory_order_relaxed);
        });
        for (uint64_t i = 0; i < n; ++i)
            if (hit[i].load() != 1) { std::printf("job %d: index %llu visited %u times\n", j, (unsigned long long)i, hit[i].load()); return 1; }
        if (sum.load() != (n ? n * (n - 1) / 2 : 0)) { std::printf("job %d: wrong sum\n", j); return 1; }
        if (pauses && j % 50 == 0) std::this_thread::sleep_for(std::chrono::milliseconds(2));
    }
    return 0;
}

int main() {
    std::mt19937_64 rng(7);
    { sg::HostPool pool(8); if (check(pool, rng, 3000, true)) return 1; }
    { sg::HostPool pool(1); if (check(pool, rng, 200, false)) return 1; }
    for (int k = 0; k < 50; ++k) {   // short-lived pools, some never started
        sg::HostPool pool(2 + k % 7);
        if (k % 3 && check(pool, rng, 5, k % 2)) return 1;
    }
    std::printf("ok\n");
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_host_pool_visits_every_index_once(tmp_path):
    src = tmp_path / "pool_test.cpp"
    exe = tmp_path / "pool_test"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", f"-I{CSRC}", str(src), "-o", str(exe)], check=True,
                   timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
