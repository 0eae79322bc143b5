// host_pool.h -- a persistent pool of host threads for the miner's per-node
// bookkeeping between device waves.
//
// run(n, chunk, fn) calls fn(lo, hi) on chunks of [0, n) taken from a shared
// counter by the caller and the pool's threads, and returns when every chunk
// is done.  The threads start on first use.  Between calls they poll for the
// next job for a short while (a wave issues several jobs within a
// millisecond or two), then sleep on a condition variable.  One owner thread
// issues the jobs, one at a time: run() is not reentrant (fn must not call it)
// and a pool is not shared between threads (each miner owns its own).
#pragma once

#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace sg {

class HostPool {
  public:
    explicit HostPool(unsigned threads) : n_(std::max(1u, threads)) {}
    HostPool(const HostPool &) = delete;
    HostPool &operator=(const HostPool &) = delete;
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_.store(true, std::memory_order_relaxed);
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }

    unsigned threads() const { return n_; }

    // fn(lo, hi) over [0, n) in chunks of `chunk`; serial when n is at most one chunk
    template <class F> void run(uint64_t n, uint64_t chunk, F &&fn) {
        if (n == 0) return;
        chunk = std::max<uint64_t>(chunk, 1);
        if (n_ == 1 || n <= chunk) {
            fn((uint64_t)0, n);
            return;
        }
        if (th_.empty()) start();
        job_ = [&fn](uint64_t lo, uint64_t hi) { fn(lo, hi); };
        n_job_ = n;
        chunk_ = chunk;
        next_.store(0, std::memory_order_relaxed);
        pending_.store((unsigned)th_.size(), std::memory_order_relaxed);
        {
            std::lock_guard<std::mutex> lk(mu_);
            gen_.fetch_add(1, std::memory_order_release);
        }
        cv_.notify_all();
        work();
        if (!poll([&] { return pending_.load(std::memory_order_acquire) == 0; })) {
            std::unique_lock<std::mutex> lk(mu_);
            done_.wait(lk, [&] { return pending_.load(std::memory_order_acquire) == 0; });
        }
        job_ = nullptr;
    }

  private:
    // polls cond() for up to kPollUs microseconds
    template <class C> static bool poll(C &&cond) {
        constexpr int64_t kPollUs = 200;
        const auto t0 = std::chrono::steady_clock::now();
        for (uint32_t i = 0;; ++i) {
            if (cond()) return true;
            if ((i & 255) == 255 &&
                std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count() >
                    kPollUs)
                return cond();
        }
    }
    void start() {
        th_.reserve(n_ - 1);
        for (unsigned i = 1; i < n_; ++i) th_.emplace_back([this] { loop(); });
    }
    void work() {
        for (;;) {
            const uint64_t lo = next_.fetch_add(chunk_, std::memory_order_relaxed);
            if (lo >= n_job_) return;
            job_(lo, std::min(n_job_, lo + chunk_));
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            auto fresh = [&] {
                return gen_.load(std::memory_order_acquire) != seen || stop_.load(std::memory_order_relaxed);
            };
            if (!poll(fresh)) {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, fresh);
            }
            if (stop_.load(std::memory_order_relaxed)) return;
            seen = gen_.load(std::memory_order_acquire);
            work();
            if (pending_.fetch_sub(1, std::memory_order_acq_rel) == 1) {
                std::lock_guard<std::mutex> lk(mu_);
                done_.notify_one();
            }
        }
    }

    const unsigned n_;
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    std::atomic<uint64_t> gen_{0};
    std::atomic<unsigned> pending_{0};
    std::atomic<bool> stop_{false};
    std::function<void(uint64_t, uint64_t)> job_;
    uint64_t n_job_ = 0, chunk_ = 1;
    std::atomic<uint64_t> next_{0};
};

}  // namespace sg
