// ring.cu -- device-resident transaction ring for sliding-window mining.
//
// No reference counterpart in the engines; the nearest code is the
// reference's window transactionisation (code/pipeline/skab_spike.py:61-80)
// followed by one engine process per window.  Here a stream of transactions
// is appended into vertical bitmap rows that live on the GPU as a ring
// (capacity = a power of two of 64-transaction words): appending a batch
// first clears the bit range it overwrites (evicting the oldest
// transactions) and then sets the new bits.  A window [start, start+len) is
// extracted by a funnel-shift copy into a handle's dataset, so no window is
// ever transposed on the host.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <set>

#include "common.cuh"
#include "engine.h"

struct sgfim_ring {
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    uint32_t d = 0;
    uint64_t cap_words = 0;   // power of two
    uint64_t head = 0;        // stream position of the next transaction
    sg::DevBuf rows;          // d x cap_words
    sg::DevBuf hm;            // horizontal item masks, cap_words*64 x 2 words (rings of <= 128 items)
    sg::DevBuf stage_ptr, stage_items;
    sg::HostBuf hstage_ptr, hstage_items;
    std::mutex mu;
    std::condition_variable cv;          // signalled when windows stop being mined
    std::multiset<uint64_t> inflight;    // starts of windows being mined
    std::string err;
};

// CTAs per SM of the cross-subtree filter (each holds one window's candidate
// rows in its own scratch).  On the 4,096 service windows, largest first: 2 per
// SM 59 ms, 4 per SM 46.5 ms, 8 per SM 45.4 ms.
#ifndef SGFIM_WFILTER_CTAS_PER_SM
#define SGFIM_WFILTER_CTAS_PER_SM 8
#endif
constexpr uint64_t kFilterCtasPerSm = SGFIM_WFILTER_CTAS_PER_SM;
// results up to this size leave the device through a pinned staging buffer
constexpr size_t kStageOutMax = 64ull << 20;

namespace sg {

// Clear ring bits [p0, p0 + n) (positions modulo the ring size) in every row.
__global__ void ring_clear_kernel(unsigned long long *__restrict__ rows, uint32_t d, uint64_t cap_words, uint64_t p0,
                                  uint64_t n) {
    const uint64_t w_first = p0 >> 6, w_last = (p0 + n - 1) >> 6;  // unwrapped word range
    const uint64_t n_w = w_last - w_first + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)d * n_w;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = (uint32_t)(i / n_w);
        const uint64_t w = w_first + (i - (uint64_t)e * n_w);
        const uint64_t lo = w * 64 > p0 ? w * 64 : p0;
        const uint64_t hi = (w * 64 + 64) < (p0 + n) ? (w * 64 + 64) : (p0 + n);
        const uint64_t m = (hi - lo == 64) ? ~0ull : (((1ull << (hi - lo)) - 1) << (lo - w * 64));
        atomicAnd(&rows[(uint64_t)e * cap_words + (w & (cap_words - 1))], ~m);
    }
}

// Set the bits of a batch of transactions (stream positions p0 .. p0+n-1)
// and, when hm is given, write each transaction's 2-word item mask.
__global__ void ring_set_kernel(unsigned long long *__restrict__ rows, uint64_t *__restrict__ hm, uint32_t d,
                                uint64_t cap_words, uint64_t p0, const uint64_t *__restrict__ ptr,
                                const uint32_t *__restrict__ items, uint64_t n) {
    const uint64_t cap_bits = cap_words * 64;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = (p0 + t) & (cap_bits - 1);
        uint64_t m0 = 0, m1 = 0;
        for (uint64_t j = ptr[t]; j < ptr[t + 1]; ++j) {
            const uint32_t e = items[j];
            if (e < d) {
                atomicOr(&rows[(uint64_t)e * cap_words + (p >> 6)], 1ull << (p & 63));
                if (e < 64) m0 |= 1ull << e;
                else if (e < 128) m1 |= 1ull << (e - 64);
            }
        }
        if (hm) {
            hm[2 * p] = m0;
            hm[2 * p + 1] = m1;
        }
    }
}

// Window extraction: out bit t of row e = ring bit (start + t) of row e, t < len.
__global__ void ring_window_kernel(const uint64_t *__restrict__ rows, uint32_t d, uint64_t cap_words, uint64_t start,
                                   uint64_t len, uint64_t *__restrict__ out, uint64_t out_stride) {
    const uint64_t n_w = (len + 63) / 64;
    const uint32_t sh = (uint32_t)(start & 63);
    const uint64_t w0 = start >> 6;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)d * out_stride;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = (uint32_t)(i / out_stride);
        const uint64_t w = i - (uint64_t)e * out_stride;
        uint64_t v = 0;
        if (w < n_w) {
            const uint64_t *r = rows + (uint64_t)e * cap_words;
            const uint64_t a = r[(w0 + w) & (cap_words - 1)];
            v = a >> sh;
            if (sh) v |= r[(w0 + w + 1) & (cap_words - 1)] << (64 - sh);
            const uint64_t rem = len - w * 64;
            if (rem < 64) v &= (1ull << rem) - 1;
        }
        out[(uint64_t)e * out_stride + w] = v;
    }
}

}  // namespace sg

using namespace sg;

extern "C" {

int sgfim_ring_open(int device, uint32_t n_items, uint64_t capacity_txn, sgfim_ring **out) {
    if (!out || n_items == 0 || capacity_txn == 0) return SGFIM_EINVAL;
    *out = nullptr;
    sgfim_ring *r = new (std::nothrow) sgfim_ring();
    if (!r) return SGFIM_ENOMEM;
    try {
        SG_CUDA_TRY(cudaSetDevice(device));
        r->device = device;
        SG_CUDA_TRY(cudaDeviceGetAttribute(&r->n_sm, cudaDevAttrMultiProcessorCount, device));
        SG_CUDA_TRY(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
        uint64_t w = 64;
        while (w * 64 < capacity_txn) w <<= 1;
        r->cap_words = w;
        r->d = n_items;
        r->rows.reserve((size_t)n_items * w * 8, r->stream);
        SG_CUDA_TRY(cudaMemsetAsync(r->rows.ptr, 0, (size_t)n_items * w * 8, r->stream));
        if (n_items <= 128) {
            r->hm.reserve((size_t)w * 64 * 16, r->stream);
            SG_CUDA_TRY(cudaMemsetAsync(r->hm.ptr, 0, (size_t)w * 64 * 16, r->stream));
        }
        SG_CUDA_TRY(cudaStreamSynchronize(r->stream));
    } catch (const CudaError &) {
        r->rows.release();
        r->hm.release();
        if (r->stream) cudaStreamDestroy(r->stream);
        delete r;
        return SGFIM_EDEVICE;
    }
    *out = r;
    return SGFIM_OK;
}

void sgfim_ring_close(sgfim_ring *r) {
    if (!r) return;
    cudaSetDevice(r->device);
    if (r->stream) cudaStreamSynchronize(r->stream);
    r->rows.release();
    r->hm.release();
    r->stage_ptr.release();
    r->stage_items.release();
    r->hstage_ptr.release();
    r->hstage_items.release();
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
}

uint64_t sgfim_ring_head(sgfim_ring *r) {
    if (!r) return 0;
    std::lock_guard<std::mutex> lock(r->mu);
    return r->head;
}

uint64_t sgfim_ring_capacity(const sgfim_ring *r) { return r ? r->cap_words * 64 : 0; }

int sgfim_ring_append(sgfim_ring *r, const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn) {
    if (!r || (n_txn && !row_ptr)) return SGFIM_EINVAL;
    if (n_txn == 0) return SGFIM_OK;
    if (row_ptr[0] != 0) return SGFIM_EINVAL;
    std::unique_lock<std::mutex> lock(r->mu);
    const uint64_t cap_bits = r->cap_words * 64;
    try {
        SG_CUDA_TRY(cudaSetDevice(r->device));
        uint64_t done = 0;
        while (done < n_txn) {
            // never append more than one ring's worth in one step
            const uint64_t n = std::min<uint64_t>(n_txn - done, cap_bits / 2);
            const uint64_t base = row_ptr[done], ni = row_ptr[done + n] - base;
            // positions below head + n - capacity get overwritten: wait for windows still being mined there
            r->cv.wait(lock, [&] { return r->inflight.empty() || r->head + n <= *r->inflight.begin() + cap_bits; });
            // the previous batch's copies must finish before the pinned buffers are reused or freed
            SG_CUDA_TRY(cudaStreamSynchronize(r->stream));
            r->hstage_ptr.reserve((n + 1) * 8);
            r->hstage_items.reserve(std::max<uint64_t>(ni, 1) * 4);
            uint64_t *hp = r->hstage_ptr.as<uint64_t>();
            for (uint64_t t = 0; t <= n; ++t) hp[t] = row_ptr[done + t] - base;
            if (ni) memcpy(r->hstage_items.ptr, items + base, ni * 4);
            r->stage_ptr.reserve((n + 1) * 8, r->stream);
            r->stage_items.reserve(std::max<uint64_t>(ni, 1) * 4, r->stream);
            SG_CUDA_TRY(cudaMemcpyAsync(r->stage_ptr.ptr, hp, (n + 1) * 8, cudaMemcpyHostToDevice, r->stream));
            if (ni)
                SG_CUDA_TRY(cudaMemcpyAsync(r->stage_items.ptr, r->hstage_items.ptr, ni * 4, cudaMemcpyHostToDevice,
                                            r->stream));
            const uint64_t p0 = r->head & (cap_bits - 1);
            const uint64_t words = ((p0 + n - 1) >> 6) - (p0 >> 6) + 1;
            const unsigned cb = (unsigned)std::min<uint64_t>(((uint64_t)r->d * words + 255) / 256, 4096);
            ring_clear_kernel<<<cb, 256, 0, r->stream>>>(reinterpret_cast<unsigned long long *>(r->rows.ptr), r->d,
                                                         r->cap_words, p0, n);
            SG_CUDA_TRY(cudaGetLastError());
            const unsigned sb = (unsigned)std::min<uint64_t>((n + 255) / 256, 4096);
            ring_set_kernel<<<sb, 256, 0, r->stream>>>(reinterpret_cast<unsigned long long *>(r->rows.ptr),
                                                       r->hm.as<uint64_t>(), r->d, r->cap_words, r->head,
                                                       r->stage_ptr.as<uint64_t>(),
                                                       r->stage_items.as<uint32_t>(), n);
            SG_CUDA_TRY(cudaGetLastError());
            r->head += n;
            done += n;
        }
        return SGFIM_OK;
    } catch (const CudaError &e) {
        r->err = e.what;
        return SGFIM_EDEVICE;
    }
}

int sgfim_ring_window_load(sgfim_ring *r, sgfim_handle *h, uint64_t start, uint64_t len) {
    if (!r || !h) return SGFIM_EINVAL;
    if (h->device != r->device) return fail(h, SGFIM_EINVAL, "ring and handle are on different devices");
    std::unique_lock<std::mutex> lock(r->mu);
    const uint64_t cap_bits = r->cap_words * 64;
    if (start + len > r->head) return fail(h, SGFIM_EINVAL, "window ends after the ring head");
    if (r->head - start > cap_bits) return fail(h, SGFIM_EINVAL, "window start already evicted from the ring");
    try {
        SG_CUDA_TRY(cudaSetDevice(h->device));
        Dataset &ds = h->ds;
        reset_dataset(ds);
        ds.source = "<ring window>";
        ds.remap_identity = true;
        ds.n_txn = len;
        ds.n_ids = r->d;
        ds.d = r->d;
        const uint64_t words = (len + 63) / 64;
        ds.n_words = (words + 1) & ~1ull;
        ds.stride = std::max<uint64_t>(ds.n_words, 2);
        ds.bitmaps.reserve((size_t)ds.d * ds.stride * 8, h->stream);
        ds.sup_dev.reserve((size_t)ds.d * 4, h->stream);
        // extraction runs on the ring's stream, after every append enqueued so far
        const unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)r->d * ds.stride + 255) / 256, 8192);
        ring_window_kernel<<<blocks, 256, 0, r->stream>>>(r->rows.as<uint64_t>(), r->d, r->cap_words, start, len,
                                                          ds.bitmaps.as<uint64_t>(), ds.stride);
        SG_CUDA_TRY(cudaGetLastError());
        cudaEvent_t ev;
        SG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        SG_CUDA_TRY(cudaEventRecord(ev, r->stream));
        lock.unlock();
        SG_CUDA_TRY(cudaStreamWaitEvent(h->stream, ev, 0));
        SG_CUDA_TRY(cudaEventDestroy(ev));
        launch_row_popc(ds.bitmaps.as<uint64_t>(), ds.stride, ds.n_words, ds.d, ds.sup_dev.as<uint32_t>(), h->stream);
        h->launches += 2;
        ds.sup.assign(ds.d, 0);
        SG_CUDA_TRY(cudaMemcpyAsync(ds.sup.data(), ds.sup_dev.ptr, (size_t)ds.d * 4, cudaMemcpyDeviceToHost,
                                    h->stream));
        SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
        ds.o2d.resize(ds.d);
        ds.d2o.resize(ds.d);
        for (uint32_t e = 0; e < ds.d; ++e) {
            ds.o2d[e] = (int32_t)e;
            ds.d2o[e] = e;
        }
        ds.occ = ds.sup;
        ds.id_min = UINT32_MAX;
        for (uint32_t e = 0; e < ds.d; ++e)
            if (ds.sup[e]) {
                ds.n_present++;
                ds.id_min = std::min(ds.id_min, e);
                ds.id_max = e;
            }
        if (!ds.n_present) ds.id_min = 0;
        ds.map_ok = encode_bitmap_map(&ds.map, ds.bitmaps.as<uint64_t>(), ds.d, ds.n_words, ds.stride);
        ds.loaded = true;
        return SGFIM_OK;
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }
}

void sgfim_windows_result_free(sgfim_windows_result *res) {
    if (!res) return;
    free(res->offset);
    free(res->masks);
    free(res->support);
    free(res->status);
    free(res->nodes);
    free(res->batched);
    free(res);
}

int sgfim_ring_mine_windows(sgfim_ring *r, sgfim_handle *h, const uint64_t *starts, const uint64_t *lens,
                            const uint32_t *min_counts, uint64_t n_windows, sgfim_windows_result **out) {
    if (!out) return SGFIM_EINVAL;
    *out = nullptr;
    if (!r || !h || (n_windows && (!starts || !lens || !min_counts))) return fail(h, SGFIM_EINVAL, "null argument");
    if (h->device != r->device) return fail(h, SGFIM_EINVAL, "ring and handle are on different devices");
    if (n_windows > 0xffffffffull) return fail(h, SGFIM_EINVAL, "too many windows");
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    const uint64_t cap_bits = r->cap_words * 64;
    const uint32_t mw = 2;                                     // batched kernel mask width
    const uint32_t words = std::max<uint32_t>(2, (r->d + 63) / 64);   // result mask width
    // register the windows as in flight (appends that would overwrite them wait)
    cudaEvent_t ev = nullptr;
    {
        std::lock_guard<std::mutex> lock(r->mu);
        for (uint64_t w = 0; w < n_windows; ++w) {
            if (starts[w] + lens[w] > r->head) return fail(h, SGFIM_EINVAL, "window ends after the ring head");
            if (r->head - starts[w] > cap_bits) return fail(h, SGFIM_EINVAL, "window start already evicted");
            if (lens[w] > 0xffffffffull) return fail(h, SGFIM_EINVAL, "window longer than 2^32-1 transactions");
        }
        for (uint64_t w = 0; w < n_windows; ++w) r->inflight.insert(starts[w]);
        try {
            SG_CUDA_TRY(cudaSetDevice(h->device));
            SG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            SG_CUDA_TRY(cudaEventRecord(ev, r->stream));
        } catch (const CudaError &e) {
            for (uint64_t w = 0; w < n_windows; ++w) r->inflight.erase(r->inflight.find(starts[w]));
            r->cv.notify_all();
            if (ev) cudaEventDestroy(ev);
            return fail(h, SGFIM_EDEVICE, e.what);
        }
    }
    struct Release {
        sgfim_ring *r;
        const uint64_t *starts;
        uint64_t n;
        cudaEvent_t ev;
        ~Release() {
            if (ev) cudaEventDestroy(ev);
            std::lock_guard<std::mutex> lock(r->mu);
            for (uint64_t w = 0; w < n; ++w) r->inflight.erase(r->inflight.find(starts[w]));
            r->cv.notify_all();
        }
    } release{r, starts, n_windows, ev};

    // per-window results
    std::vector<uint64_t> res_cnt(n_windows, 0), nodes(n_windows, 0);
    std::vector<int32_t> status(n_windows, SGFIM_OK);
    std::vector<uint8_t> batched(n_windows, 0);
    std::vector<uint64_t> root_cand;         // (window, mask words...) of split windows with a terminal root
    std::vector<uint32_t> root_cand_sup;
    std::vector<uint64_t> wave;              // windows for the wave miner
    double kernel_ms = 0.0;
    uint32_t launches = 0;
    // batched results, gathered on the device into window order at the end
    std::vector<uint64_t> task_dst;          // per task: destination slot (~0 = dropped)
    uint64_t n_tasks_total = 0;
    WindowWorkspace &ws = h->wws;
    uint64_t *d_task_off = nullptr;
    uint32_t *d_task_cnt = nullptr;
    uint8_t *d_keep = nullptr;
    std::vector<uint64_t> t_win_of;          // task -> window
    std::vector<uint32_t> kept;              // per task: candidates kept
    uint32_t task_warps = 0;
    double task_kernel_ms = 0.0, task_ms_max = 0.0, task_ms_sum = 0.0;
    try {
        SG_CUDA_TRY(cudaSetDevice(h->device));
        cudaStream_t st = h->stream;
        if (r->hm.ptr && n_windows) {
            // windows of at least kSplitMin transactions are split at the root: even a short
            // window's tree has tens of thousands of nodes, too many for one warp in a batch
            constexpr uint64_t kSplitMin = 64;
            uint64_t max_len = 0;
            std::vector<uint32_t> split;
            for (uint64_t w = 0; w < n_windows; ++w) {
                max_len = std::max(max_len, lens[w]);
                if (lens[w] >= kSplitMin) split.push_back((uint32_t)w);
            }
            // the vertical search keeps only the task's base database as entries; the horizontal
            // one stacks every level's database
            const bool vertical = !(h->flags & SGFIM_F_WINDOWS_HORIZONTAL);
            const uint64_t list_cap = std::min<uint64_t>(
                std::max<uint64_t>(8192, (vertical ? 1 : 2) * max_len + 1024), 1ull << 30);
            const uint64_t lmfi_cap = 1u << 16, pool_cap = 1u << 16;
            const uint64_t v_words = vertical ? (max_len + 31) / 32 + 1 : 0;
            const size_t v_bytes = (size_t)(128 + wmine_depth()) * v_words * 4;
            const size_t per_warp =
                list_cap * mw * 8 + lmfi_cap * 4 + pool_cap * (mw * 8 + 4) + wmine_level_bytes(mw) + v_bytes;
            uint64_t warps = (uint64_t)h->n_sm * 4 * (uint64_t)wtask_blocks_per_sm(vertical);
            warps = std::min<uint64_t>(warps, std::max<uint64_t>(4, (h->hbm_budget / 2) / per_warp));
            warps = std::max<uint64_t>(4, warps & ~3ull);
            const size_t cand_bytes = mw * 8 + 4 + 1;
            const uint64_t out_cap = std::max<uint64_t>(
                1u << 20, std::min<uint64_t>(n_windows * 65536, (h->hbm_budget / 4) / cand_bytes));
            const size_t root_b = wmine_root_bytes(mw);
            ws.lists.reserve(warps * list_cap * mw * 8, st);
            ws.lmfi.reserve(warps * lmfi_cap * 4, st);
            ws.pool_m.reserve(warps * pool_cap * mw * 8, st);
            ws.pool_s.reserve(warps * pool_cap * 4, st);
            ws.levels.reserve(warps * wmine_level_bytes(mw), st);
            if (vertical) ws.vbuf.reserve(warps * v_bytes, st);
            ws.out_m.reserve(out_cap * mw * 8, st);
            ws.out_s.reserve(out_cap * 5, st);   // supports, then the keep flags
            ws.ctrl.reserve(256, st);
            ws.res.reserve(n_windows * root_b, st);
            // window table: starts u64 | lens u32 | thrs u32 | split u32
            const size_t tb = n_windows * 8 + 3 * n_windows * 4;
            ws.table.reserve(tb, st);
            ws.h_table.reserve(tb);
            uint64_t *t_start = ws.h_table.as<uint64_t>();
            uint32_t *t_len = reinterpret_cast<uint32_t *>(t_start + n_windows);
            uint32_t *t_thr = t_len + n_windows;
            uint32_t *t_split = t_thr + n_windows;
            for (uint64_t w = 0; w < n_windows; ++w) {
                t_start[w] = starts[w];
                t_len[w] = (uint32_t)lens[w];
                t_thr[w] = min_counts[w] ? min_counts[w] : 1;
            }
            if (!split.empty()) memcpy(t_split, split.data(), split.size() * 4);
            SG_CUDA_TRY(cudaStreamWaitEvent(st, ev, 0));
            SG_CUDA_TRY(cudaMemcpyAsync(ws.table.ptr, ws.h_table.ptr, tb, cudaMemcpyHostToDevice, st));
            SG_CUDA_TRY(cudaMemsetAsync(ws.ctrl.ptr, 0, 256, st));
            uint64_t *d_start = ws.table.as<uint64_t>();
            uint32_t *d_len = reinterpret_cast<uint32_t *>(d_start + n_windows);
            uint32_t *d_thr = d_len + n_windows;
            uint32_t *d_split = d_thr + n_windows;
            cudaEvent_t k0, k1;
            SG_CUDA_TRY(cudaEventCreate(&k0));
            SG_CUDA_TRY(cudaEventCreate(&k1));
            struct EvPair {
                cudaEvent_t a, b;
                ~EvPair() { cudaEventDestroy(a); cudaEventDestroy(b); }
            } evp{k0, k1};
            auto timed_ms = [&]() {
                float ms = 0.f;
                SG_CUDA_TRY(cudaEventElapsedTime(&ms, k0, k1));
                return (double)ms;
            };
            WMineParams p;
            p.hm = r->hm.as<uint64_t>();
            p.cap_mask = cap_bits - 1;
            p.ring_rows = r->rows.as<uint64_t>();
            p.ring_words = r->cap_words;
            p.d = r->d;
            p.starts = d_start;
            p.lens = d_len;
            p.thrs = d_thr;
            p.roots = ws.res.ptr;
            p.split_win = d_split;
            p.n_split = (uint32_t)split.size();
            p.next = ws.ctrl.as<uint32_t>();
            p.out_pos = reinterpret_cast<unsigned long long *>(ws.ctrl.as<uint64_t>() + 2);
            p.lists = ws.lists.as<uint64_t>();
            p.list_cap = (uint32_t)list_cap;
            p.lmfi = ws.lmfi.as<uint32_t>();
            p.lmfi_cap = (uint32_t)lmfi_cap;
            p.pool_m = ws.pool_m.as<uint64_t>();
            p.pool_s = ws.pool_s.as<uint32_t>();
            p.pool_cap = (uint32_t)pool_cap;
            p.levels = ws.levels.ptr;
            p.vbuf = vertical ? ws.vbuf.as<uint32_t>() : nullptr;
            p.v_words = (uint32_t)v_words;
            p.out_m = ws.out_m.as<uint64_t>();
            p.out_s = ws.out_s.as<uint32_t>();
            p.out_cap = out_cap;
            // record fields read here (WRoot<2>: hp[2], cand[2], cand_sup, has_cand, k, overflow, f[128], c[128])
            const size_t o_cand = 16, o_csup = 32, o_has = 36, o_k = 40, o_ovf = 44, o_f = 48, o_c = 176;
            auto u32_at = [](const unsigned char *rec, size_t off) {
                uint32_t v;
                memcpy(&v, rec + off, 4);
                return v;
            };
            // ---- 1. roots of the split windows
            std::vector<unsigned char> roots_h;
            if (!split.empty()) {
                SG_CUDA_TRY(cudaEventRecord(k0, st));
                launch_wroot(p, (int)mw, (unsigned)std::min<uint64_t>((split.size() + 3) / 4, (uint64_t)h->n_sm * 8),
                             st);
                SG_CUDA_TRY(cudaEventRecord(k1, st));
                ++launches;
                ++h->launches;
                roots_h.resize(n_windows * root_b);
                SG_CUDA_TRY(cudaMemcpyAsync(roots_h.data(), ws.res.ptr, n_windows * root_b, cudaMemcpyDeviceToHost, st));
                h->sync();
                kernel_ms += timed_ms();
            }
            auto root_at = [&](uint64_t w) { return roots_h.data() + (size_t)w * root_b; };
            // cost estimate of a subtree: its database size plus a fixed per-node share, per tail item
            auto child_cost = [](uint32_t sup, uint32_t tail) { return ((double)sup + 512.0) * (double)tail; };
            std::vector<uint8_t> is_split(n_windows, 0), bad(n_windows, 0);
            for (uint32_t w : split) is_split[w] = 1;
            // ---- 2. the costliest root children are split again (their own expansion in wsub_kernel)
            double total_cost = 0.0;
            for (uint64_t w = 0; w < n_windows; ++w) {
                if (!is_split[w]) {
                    total_cost += 1300.0 * (double)lens[w];
                    continue;
                }
                const unsigned char *R = root_at(w);
                const uint32_t k = u32_at(R, o_has) ? 0 : u32_at(R, o_k);
                for (uint32_t j = 0; j < k; ++j) total_cost += child_cost(u32_at(R, o_c + 4 * j), k - j);
            }
            const double split_above = total_cost / (double)(warps * 2);
            std::vector<uint32_t> sub_win, sub_child;
            std::vector<uint32_t> sub_of_first(n_windows, 0);   // first sub index of each split window
            for (uint32_t w : split) {
                sub_of_first[w] = (uint32_t)sub_win.size();
                const unsigned char *R = root_at(w);
                if (u32_at(R, o_has)) continue;
                const uint32_t k = u32_at(R, o_k);
                for (uint32_t j = 0; j + 2 < k; ++j)
                    if (child_cost(u32_at(R, o_c + 4 * j), k - j) > split_above) {
                        sub_win.push_back(w);
                        sub_child.push_back(j);
                    }
            }
            std::vector<unsigned char> subs_h;
            if (!sub_win.empty()) {
                const size_t ns = sub_win.size();
                ws.sub.reserve(ns * root_b + ns * 8 + 256, st);
                uint32_t *d_sw = reinterpret_cast<uint32_t *>(ws.sub.as<char>() + ((ns * root_b + 255) & ~(size_t)255));
                std::vector<uint32_t> sw(sub_win);
                sw.insert(sw.end(), sub_child.begin(), sub_child.end());
                SG_CUDA_TRY(cudaMemcpyAsync(d_sw, sw.data(), sw.size() * 4, cudaMemcpyHostToDevice, st));
                p.subs = ws.sub.ptr;
                p.sub_win = d_sw;
                p.sub_child = d_sw + ns;
                p.n_sub = (uint32_t)ns;
                SG_CUDA_TRY(cudaEventRecord(k0, st));
                launch_wsub(p, (int)mw, (unsigned)(std::min<uint64_t>(warps, (ns + 3) & ~3ull) / 4), st);
                SG_CUDA_TRY(cudaEventRecord(k1, st));
                ++launches;
                ++h->launches;
                subs_h.resize(ns * root_b);
                SG_CUDA_TRY(cudaMemcpyAsync(subs_h.data(), ws.sub.ptr, ns * root_b, cudaMemcpyDeviceToHost, st));
                h->sync();
                kernel_ms += timed_ms();
            }
            // ---- 3. tasks in depth-first order within each window
            std::vector<uint32_t> t_win, t_child, t_sub, t_gchild;
            std::vector<double> t_cost;
            {
                size_t est = n_windows;
                for (uint32_t w : split) {
                    const unsigned char *R = root_at(w);
                    if (!u32_at(R, o_has)) est += u32_at(R, o_k);
                }
                for (size_t i = 0; i < sub_win.size(); ++i) est += u32_at(subs_h.data() + i * root_b, o_k);
                t_win.reserve(est);
                t_child.reserve(est);
                t_sub.reserve(est);
                t_gchild.reserve(est);
                t_cost.reserve(est);
            }
            auto add_task = [&](uint32_t w, uint32_t c, uint32_t sb, uint32_t g, double cost) {
                t_win.push_back(w);
                t_child.push_back(c);
                t_sub.push_back(sb);
                t_gchild.push_back(g);
                t_cost.push_back(cost);
            };
            for (uint64_t w = 0; w < n_windows; ++w) {
                if (!is_split[w]) {
                    add_task((uint32_t)w, kWholeWindow, kWholeWindow, kWholeWindow, 1300.0 * (double)lens[w]);
                    continue;
                }
                const unsigned char *R = root_at(w);
                if (u32_at(R, o_has)) {
                    uint64_t m[2];
                    memcpy(m, R + o_cand, 16);
                    root_cand.push_back(w);
                    root_cand.push_back(m[0]);
                    root_cand.push_back(m[1]);
                    root_cand_sup.push_back(u32_at(R, o_csup));
                    continue;
                }
                const uint32_t k = u32_at(R, o_k);
                uint32_t si = sub_of_first[w];
                for (uint32_t j = 0; j < k; ++j) {
                    if (si < sub_win.size() && sub_win[si] == w && sub_child[si] == j) {
                        const unsigned char *S = subs_h.data() + (size_t)si * root_b;
                        if (u32_at(S, o_ovf)) {
                            bad[w] = 1;
                        } else if (u32_at(S, o_has)) {
                            add_task((uint32_t)w, j, si, kWholeWindow, 1.0);
                        } else {
                            const uint32_t k1 = u32_at(S, o_k);
                            for (uint32_t g = 0; g < k1; ++g)
                                add_task((uint32_t)w, j, si, g, child_cost(u32_at(S, o_c + 4 * g), k1 - g));
                        }
                        ++si;
                    } else {
                        add_task((uint32_t)w, j, kWholeWindow, kWholeWindow, child_cost(u32_at(R, o_c + 4 * j), k - j));
                    }
                }
            }
            (void)o_f;
            const uint64_t nt = t_win.size();
            n_tasks_total = nt;
            std::vector<uint32_t> order(nt);
            for (uint64_t i = 0; i < nt; ++i) order[i] = (uint32_t)i;
            // costliest first to within a factor of two (a counting sort on the cost's binary
            // exponent, creation order inside an exponent): the order only schedules the tasks
            {
                std::vector<uint32_t> bucket(nt);
                uint64_t cnt[129] = {0};
                for (uint64_t i = 0; i < nt; ++i) {
                    int e = 0;
                    std::frexp(t_cost[i], &e);
                    bucket[i] = 127u - (uint32_t)std::min(127, std::max(0, e));
                    ++cnt[bucket[i] + 1];
                }
                for (int b = 0; b < 128; ++b) cnt[b + 1] += cnt[b];
                for (uint64_t i = 0; i < nt; ++i) order[cnt[bucket[i]]++] = (uint32_t)i;
            }
            // task arrays: win | child | sub | gchild | order | cnt | kept | status (u32) | off | nodes (u64)
            const size_t nt1 = std::max<uint64_t>(nt, 1);
            const size_t u32_bytes = (8 * 4 * nt1 + 15) & ~(size_t)15;
            ws.tasks.reserve(u32_bytes + 3 * 8 * nt1, st);
            uint32_t *dt_win = ws.tasks.as<uint32_t>();
            uint32_t *dt_child = dt_win + nt1;
            uint32_t *dt_sub = dt_child + nt1;
            uint32_t *dt_gchild = dt_sub + nt1;
            uint32_t *dt_order = dt_gchild + nt1;
            uint32_t *dt_cnt = dt_order + nt1;
            uint32_t *dt_kept = dt_cnt + nt1;
            int32_t *dt_status = reinterpret_cast<int32_t *>(dt_kept + nt1);
            uint64_t *dt_off = reinterpret_cast<uint64_t *>(ws.tasks.as<char>() + u32_bytes);
            uint64_t *dt_nodes = dt_off + nt1;
            uint64_t *dt_ns = dt_nodes + nt1;
            d_task_off = dt_off;
            d_task_cnt = dt_cnt;
            if (nt) {
                ws.h_res.reserve(5 * nt1 * 4);
                uint32_t *hw = ws.h_res.as<uint32_t>();
                memcpy(hw, t_win.data(), nt * 4);
                memcpy(hw + nt1, t_child.data(), nt * 4);
                memcpy(hw + 2 * nt1, t_sub.data(), nt * 4);
                memcpy(hw + 3 * nt1, t_gchild.data(), nt * 4);
                memcpy(hw + 4 * nt1, order.data(), nt * 4);
                SG_CUDA_TRY(cudaMemcpyAsync(dt_win, hw, 5 * nt1 * 4, cudaMemcpyHostToDevice, st));
                p.task_win = dt_win;
                p.task_child = dt_child;
                p.task_sub = dt_sub;
                p.task_gchild = dt_gchild;
                p.task_order = dt_order;
                p.n_tasks = (uint32_t)nt;
                p.task_off = dt_off;
                p.task_cnt = dt_cnt;
                p.task_status = dt_status;
                p.task_nodes = dt_nodes;
                p.task_ns = dt_ns;
                // ---- 4. all tasks in one persistent launch
                const uint64_t use_warps = std::min<uint64_t>(warps, (nt + 3) & ~3ull);
                SG_CUDA_TRY(cudaEventRecord(k0, st));
                launch_wtask(p, (int)mw, (unsigned)(use_warps / 4), st);
                SG_CUDA_TRY(cudaEventRecord(k1, st));
                ++launches;
                ++h->launches;
                std::vector<uint32_t> cnt_h(nt), st_h(nt);
                std::vector<uint64_t> nodes_h(nt), ns_h(nt);
                SG_CUDA_TRY(cudaMemcpyAsync(ns_h.data(), dt_ns, nt * 8, cudaMemcpyDeviceToHost, st));
                SG_CUDA_TRY(cudaMemcpyAsync(cnt_h.data(), dt_cnt, nt * 4, cudaMemcpyDeviceToHost, st));
                SG_CUDA_TRY(cudaMemcpyAsync(st_h.data(), dt_status, nt * 4, cudaMemcpyDeviceToHost, st));
                SG_CUDA_TRY(cudaMemcpyAsync(nodes_h.data(), dt_nodes, nt * 8, cudaMemcpyDeviceToHost, st));
                uint64_t used = 0;
                SG_CUDA_TRY(cudaMemcpyAsync(&used, p.out_pos, 8, cudaMemcpyDeviceToHost, st));
                h->sync();
                task_kernel_ms = timed_ms();
                kernel_ms += task_kernel_ms;
                task_warps = (uint32_t)use_warps;
                for (uint64_t t = 0; t < nt; ++t) {
                    task_ms_max = std::max(task_ms_max, ns_h[t] * 1e-6);
                    task_ms_sum += ns_h[t] * 1e-6;
                }
                used = std::min<uint64_t>(used, out_cap);
                for (uint64_t t = 0; t < nt; ++t) {
                    nodes[t_win[t]] += nodes_h[t];
                    if (st_h[t] != 0) bad[t_win[t]] = 1;
                }
                // ---- 5. cross-subtree filter of the split windows whose tasks all succeeded,
                // largest candidate sets first (a CTA per window; the big ones set the makespan)
                struct FWin {
                    uint32_t w;
                    uint64_t t_lo, t_hi, m;
                };
                std::vector<FWin> fw;
                uint64_t max_m = 0;
                for (uint64_t t = 0; t < nt;) {
                    const uint32_t w = t_win[t];
                    uint64_t t2 = t;
                    while (t2 < nt && t_win[t2] == w) ++t2;
                    if (is_split[w] && !bad[w]) {
                        uint64_t m = 0;
                        for (uint64_t x = t; x < t2; ++x) m += cnt_h[x];
                        fw.push_back({w, t, t2, m});
                        max_m = std::max(max_m, m);
                    }
                    t = t2;
                }
                std::stable_sort(fw.begin(), fw.end(), [](const FWin &a, const FWin &b) { return a.m > b.m; });
                std::vector<uint32_t> fwin, task0, task_of;
                std::vector<uint64_t> first, wtotal;
                for (const FWin &f : fw) {
                    task0.push_back((uint32_t)task_of.size());
                    uint64_t m = 0;
                    for (uint64_t x = f.t_lo; x < f.t_hi; ++x) {
                        task_of.push_back((uint32_t)x);   // tasks were created in depth-first order
                        first.push_back(m);
                        m += cnt_h[x];
                    }
                    fwin.push_back(f.w);
                    wtotal.push_back(m);
                }
                task0.push_back((uint32_t)task_of.size());
                kept.assign(cnt_h.begin(), cnt_h.end());
                uint8_t *keep = reinterpret_cast<uint8_t *>(p.out_s + out_cap);
                d_keep = nullptr;
                if (!fwin.empty() && used) {
                    d_keep = keep;
                    SG_CUDA_TRY(cudaMemsetAsync(keep, 1, used, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(dt_kept, dt_cnt, nt * 4, cudaMemcpyDeviceToDevice, st));
                    const uint64_t W = (max_m + 63) / 64;
                    const uint64_t scratch_words = std::max<uint64_t>(W * r->d, 64);
                    const uint64_t ctas = std::min<uint64_t>(
                        fwin.size(), std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)h->n_sm * kFilterCtasPerSm,
                                                                              (h->hbm_budget / 8) / (scratch_words * 8))));
                    // tables: first u64 | total u64 | task0 u32 | task_of u32 | status i32, then the scratch
                    const size_t tab =
                        ((first.size() + wtotal.size()) * 8 + (task0.size() + task_of.size() + fwin.size()) * 4 + 255) &
                        ~(size_t)255;
                    ws.lists.reserve(tab + ctas * scratch_words * 8, st);
                    char *fb = ws.lists.as<char>();
                    uint64_t *d_first = reinterpret_cast<uint64_t *>(fb);
                    uint64_t *d_total = d_first + first.size();
                    uint32_t *d_task0 = reinterpret_cast<uint32_t *>(d_total + wtotal.size());
                    uint32_t *d_task_of = d_task0 + task0.size();
                    int32_t *d_wstat = reinterpret_cast<int32_t *>(d_task_of + task_of.size());
                    std::vector<uint64_t> t64(first);
                    t64.insert(t64.end(), wtotal.begin(), wtotal.end());
                    std::vector<uint32_t> t32(task0);
                    t32.insert(t32.end(), task_of.begin(), task_of.end());
                    SG_CUDA_TRY(cudaMemcpyAsync(d_first, t64.data(), t64.size() * 8, cudaMemcpyHostToDevice, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(d_task0, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, st));
                    SG_CUDA_TRY(cudaMemsetAsync(d_wstat, 0, fwin.size() * 4, st));
                    WFilterParams fp;
                    fp.d = r->d;
                    fp.n_win = (uint32_t)fwin.size();
                    fp.win_task0 = d_task0;
                    fp.task_of = d_task_of;
                    fp.task_first = d_first;
                    fp.win_total = d_total;
                    fp.task_off = dt_off;
                    fp.task_cnt = dt_cnt;
                    fp.task_kept = dt_kept;
                    fp.out_m = p.out_m;
                    fp.keep = keep;
                    fp.scratch = reinterpret_cast<uint64_t *>(fb + tab);
                    fp.scratch_words = scratch_words;
                    fp.win_status = d_wstat;
                    fp.next = ws.ctrl.as<uint32_t>() + 8;
                    SG_CUDA_TRY(cudaEventRecord(k0, st));
                    // few windows (a service batch): 1,024 threads per window's CTA, so the
                    // largest window's candidates are scanned four times as wide
                    launch_wfilter(fp, (int)mw, (unsigned)ctas, fwin.size() <= (size_t)h->n_sm * 2 ? 1024u : 256u, st);
                    SG_CUDA_TRY(cudaEventRecord(k1, st));
                    ++launches;
                    ++h->launches;
                    std::vector<int32_t> wstat(fwin.size());
                    SG_CUDA_TRY(cudaMemcpyAsync(kept.data(), dt_kept, nt * 4, cudaMemcpyDeviceToHost, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(wstat.data(), d_wstat, fwin.size() * 4, cudaMemcpyDeviceToHost, st));
                    h->sync();
                    kernel_ms += timed_ms();
                    for (size_t i = 0; i < fwin.size(); ++i)
                        if (wstat[i]) bad[fwin[i]] = 1;
                }
                t_win_of.assign(t_win.begin(), t_win.end());
                for (uint64_t t = 0; t < nt; ++t)
                    if (!bad[t_win[t]]) {
                        res_cnt[t_win[t]] += kept[t];
                        batched[t_win[t]] = 1;
                    }
                task_dst.assign(nt, ~0ull);
            }
            for (size_t i = 0; i < root_cand_sup.size(); ++i) {
                const uint64_t w = root_cand[3 * i];
                res_cnt[w] = 1;
                batched[w] = 1;
            }
            // split windows whose root has neither a candidate nor a frequent tail: empty
            for (uint32_t w : split) {
                const unsigned char *R = root_at(w);
                if (!u32_at(R, o_has) && u32_at(R, o_k) == 0) batched[w] = 1;
            }
            for (uint64_t w = 0; w < n_windows; ++w)
                if (bad[w]) {
                    batched[w] = 0;
                    res_cnt[w] = 0;
                    nodes[w] = 0;
                    wave.push_back(w);
                }
        } else {
            for (uint64_t w = 0; w < n_windows; ++w) wave.push_back(w);
        }
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }

    // windows the batched kernels did not take: load and mine each on the handle
    std::vector<uint64_t> wave_m;
    std::vector<uint32_t> wave_s;
    std::vector<uint64_t> wave_off(n_windows, 0);
    std::sort(wave.begin(), wave.end());
    for (uint64_t w : wave) {
        batched[w] = 0;
        int rc = sgfim_ring_window_load(r, h, starts[w], lens[w]);
        sgfim_result *res = nullptr;
        if (rc == SGFIM_OK) {
            sgfim_mine_params mp{};
            mp.min_count = min_counts[w] ? min_counts[w] : 1;
            mp.root_rule = SGFIM_ROOTS_ALL;
            mp.order = SGFIM_ORDER_SUPPORT;
            rc = mine_impl(h, &mp, nullptr, 0, nullptr, nullptr, &res);
        }
        status[w] = rc;
        wave_off[w] = wave_s.size();
        if (rc == SGFIM_OK && res) {
            for (uint64_t i = 0; i < res->n_sets; ++i) {
                const size_t at = wave_m.size();
                wave_m.resize(at + words, 0);
                for (uint64_t k = res->set_ptr[i]; k < res->set_ptr[i + 1]; ++k) {
                    const uint32_t e = res->items[k];
                    wave_m[at + (e >> 6)] |= 1ull << (e & 63);
                }
                wave_s.push_back(res->support[i]);
            }
            res_cnt[w] = res->n_sets;
            nodes[w] = res->nodes;
        } else {
            res_cnt[w] = 0;
        }
        sgfim_result_free(res);
    }

    // assemble in window order
    sgfim_windows_result *R = static_cast<sgfim_windows_result *>(calloc(1, sizeof(sgfim_windows_result)));
    if (!R) return fail(h, SGFIM_ENOMEM, "result allocation failed");
    uint64_t total = 0;
    for (uint64_t w = 0; w < n_windows; ++w) total += res_cnt[w];
    R->n_windows = n_windows;
    R->mask_words = words;
    R->offset = static_cast<uint64_t *>(malloc((n_windows + 1) * 8));
    R->masks = static_cast<uint64_t *>(malloc(std::max<uint64_t>(total, 1) * words * 8));
    R->support = static_cast<uint32_t *>(malloc(std::max<uint64_t>(total, 1) * 4));
    R->status = static_cast<int32_t *>(malloc(std::max<uint64_t>(n_windows, 1) * 4));
    R->nodes = static_cast<uint64_t *>(malloc(std::max<uint64_t>(n_windows, 1) * 8));
    R->batched = static_cast<uint8_t *>(malloc(std::max<uint64_t>(n_windows, 1)));
    if (!R->offset || !R->masks || !R->support || !R->status || !R->nodes || !R->batched) {
        sgfim_windows_result_free(R);
        return fail(h, SGFIM_ENOMEM, "result allocation failed");
    }
    uint64_t at = 0;
    for (uint64_t w = 0; w < n_windows; ++w) {
        R->offset[w] = at;
        at += res_cnt[w];
        R->status[w] = status[w];
        R->nodes[w] = nodes[w];
        R->batched[w] = batched[w];
    }
    // batched tasks: the device gathers the kept candidates into window order
    try {
        if (n_tasks_total && at) {
            std::vector<uint64_t> fill(n_windows, 0);
            uint64_t gathered = 0;
            for (uint64_t t = 0; t < n_tasks_total; ++t) {
                const uint64_t w = t_win_of[t];
                if (!batched[w]) continue;
                task_dst[t] = R->offset[w] + fill[w];
                fill[w] += kept[t];
                gathered += kept[t];
            }
            if (gathered) {
                cudaStream_t st = h->stream;
                WindowWorkspace &ws2 = h->wws;
                // destination: the pool buffer (the tasks are done with it), masks then supports
                const size_t need = at * mw * 8 + at * 4 + n_tasks_total * 8 + 512;
                ws2.pool_m.reserve(need, st);
                uint64_t *d_dst_m = ws2.pool_m.as<uint64_t>();
                uint32_t *d_dst_s = reinterpret_cast<uint32_t *>(d_dst_m + at * mw);
                uint64_t *d_task_dst = reinterpret_cast<uint64_t *>(
                    (reinterpret_cast<uintptr_t>(d_dst_s + at) + 15) & ~(uintptr_t)15);
                SG_CUDA_TRY(cudaMemcpyAsync(d_task_dst, task_dst.data(), n_tasks_total * 8, cudaMemcpyHostToDevice,
                                            st));
                WGatherParams gp;
                gp.n_tasks = n_tasks_total;
                gp.task_off = d_task_off;
                gp.task_cnt = d_task_cnt;
                gp.task_dst = d_task_dst;
                gp.keep = d_keep;
                gp.out_m = ws2.out_m.as<uint64_t>();
                gp.out_s = ws2.out_s.as<uint32_t>();
                gp.dst_m = d_dst_m;
                gp.dst_s = d_dst_s;
                launch_wgather(gp, (int)mw, (unsigned)std::min<uint64_t>((n_tasks_total + 3) / 4, (uint64_t)h->n_sm * 8),
                               st);
                ++launches;
                ++h->launches;
                const size_t out_b = at * mw * 8 + at * 4;
                if (out_b <= kStageOutMax && words == mw) {
                    // small results through the handle's pinned staging buffer: the copy into the
                    // freshly allocated (pageable) result arrays would fault their pages in
                    // during the DMA
                    ws2.h_out.reserve(out_b);
                    uint64_t *h_m = ws2.h_out.as<uint64_t>();
                    uint32_t *h_s = reinterpret_cast<uint32_t *>(h_m + at * mw);
                    SG_CUDA_TRY(cudaMemcpyAsync(h_m, d_dst_m, at * mw * 8, cudaMemcpyDeviceToHost, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(h_s, d_dst_s, at * 4, cudaMemcpyDeviceToHost, st));
                    h->sync();
                    memcpy(R->masks, h_m, at * mw * 8);
                    memcpy(R->support, h_s, at * 4);
                } else {
                    SG_CUDA_TRY(cudaMemcpyAsync(R->masks, d_dst_m, at * mw * 8, cudaMemcpyDeviceToHost, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(R->support, d_dst_s, at * 4, cudaMemcpyDeviceToHost, st));
                    h->sync();
                }
            }
        }
    } catch (const CudaError &e) {
        sgfim_windows_result_free(R);
        return fail(h, SGFIM_EDEVICE, e.what);
    }
    // terminal roots and wave-mined windows: host copies into their slots
    for (size_t i = 0; i < root_cand_sup.size(); ++i) {
        const uint64_t w = root_cand[3 * i];
        if (!batched[w]) continue;
        uint64_t *dstm = R->masks + R->offset[w] * words;
        for (uint32_t k = 0; k < words; ++k) dstm[k] = k < 2 ? root_cand[3 * i + 1 + k] : 0;
        R->support[R->offset[w]] = root_cand_sup[i];
    }
    for (uint64_t w : wave) {
        const uint64_t c = res_cnt[w];
        if (!c) continue;
        memcpy(R->masks + R->offset[w] * words, wave_m.data() + wave_off[w] * words, c * words * 8);
        memcpy(R->support + R->offset[w], wave_s.data() + wave_off[w], c * 4);
    }
    R->offset[n_windows] = at;
    R->elapsed_s = std::chrono::duration<double>(clk::now() - t0).count();
    R->kernel_ms = kernel_ms;
    R->launches = launches;
    R->warps = task_warps;
    R->tasks = n_tasks_total;
    R->task_kernel_ms = task_kernel_ms;
    R->task_ms_max = task_ms_max;
    R->task_ms_sum = task_ms_sum;
    *out = R;
    return SGFIM_OK;
}

}  // extern "C"
