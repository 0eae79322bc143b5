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

    // per-window results: [first, count) in `found` (batched) or in `wave_sets`
    std::vector<uint64_t> res_off(n_windows, 0), res_cnt(n_windows, 0), nodes(n_windows, 0);
    std::vector<int32_t> status(n_windows, SGFIM_OK);
    std::vector<uint8_t> batched(n_windows, 0);
    std::vector<uint64_t> found_m;
    std::vector<uint32_t> found_s;
    std::vector<uint64_t> wave;   // windows for the wave miner
    double kernel_ms = 0.0;
    uint32_t launches = 0;
    try {
        SG_CUDA_TRY(cudaSetDevice(h->device));
        cudaStream_t st = h->stream;
        if (r->hm.ptr && n_windows) {
            WindowWorkspace &ws = h->wws;
            uint64_t max_len = 0;
            for (uint64_t w = 0; w < n_windows; ++w) max_len = std::max(max_len, lens[w]);
            const uint64_t list_cap = std::min<uint64_t>(std::max<uint64_t>(8192, 2 * max_len + 1024), 1ull << 30);
            const uint64_t lmfi_cap = 1u << 16, pool_cap = 1u << 16;
            const size_t per_warp = list_cap * mw * 8 + lmfi_cap * 4 + pool_cap * (mw * 8 + 4) + wmine_level_bytes(mw);
            uint64_t warps = std::min<uint64_t>((uint64_t)h->n_sm * 16, (n_windows + 3) & ~3ull);
            warps = std::min<uint64_t>(warps, std::max<uint64_t>(4, (h->hbm_budget / 2) / per_warp));
            warps = std::max<uint64_t>(4, warps & ~3ull);
            const uint64_t out_cap =
                std::max<uint64_t>(1u << 20, std::min<uint64_t>(n_windows * 32768, (h->hbm_budget / 4) / (mw * 8 + 4)));
            ws.lists.reserve(warps * list_cap * mw * 8, st);
            ws.lmfi.reserve(warps * lmfi_cap * 4, st);
            ws.pool_m.reserve(warps * pool_cap * mw * 8, st);
            ws.pool_s.reserve(warps * pool_cap * 4, st);
            ws.levels.reserve(warps * wmine_level_bytes(mw), st);
            ws.out_m.reserve(out_cap * mw * 8, st);
            ws.out_s.reserve(out_cap * 4, st);
            ws.ctrl.reserve(256, st);
            // window table: starts u64 | lens u32 | thrs u32 | order u32
            const size_t tb = n_windows * 8 + 3 * n_windows * 4;
            ws.table.reserve(tb, st);
            ws.h_table.reserve(tb);
            // results: off u64 | nodes u64 | cnt u32 | status i32
            const size_t rb = n_windows * 24;
            ws.res.reserve(rb, st);
            ws.h_res.reserve(rb);
            uint64_t *t_start = ws.h_table.as<uint64_t>();
            uint32_t *t_len = reinterpret_cast<uint32_t *>(t_start + n_windows);
            uint32_t *t_thr = t_len + n_windows;
            uint32_t *t_order = t_thr + n_windows;
            for (uint64_t w = 0; w < n_windows; ++w) {
                t_start[w] = starts[w];
                t_len[w] = (uint32_t)lens[w];
                t_thr[w] = min_counts[w] ? min_counts[w] : 1;
            }
            std::vector<uint32_t> pending(n_windows);
            for (uint64_t w = 0; w < n_windows; ++w) pending[w] = (uint32_t)w;
            // largest windows first
            std::stable_sort(pending.begin(), pending.end(), [&](uint32_t a, uint32_t b) { return lens[a] > lens[b]; });
            SG_CUDA_TRY(cudaStreamWaitEvent(st, ev, 0));
            cudaEvent_t k0, k1;
            SG_CUDA_TRY(cudaEventCreate(&k0));
            SG_CUDA_TRY(cudaEventCreate(&k1));
            struct EvPair {
                cudaEvent_t a, b;
                ~EvPair() { cudaEventDestroy(a); cudaEventDestroy(b); }
            } evp{k0, k1};
            uint64_t *d_start = ws.table.as<uint64_t>();
            uint32_t *d_len = reinterpret_cast<uint32_t *>(d_start + n_windows);
            uint32_t *d_thr = d_len + n_windows;
            uint32_t *d_order = d_thr + n_windows;
            uint64_t *d_off = ws.res.as<uint64_t>();
            uint64_t *d_nodes = d_off + n_windows;
            uint32_t *d_cnt = reinterpret_cast<uint32_t *>(d_nodes + n_windows);
            int32_t *d_status = reinterpret_cast<int32_t *>(d_cnt + n_windows);
            bool first = true;
            while (!pending.empty()) {
                memcpy(t_order, pending.data(), pending.size() * 4);
                SG_CUDA_TRY(cudaMemcpyAsync(ws.table.ptr, ws.h_table.ptr, first ? tb : 0, cudaMemcpyHostToDevice, st));
                SG_CUDA_TRY(cudaMemcpyAsync(d_order, t_order, pending.size() * 4, cudaMemcpyHostToDevice, st));
                first = false;
                SG_CUDA_TRY(cudaMemsetAsync(ws.ctrl.ptr, 0, 256, st));
                WMineParams p;
                p.hm = r->hm.as<uint64_t>();
                p.cap_mask = cap_bits - 1;
                p.d = r->d;
                p.starts = d_start;
                p.lens = d_len;
                p.thrs = d_thr;
                p.order = d_order;
                p.n_win = (uint32_t)pending.size();
                p.next = ws.ctrl.as<uint32_t>();
                p.out_pos = reinterpret_cast<unsigned long long *>(ws.ctrl.as<uint64_t>() + 1);
                p.lists = ws.lists.as<uint64_t>();
                p.list_cap = (uint32_t)list_cap;
                p.lmfi = ws.lmfi.as<uint32_t>();
                p.lmfi_cap = (uint32_t)lmfi_cap;
                p.pool_m = ws.pool_m.as<uint64_t>();
                p.pool_s = ws.pool_s.as<uint32_t>();
                p.pool_cap = (uint32_t)pool_cap;
                p.levels = ws.levels.ptr;
                p.out_m = ws.out_m.as<uint64_t>();
                p.out_s = ws.out_s.as<uint32_t>();
                p.out_cap = out_cap;
                p.win_off = d_off;
                p.win_cnt = d_cnt;
                p.win_status = d_status;
                p.win_nodes = d_nodes;
                const uint64_t use_warps = std::min<uint64_t>(warps, (pending.size() + 3) & ~3ull);
                SG_CUDA_TRY(cudaEventRecord(k0, st));
                launch_wmine(p, (int)mw, (unsigned)(use_warps / 4), st);
                SG_CUDA_TRY(cudaEventRecord(k1, st));
                ++launches;
                ++h->launches;
                SG_CUDA_TRY(cudaMemcpyAsync(ws.h_res.ptr, ws.res.ptr, rb, cudaMemcpyDeviceToHost, st));
                uint64_t used = 0;
                SG_CUDA_TRY(cudaMemcpyAsync(&used, p.out_pos, 8, cudaMemcpyDeviceToHost, st));
                h->sync();
                float ms = 0.f;
                SG_CUDA_TRY(cudaEventElapsedTime(&ms, k0, k1));
                kernel_ms += ms;
                used = std::min<uint64_t>(used, out_cap);
                const uint64_t base = found_s.size();
                found_m.resize((base + used) * mw);
                found_s.resize(base + used);
                if (used) {
                    SG_CUDA_TRY(cudaMemcpyAsync(found_m.data() + base * mw, ws.out_m.ptr, used * mw * 8,
                                                cudaMemcpyDeviceToHost, st));
                    SG_CUDA_TRY(cudaMemcpyAsync(found_s.data() + base, ws.out_s.ptr, used * 4, cudaMemcpyDeviceToHost,
                                                st));
                    h->sync();
                }
                const uint64_t *h_off = ws.h_res.as<uint64_t>();
                const uint64_t *h_nodes = h_off + n_windows;
                const uint32_t *h_cnt = reinterpret_cast<const uint32_t *>(h_nodes + n_windows);
                const int32_t *h_status = reinterpret_cast<const int32_t *>(h_cnt + n_windows);
                std::vector<uint32_t> retry;
                for (uint32_t w : pending) {
                    if (h_status[w] == 0) {
                        res_off[w] = base + h_off[w];
                        res_cnt[w] = h_cnt[w];
                        nodes[w] = h_nodes[w];
                        batched[w] = 1;
                    } else if (h_status[w] == 2) {
                        retry.push_back(w);
                    } else {
                        wave.push_back(w);
                    }
                }
                if (retry.size() == pending.size()) {
                    // nothing fitted the output arena: these go to the wave miner
                    wave.insert(wave.end(), retry.begin(), retry.end());
                    retry.clear();
                }
                pending.swap(retry);
            }
        } else {
            for (uint64_t w = 0; w < n_windows; ++w) wave.push_back(w);
        }
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }

    // windows the batched kernel did not take: load and mine each on the handle
    std::vector<uint64_t> wave_m;
    std::vector<uint32_t> wave_s;
    std::vector<uint64_t> wave_off(n_windows, 0);
    std::sort(wave.begin(), wave.end());
    for (uint64_t w : wave) {
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
        const uint64_t c = res_cnt[w];
        if (c) {
            // batched results exist only for rings of <= 128 items, where words == mw
            const uint64_t *ms = batched[w] ? found_m.data() + res_off[w] * mw : wave_m.data() + wave_off[w] * words;
            const uint32_t *ss = batched[w] ? found_s.data() + res_off[w] : wave_s.data() + wave_off[w];
            memcpy(R->masks + at * words, ms, c * words * 8);
            memcpy(R->support + at, ss, c * 4);
        }
        at += c;
        R->status[w] = status[w];
        R->nodes[w] = nodes[w];
        R->batched[w] = batched[w];
    }
    R->offset[n_windows] = at;
    R->elapsed_s = std::chrono::duration<double>(clk::now() - t0).count();
    R->kernel_ms = kernel_ms;
    R->launches = launches;
    *out = R;
    return SGFIM_OK;
}

}  // extern "C"
