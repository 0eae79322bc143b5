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
#include <mutex>

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
    sg::DevBuf stage_ptr, stage_items;
    sg::HostBuf hstage_ptr, hstage_items;
    std::mutex mu;
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

// Set the bits of a batch of transactions (stream positions p0 .. p0+n-1).
__global__ void ring_set_kernel(unsigned long long *__restrict__ rows, uint32_t d, uint64_t cap_words, uint64_t p0,
                                const uint64_t *__restrict__ ptr, const uint32_t *__restrict__ items, uint64_t n) {
    const uint64_t cap_bits = cap_words * 64;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = (p0 + t) & (cap_bits - 1);
        for (uint64_t j = ptr[t]; j < ptr[t + 1]; ++j) {
            const uint32_t e = items[j];
            if (e < d) atomicOr(&rows[(uint64_t)e * cap_words + (p >> 6)], 1ull << (p & 63));
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
        SG_CUDA_TRY(cudaStreamSynchronize(r->stream));
    } catch (const CudaError &) {
        r->rows.release();
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
    std::lock_guard<std::mutex> lock(r->mu);
    const uint64_t cap_bits = r->cap_words * 64;
    try {
        SG_CUDA_TRY(cudaSetDevice(r->device));
        uint64_t done = 0;
        while (done < n_txn) {
            // never append more than one ring's worth in one step
            const uint64_t n = std::min<uint64_t>(n_txn - done, cap_bits / 2);
            const uint64_t base = row_ptr[done], ni = row_ptr[done + n] - base;
            r->hstage_ptr.reserve((n + 1) * 8);
            r->hstage_items.reserve(std::max<uint64_t>(ni, 1) * 4);
            // the previous batch's copies must finish before the pinned buffers are reused
            SG_CUDA_TRY(cudaStreamSynchronize(r->stream));
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
            ring_set_kernel<<<sb, 256, 0, r->stream>>>(reinterpret_cast<unsigned long long *>(r->rows.ptr), r->d,
                                                       r->cap_words, r->head, r->stage_ptr.as<uint64_t>(),
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
        ds = Dataset{};
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

}  // extern "C"
