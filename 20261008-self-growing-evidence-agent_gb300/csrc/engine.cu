// engine.cu -- C ABI of the sgfim engine: handles, loading, counting.
//
// The reference's engines are executables (kernel_bitmap.cu:796-911,
// AnytimeMining/kernel.cu:798-951) driven by engine_adapter.py over a process
// boundary.  Here the same steps are library calls on a persistent handle: the
// bitmaps stay resident in HBM between calls and every call returns a code.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "common.cuh"
#include "engine.h"

using namespace sg;

namespace sg {

void DevBuf::reserve(size_t want, cudaStream_t st) {
    (void)st;
    if (want <= bytes) return;
    size_t nb = std::max(want, bytes + bytes / 2);
    nb = (nb + 255) & ~(size_t)255;
    void *p = nullptr;
    SG_CUDA_TRY(cudaMalloc(&p, nb));
    if (ptr) SG_CUDA_TRY(cudaFree(ptr));
    ptr = p;
    bytes = nb;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

void HostBuf::reserve(size_t want) {
    if (want <= bytes) return;
    size_t nb = std::max(want, bytes + bytes / 2);
    void *p = nullptr;
    SG_CUDA_TRY(cudaMallocHost(&p, nb));
    if (ptr) cudaFreeHost(ptr);
    ptr = p;
    bytes = nb;
}

void HostBuf::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

int fail(sgfim_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

int check_device_error(sgfim_handle *h) {
    uint32_t e = 0;
    SG_CUDA_TRY(cudaMemcpyAsync(&e, h->dev_err.ptr, 4, cudaMemcpyDeviceToHost, h->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (e != DEVERR_NONE) {
        SG_CUDA_TRY(cudaMemsetAsync(h->dev_err.ptr, 0, 4, h->stream));
        return fail(h, SGFIM_EDEVICE, "device wait or bounds check failed (code " + std::to_string(e) + ")");
    }
    return SGFIM_OK;
}

}  // namespace sg

cudaEvent_t *sgfim_handle::timer_quad() {
    if (!(flags & SGFIM_F_PHASE_TIMERS)) return nullptr;
    if (timer_free.empty()) {
        Quad q;
        for (auto &e : q.e) SG_CUDA_TRY(cudaEventCreate(&e));
        timer_free.push_back(q);
    }
    timer_busy.push_back(timer_free.back());
    timer_free.pop_back();
    return timer_busy.back().e;
}


extern "C" {

int sgfim_abi_version(void) { return SGFIM_ABI_VERSION; }

int sgfim_open(const sgfim_config *cfg, sgfim_handle **out) {
    if (!out) return SGFIM_EINVAL;
    *out = nullptr;
    sgfim_handle *h = new (std::nothrow) sgfim_handle();
    if (!h) return SGFIM_ENOMEM;
    int dev = cfg ? cfg->device : 0;
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) {
        delete h;
        return SGFIM_EDEVICE;
    }
    if (dev < 0 || dev >= n_dev) {
        delete h;
        return SGFIM_EINVAL;
    }
    API_GUARD_BEGIN
    h->device = dev;
    SG_CUDA_TRY(cudaSetDevice(dev));
    SG_CUDA_TRY(cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, dev));
    SG_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    SG_CUDA_TRY(cudaEventCreate(&h->ev_a));
    SG_CUDA_TRY(cudaEventCreate(&h->ev_b));
    if (cfg && (cfg->flags & SGFIM_F_BLOCKING_SYNC))
        SG_CUDA_TRY(cudaEventCreateWithFlags(&h->ev_sync, cudaEventBlockingSync | cudaEventDisableTiming));
    size_t free_b = 0, total_b = 0;
    SG_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    h->hbm_budget = (cfg && cfg->hbm_budget) ? cfg->hbm_budget : (uint64_t)(free_b * 0.9);
    h->wave_nodes = cfg ? cfg->wave_nodes : 0;
    h->flags = cfg ? cfg->flags : 0;
    h->dev_err.reserve(256, h->stream);
    SG_CUDA_TRY(cudaMemsetAsync(h->dev_err.ptr, 0, 256, h->stream));
    const uint32_t wait_us = cfg ? cfg->wait_limit_us : 0u;
    SG_CUDA_TRY(cudaMemcpyAsync(h->dev_err.as<uint32_t>() + kCtlWaitUs, &wait_us, 4, cudaMemcpyHostToDevice,
                                h->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    *out = h;
    return SGFIM_OK;
    }
    catch (const sg::CudaError &e) {
        delete h;
        return SGFIM_EDEVICE;
    }
}

void sgfim_close(sgfim_handle *h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->ds.bitmaps.release();
    h->ds.remap.release();
    h->ds.sup_dev.release();
    h->ds.ext_cooc.release();
    h->ds.ext_d2o.release();
    h->ext.release();
    h->support_scratch.release();
    h->cand_ptr_dev.release();
    h->cand_items_dev.release();
    h->out_dev.release();
    h->dev_err.release();
    h->cooc_scratch.release();
    h->mws.release();
    h->wws.release();
    h->scorer.w1.release(); h->scorer.b1.release(); h->scorer.w2.release();
    h->scorer.b2.release(); h->scorer.w3.release(); h->scorer.b3.release();
    for (auto &q : h->timer_busy)
        for (auto &e : q.e) cudaEventDestroy(e);
    for (auto &q : h->timer_free)
        for (auto &e : q.e) cudaEventDestroy(e);
    if (h->ev_sync) cudaEventDestroy(h->ev_sync);
    if (h->ev_a) cudaEventDestroy(h->ev_a);
    if (h->ev_b) cudaEventDestroy(h->ev_b);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

const char *sgfim_last_error(const sgfim_handle *h) { return h ? h->err.c_str() : "null handle"; }

int sgfim_device_status(sgfim_handle *h, void *stream) {
    if (!h) return SGFIM_EINVAL;
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (cudaStream_t)0;
    uint32_t e = 0;
    SG_CUDA_TRY(cudaMemcpyAsync(&e, h->dev_err.as<uint32_t>() + kCtlCode, 4, cudaMemcpyDeviceToHost, st));
    SG_CUDA_TRY(cudaStreamSynchronize(st));
    if (e == DEVERR_NONE) return SGFIM_OK;
    SG_CUDA_TRY(cudaMemsetAsync(h->dev_err.as<uint32_t>() + kCtlCode, 0, 4, st));
    SG_CUDA_TRY(cudaStreamSynchronize(st));
    return fail(h, SGFIM_EDEVICE, "device wait or bounds check failed (code " + std::to_string(e) + ")");
    API_GUARD_END(h)
}

int sgfim_selftest_wait(sgfim_handle *h) {
    if (!h) return SGFIM_EINVAL;
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    launch_wait_probe(h->dev_err.as<uint32_t>(), h->stream);
    ++h->launches;
    return check_device_error(h);
    API_GUARD_END(h)
}

}  // extern "C"

// ------------------------------------------------------------------ loading
namespace {

// Build dense ids (present ids in ascending original order), upload the CSR,
// transpose on the device and read back the per-row supports.
int load_rows(sgfim_handle *h, const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn,
              const std::string &source) {
    Dataset &ds = h->ds;
    reset_dataset(ds);
    ds.source = source;
    const uint64_t n_items = n_txn ? row_ptr[n_txn] : 0;
    uint32_t max_id = 0;
    for (uint64_t j = 0; j < n_items; ++j) max_id = std::max(max_id, items[j]);
    ds.n_txn = n_txn;
    ds.n_ids = n_items ? max_id + 1 : 0;
    ds.occ.assign(ds.n_ids, 0);
    for (uint64_t j = 0; j < n_items; ++j) ds.occ[items[j]]++;
    ds.len_min = n_txn ? UINT64_MAX : 0;
    ds.len_max = 0;
    double sum = 0;
    for (uint64_t t = 0; t < n_txn; ++t) {
        const uint64_t len = row_ptr[t + 1] - row_ptr[t];
        ds.len_min = std::min(ds.len_min, len);
        ds.len_max = std::max(ds.len_max, len);
        sum += (double)len;
    }
    ds.len_mean = n_txn ? sum / (double)n_txn : 0.0;
    ds.o2d.assign(ds.n_ids, -1);
    ds.id_min = UINT32_MAX;
    for (uint32_t id = 0; id < ds.n_ids; ++id) {
        if (ds.occ[id]) {
            ds.o2d[id] = (int32_t)ds.d2o.size();
            ds.d2o.push_back(id);
            ds.id_min = std::min(ds.id_min, id);
            ds.id_max = id;
        }
    }
    if (ds.d2o.empty()) ds.id_min = 0;
    ds.n_present = (uint32_t)ds.d2o.size();
    ds.d = ds.n_present;
    const uint64_t words = (n_txn + 63) / 64;
    ds.n_words = (words + 1) & ~1ull;
    ds.stride = std::max<uint64_t>(ds.n_words, 2);
    ds.sup.assign(ds.d, 0);
    if (ds.d > 0 && n_txn > 0) {
        ds.bitmaps.reserve((size_t)ds.d * ds.stride * 8, h->stream);
        DevBuf d_ptr, d_items;
        d_ptr.reserve((n_txn + 1) * 8, h->stream);
        d_items.reserve(std::max<uint64_t>(n_items, 1) * 4, h->stream);
        ds.remap.reserve((size_t)ds.n_ids * 4, h->stream);
        ds.sup_dev.reserve((size_t)ds.d * 4, h->stream);
        SG_CUDA_TRY(cudaMemcpyAsync(d_ptr.ptr, row_ptr, (n_txn + 1) * 8, cudaMemcpyHostToDevice, h->stream));
        if (n_items)
            SG_CUDA_TRY(cudaMemcpyAsync(d_items.ptr, items, n_items * 4, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(ds.remap.ptr, ds.o2d.data(), (size_t)ds.n_ids * 4, cudaMemcpyHostToDevice,
                                    h->stream));
        launch_transpose(d_ptr.as<uint64_t>(), d_items.as<uint32_t>(), n_txn, ds.remap.as<int32_t>(), ds.d,
                         ds.bitmaps.as<uint64_t>(), ds.stride, ds.sup_dev.as<uint32_t>(), h->stream, h->n_sm);
        h->launches += 2;
        SG_CUDA_TRY(cudaMemcpyAsync(ds.sup.data(), ds.sup_dev.ptr, (size_t)ds.d * 4, cudaMemcpyDeviceToHost,
                                    h->stream));
        SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
        d_ptr.release();
        d_items.release();
        ds.map_ok = encode_bitmap_map(&ds.map, ds.bitmaps.as<uint64_t>(), ds.d, ds.n_words, ds.stride);
    }
    ds.loaded = true;
    return SGFIM_OK;
}

}  // namespace

extern "C" {

int sgfim_load_csr(sgfim_handle *h, const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn) {
    if (!h || (!row_ptr && n_txn)) return fail(h, SGFIM_EINVAL, "null argument");
    if (n_txn && row_ptr[0] != 0) return fail(h, SGFIM_EINVAL, "row_ptr[0] must be 0");
    for (uint64_t t = 0; t < n_txn; ++t)
        if (row_ptr[t + 1] < row_ptr[t]) return fail(h, SGFIM_EINVAL, "row_ptr must be non-decreasing");
    if (n_txn && row_ptr[n_txn] && !items) return fail(h, SGFIM_EINVAL, "null items");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    return load_rows(h, row_ptr, items, n_txn, "<memory>");
    API_GUARD_END(h)
}

int sgfim_load_fimi(sgfim_handle *h, const char *path) {
    if (!h || !path) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    std::vector<uint64_t> rp;
    std::vector<uint32_t> it;
    std::string err;
    int rc = parse_fimi_file(path, rp, it, err);
    if (rc != SGFIM_OK) return fail(h, rc, err);
    if (h->flags & SGFIM_F_IGNORE_ID0) {
        size_t w = 0, r = 0;
        for (size_t t = 0; t + 1 < rp.size(); ++t) {
            const size_t end = rp[t + 1];
            for (; r < end; ++r)
                if (it[r] != 0) it[w++] = it[r];
            rp[t + 1] = w;
        }
        it.resize(w);
    }
    return load_rows(h, rp.data(), it.data(), rp.size() - 1, path);
    API_GUARD_END(h)
}

int sgfim_load_bitmaps(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_txn, uint64_t n_words) {
    if (!h || (!bitmaps && d)) return fail(h, SGFIM_EINVAL, "null argument");
    if (n_words < (n_txn + 63) / 64) return fail(h, SGFIM_EINVAL, "n_words too small for n_txn");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    Dataset &ds = h->ds;
    reset_dataset(ds);
    ds.source = "<bitmaps>";
    ds.remap_identity = true;
    ds.n_txn = n_txn;
    ds.n_ids = d;
    ds.d = d;
    const uint64_t words = (n_txn + 63) / 64;
    ds.n_words = (words + 1) & ~1ull;
    ds.stride = std::max<uint64_t>(ds.n_words, 2);
    ds.sup.assign(d, 0);
    ds.o2d.resize(d);
    ds.d2o.resize(d);
    for (uint32_t e = 0; e < d; ++e) { ds.o2d[e] = (int32_t)e; ds.d2o[e] = e; }
    if (d) {
        ds.bitmaps.reserve((size_t)d * ds.stride * 8, h->stream);
        SG_CUDA_TRY(cudaMemsetAsync(ds.bitmaps.ptr, 0, (size_t)d * ds.stride * 8, h->stream));
        SG_CUDA_TRY(cudaMemcpy2DAsync(ds.bitmaps.ptr, ds.stride * 8, bitmaps, n_words * 8, words * 8, d,
                                      cudaMemcpyHostToDevice, h->stream));
        ds.sup_dev.reserve((size_t)d * 4, h->stream);
        launch_row_popc(ds.bitmaps.as<uint64_t>(), ds.stride, ds.n_words, d, ds.sup_dev.as<uint32_t>(), h->stream);
        SG_CUDA_TRY(cudaMemcpyAsync(ds.sup.data(), ds.sup_dev.ptr, (size_t)d * 4, cudaMemcpyDeviceToHost, h->stream));
        SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
        ds.map_ok = encode_bitmap_map(&ds.map, ds.bitmaps.as<uint64_t>(), d, ds.n_words, ds.stride);
    }
    // occurrence counts equal supports for bitmap input
    ds.occ = ds.sup;
    ds.id_min = UINT32_MAX;
    for (uint32_t e = 0; e < d; ++e)
        if (ds.sup[e]) { ds.n_present++; ds.id_min = std::min(ds.id_min, e); ds.id_max = e; }
    if (!ds.n_present) ds.id_min = 0;
    ds.loaded = true;
    return SGFIM_OK;
    API_GUARD_END(h)
}

int sgfim_dataset_info_get(sgfim_handle *h, sgfim_dataset_info *out) {
    if (!h || !out) return fail(h, SGFIM_EINVAL, "null argument");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    const Dataset &ds = h->ds;
    out->n_txn = ds.n_txn;
    out->n_ids = ds.n_ids;
    out->n_present = ds.n_present;
    out->id_min = ds.id_min;
    out->id_max = ds.id_max;
    out->len_min = ds.len_min;
    out->len_max = ds.len_max;
    out->len_mean = ds.len_mean;
    out->words = ds.stride;
    out->rows = ds.d;
    return SGFIM_OK;
}

int sgfim_item_counts(sgfim_handle *h, uint32_t *out, uint32_t n) {
    if (!h || (!out && n)) return fail(h, SGFIM_EINVAL, "null argument");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    for (uint32_t i = 0; i < n; ++i) out[i] = i < h->ds.occ.size() ? h->ds.occ[i] : 0;
    return SGFIM_OK;
}

// ------------------------------------------------------------------ counting
int sgfim_support_batch_device(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                               uint64_t row_stride, const uint64_t *cand_ptr, const uint32_t *cand_items,
                               uint64_t n_cand, uint32_t *out, void *stream) {
    if (!h || (n_cand && (!cand_ptr || !out)) || (d && !bitmaps)) return fail(h, SGFIM_EINVAL, "null argument");
    if (row_stride & 1) return fail(h, SGFIM_EINVAL, "row_stride must be even");
    if (n_words > row_stride) return fail(h, SGFIM_EINVAL, "n_words exceeds row_stride");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (cudaStream_t)0;
    const uint64_t n_even = (n_words + 1) & ~1ull;
    if (n_even > row_stride) return fail(h, SGFIM_EINVAL, "odd n_words needs one padding word in the row stride");
    // The tensor map is cached per (pointer, shape).
    static thread_local CUtensorMap map;
    static thread_local const void *map_ptr = nullptr;
    static thread_local uint64_t map_key[3] = {0, 0, 0};
    bool map_ok = true;
    if (map_ptr != bitmaps || map_key[0] != d || map_key[1] != n_even || map_key[2] != row_stride) {
        map_ok = encode_bitmap_map(&map, bitmaps, d, n_even, row_stride);
        map_ptr = map_ok ? bitmaps : nullptr;
        map_key[0] = d; map_key[1] = n_even; map_key[2] = row_stride;
    }
    h->support_scratch.reserve(support_scratch_bytes(n_cand), st);
    SupportScratch sc{h->support_scratch.ptr, h->support_scratch.bytes};
    const SupportPlan &plan = h->plan;
    const uint64_t n_txn = n_words * 64;
    const uint64_t before = h->launches;
    int rc = support_batch_device(bitmaps, d, n_even, row_stride, n_txn, cand_ptr, cand_items, n_cand, out, sc, plan,
                                  map_ok ? &map : nullptr, h->dev_err.as<uint32_t>(), st, h->n_sm, &h->launches,
                                  h->timer_quad());
    if (rc) return fail(h, SGFIM_ENOMEM, "support scratch too small");
    if (h->flags & SGFIM_F_PHASE_TIMERS) {
        h->pstats.calls++;
        h->pstats.launches += h->launches - before;
    }
    return SGFIM_OK;
    API_GUARD_END(h)
}

int sgfim_support_batch(sgfim_handle *h, const uint64_t *cand_ptr, const uint32_t *cand_items, uint64_t n_cand,
                        uint32_t *out) {
    if (!h || (n_cand && (!cand_ptr || !out))) return fail(h, SGFIM_EINVAL, "null argument");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    if (n_cand && cand_ptr[0] != 0) return fail(h, SGFIM_EINVAL, "cand_ptr[0] must be 0");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    Dataset &ds = h->ds;
    const uint64_t n_items = n_cand ? cand_ptr[n_cand] : 0;
    if (n_cand == 0) return SGFIM_OK;
    if (ds.d == 0 || ds.n_txn == 0) {
        for (uint64_t c = 0; c < n_cand; ++c)
            if (cand_ptr[c + 1] < cand_ptr[c]) return fail(h, SGFIM_EINVAL, "cand_ptr must be non-decreasing");
        for (uint64_t c = 0; c < n_cand; ++c) out[c] = cand_ptr[c + 1] == cand_ptr[c] ? (uint32_t)ds.n_txn : 0;
        return SGFIM_OK;
    }
    // the CSR goes to the device as given; the monotonicity check and the original id ->
    // dense row mapping (ids that never occur map past the last row: support 0) run there
    h->cand_ptr_dev.reserve((n_cand + 1) * 8 + 8, h->stream);
    h->cand_items_dev.reserve(std::max<uint64_t>(n_items, 1) * 4, h->stream);
    h->out_dev.reserve(n_cand * 4, h->stream);
    uint32_t *d_bad = reinterpret_cast<uint32_t *>(h->cand_ptr_dev.as<uint64_t>() + n_cand + 1);
    SG_CUDA_TRY(cudaMemcpyAsync(h->cand_ptr_dev.ptr, cand_ptr, (n_cand + 1) * 8, cudaMemcpyHostToDevice, h->stream));
    SG_CUDA_TRY(cudaMemsetAsync(d_bad, 0, 4, h->stream));
    if (n_items)
        SG_CUDA_TRY(cudaMemcpyAsync(h->cand_items_dev.ptr, cand_items, n_items * 4, cudaMemcpyHostToDevice,
                                    h->stream));
    launch_cand_prep(h->cand_ptr_dev.as<uint64_t>(), n_cand, h->cand_items_dev.as<uint32_t>(), n_items,
                     ds.remap_identity ? nullptr : ds.remap.as<int32_t>(), ds.n_ids, d_bad, h->stream, h->n_sm);
    ++h->launches;
    uint32_t bad_h = 0;
    SG_CUDA_TRY(cudaMemcpyAsync(&bad_h, d_bad, 4, cudaMemcpyDeviceToHost, h->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (bad_h) return fail(h, SGFIM_EINVAL, "cand_ptr must be non-decreasing");
    h->support_scratch.reserve(support_scratch_bytes(n_cand), h->stream);
    SupportScratch sc{h->support_scratch.ptr, h->support_scratch.bytes};
    const SupportPlan &plan = h->plan;
    const uint64_t before = h->launches;
    int rc = support_batch_device(ds.bitmaps.as<uint64_t>(), ds.d, ds.n_words, ds.stride, ds.n_txn,
                                  h->cand_ptr_dev.as<uint64_t>(), h->cand_items_dev.as<uint32_t>(), n_cand,
                                  h->out_dev.as<uint32_t>(), sc, plan, ds.map_ok ? &ds.map : nullptr,
                                  h->dev_err.as<uint32_t>(), h->stream, h->n_sm, &h->launches, h->timer_quad());
    if (rc) return fail(h, SGFIM_ENOMEM, "support scratch too small");
    if (h->flags & SGFIM_F_PHASE_TIMERS) {
        h->pstats.calls++;
        h->pstats.launches += h->launches - before;
    }
    SG_CUDA_TRY(cudaMemcpyAsync(out, h->out_dev.ptr, n_cand * 4, cudaMemcpyDeviceToHost, h->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return check_device_error(h);
    API_GUARD_END(h)
}

int sgfim_support_plan_set(sgfim_handle *h, int kernel, uint32_t cands_per_cta, uint32_t waves) {
    if (!h) return SGFIM_EINVAL;
    if (kernel < SGFIM_KERNEL_AUTO || kernel > SGFIM_KERNEL_LANE_TM) return fail(h, SGFIM_EINVAL, "unknown kernel");
    h->plan.kernel = kernel;
    h->plan.cands_per_cta = cands_per_cta;
    h->plan.waves = waves;
    return SGFIM_OK;
}

int sgfim_phase_stats_get(sgfim_handle *h, sgfim_phase_stats *out, int reset) {
    if (!h || !out) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    for (auto &q : h->timer_busy) {
        SG_CUDA_TRY(cudaEventSynchronize(q.e[3]));
        float a = 0, b = 0, c = 0;
        SG_CUDA_TRY(cudaEventElapsedTime(&a, q.e[0], q.e[1]));
        SG_CUDA_TRY(cudaEventElapsedTime(&b, q.e[1], q.e[2]));
        SG_CUDA_TRY(cudaEventElapsedTime(&c, q.e[2], q.e[3]));
        h->pstats.prep_ms += a;
        h->pstats.count_ms += b;
        h->pstats.tail_ms += c;
        h->timer_free.push_back(q);
    }
    h->timer_busy.clear();
    *out = h->pstats;
    if (reset) h->pstats = sgfim_phase_stats{};
    return SGFIM_OK;
    API_GUARD_END(h)
}

int sgfim_cooccurrence_device(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                              uint64_t row_stride, uint32_t *out, int kind, void *stream) {
    if (!h || (d && (!bitmaps || !out))) return fail(h, SGFIM_EINVAL, "null argument");
    if (row_stride & 1) return fail(h, SGFIM_EINVAL, "row_stride must be even");
    if (kind < 0 || kind > 4) return fail(h, SGFIM_EINVAL, "unknown co-occurrence kernel");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (cudaStream_t)0;
    // AUTO: the tcgen05 e4m3 GEMM with 256 x 256 blocks (the fastest on GB300 at
    // 1,024 x 1,024 x 2^20: 0.53 ms, against 1.29 ms with 128 x 128 tiles and 4.97 ms for the
    // CUDA-core popcount); the popcount kernel when the layout does not suit it
    int rc = -1;
    if (kind == SGFIM_COOC_AUTO) {
        rc = cooc_device(bitmaps, d, n_words, row_stride, out, SGFIM_COOC_TC_F8_256, st, h->n_sm, nullptr, 0,
                         &h->launches, h->dev_err.as<uint32_t>());
        if (rc == 0) return SGFIM_OK;
        kind = SGFIM_COOC_POPC;
    }
    const size_t sb = cooc_scratch_bytes(d, n_words, kind);
    if (sb) h->cooc_scratch.reserve(sb, st);
    rc = cooc_device(bitmaps, d, n_words, row_stride, out, kind, st, h->n_sm, h->cooc_scratch.ptr,
                     h->cooc_scratch.bytes, &h->launches, h->dev_err.as<uint32_t>());
    if (rc) return fail(h, SGFIM_EINVAL, "co-occurrence kernel unavailable for this shape");
    return SGFIM_OK;
    API_GUARD_END(h)
}

int sgfim_cooccurrence(sgfim_handle *h, uint32_t *out, uint32_t d) {
    if (!h || (!out && d)) return fail(h, SGFIM_EINVAL, "null argument");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    if (d != h->ds.d) return fail(h, SGFIM_EINVAL, "d must equal the number of bitmap rows");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    if (d == 0) return SGFIM_OK;
    h->out_dev.reserve((size_t)d * d * 4, h->stream);
    int rc = sgfim_cooccurrence_device(h, h->ds.bitmaps.as<uint64_t>(), d, h->ds.n_words, h->ds.stride,
                                       h->out_dev.as<uint32_t>(), SGFIM_COOC_AUTO, h->stream);
    if (rc) return rc;
    SG_CUDA_TRY(cudaMemcpyAsync(out, h->out_dev.ptr, (size_t)d * d * 4, cudaMemcpyDeviceToHost, h->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return check_device_error(h);
    API_GUARD_END(h)
}

// ------------------------------------------------------------------ mining
int sgfim_mine(sgfim_handle *h, const sgfim_mine_params *p, sgfim_result **out) {
    if (!h || !p || !out) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    return mine_impl(h, p, nullptr, 0, nullptr, nullptr, out);
    API_GUARD_END(h)
}

int sgfim_mine_anytime(sgfim_handle *h, const sgfim_mine_params *p, const double *checkpoints_s,
                       uint32_t n_checkpoints, sgfim_ckpt_cb cb, void *user, sgfim_result **out) {
    if (!h || !p || !out || (n_checkpoints && !checkpoints_s)) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    return mine_impl(h, p, checkpoints_s, n_checkpoints, cb, user, out);
    API_GUARD_END(h)
}

void sgfim_result_free(sgfim_result *r) {
    if (!r) return;
    free(r->set_ptr);
    free(r->items);
    free(r->support);
    free(r->emit_time_s);
    free(r->emit_node);
    free(r->trace_features);
    free(r->trace_labels);
    free(r);
}

int sgfim_write_tensorfim(sgfim_handle *h, const sgfim_result *r, const sgfim_tf_meta *meta, const char *path) {
    if (!h || !r || !path) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    int rc = write_tensorfim_file(path, h, r, meta);
    if (rc) return fail(h, rc, std::string("cannot write ") + path);
    return SGFIM_OK;
    API_GUARD_END(h)
}

int sgfim_write_anyfim(sgfim_handle *h, sgfim_result *const *stages, const sgfim_af_meta *meta, const char *path) {
    if (!h || !stages || !meta || !path) return fail(h, SGFIM_EINVAL, "null argument");
    API_GUARD_BEGIN
    int rc = write_anyfim_file(path, h, stages, meta);
    if (rc) return fail(h, rc, std::string("cannot write ") + path);
    return SGFIM_OK;
    API_GUARD_END(h)
}

}  // extern "C"
