// engine.h -- internal state of an sgfim handle.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/sgfim.h"
#include "errors.h"
#include "kernels.h"

namespace sg {

// Device buffer with geometric growth; never shrinks until the handle closes.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    void reserve(size_t want, cudaStream_t st);
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// Pinned host buffer with geometric growth.
struct HostBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    void reserve(size_t want);
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

struct Dataset {
    bool loaded = false;
    uint64_t n_txn = 0;
    uint32_t n_ids = 0;          // max id + 1
    uint32_t n_present = 0;
    uint32_t id_min = 0, id_max = 0;
    uint64_t len_min = 0, len_max = 0;
    double len_mean = 0;
    std::vector<uint32_t> occ;   // occurrences per original id (duplicates counted)
    std::vector<int32_t> o2d;    // original id -> dense row (-1 absent)
    std::vector<uint32_t> d2o;   // dense row -> original id
    std::vector<uint32_t> sup;   // dense row -> support (bitmap popcount)
    uint32_t d = 0;              // bitmap rows
    uint64_t n_words = 0;        // valid words per row (even)
    uint64_t stride = 0;         // words per row (even)
    DevBuf bitmaps;
    DevBuf remap;                // int32 o2d on device (load_fimi/csr path)
    bool remap_identity = false; // bitmap loads: row = original id, remap unused
    DevBuf sup_dev;
    CUtensorMap map{};
    bool map_ok = false;
    std::string source;          // file name or "<memory>"
    // sgfim_frequent_extensions: the rows' co-occurrence matrix and dense -> original ids
    DevBuf ext_cooc, ext_d2o;
    bool ext_cooc_ready = false;
};

// Forget a dataset's contents but keep its device buffers for the next load
// (DevBuf has no destructor: assigning a fresh Dataset would leak them).
inline void reset_dataset(Dataset &ds) {
    const DevBuf bm = ds.bitmaps, remap = ds.remap, sup = ds.sup_dev, cooc = ds.ext_cooc, d2o = ds.ext_d2o;
    ds = Dataset{};
    ds.bitmaps = bm;
    ds.remap = remap;
    ds.sup_dev = sup;
    ds.ext_cooc = cooc;
    ds.ext_d2o = d2o;
}

// A device copy staged through a pinned host buffer (both grow, never shrink).
// The pinned buffer is written again only after the previous copy out of it
// has executed (an event recorded behind each copy): a caller that puts twice
// without synchronising the stream in between would otherwise overwrite bytes
// the DMA engine has not read yet.
struct Staged {
    DevBuf dev;
    HostBuf host;
    cudaEvent_t ev = nullptr;
    bool pending = false;
    template <class T> T *put(const T *src, size_t n, cudaStream_t st) {
        const size_t b = (n ? n : 1) * sizeof(T);
        if (pending) {
            cudaError_t e = cudaEventSynchronize(ev);
            if (e != cudaSuccess) throw CudaError(e, "cudaEventSynchronize", __FILE__, __LINE__);
            pending = false;
        }
        host.reserve(b);
        dev.reserve(b, st);
        if (n) {
            memcpy(host.ptr, src, n * sizeof(T));
            cudaError_t e = cudaMemcpyAsync(dev.ptr, host.ptr, n * sizeof(T), cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) throw CudaError(e, "cudaMemcpyAsync", __FILE__, __LINE__);
            if (!ev) {
                e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
                if (e != cudaSuccess) throw CudaError(e, "cudaEventCreateWithFlags", __FILE__, __LINE__);
            }
            e = cudaEventRecord(ev, st);
            if (e != cudaSuccess) throw CudaError(e, "cudaEventRecord", __FILE__, __LINE__);
            pending = true;
        }
        return dev.template as<T>();
    }
    void release() {
        if (ev) {
            if (pending) cudaEventSynchronize(ev);
            cudaEventDestroy(ev);
        }
        ev = nullptr;
        pending = false;
        dev.release();
        host.release();
    }
};

// Buffers of the batched window miner (sgfim_ring_mine_windows), kept by the
// handle across calls: per-warp workspaces, the output arena, the window
// table and its per-window results.
struct WindowWorkspace {
    DevBuf lists, lmfi, pool_m, pool_s, levels, out_m, out_s, ctrl, table, res, sub, tasks, vbuf;
    HostBuf h_table, h_res, h_out;
    void release() {
        for (DevBuf *b : {&lists, &lmfi, &pool_m, &pool_s, &levels, &out_m, &out_s, &ctrl, &table, &res, &sub, &tasks,
                          &vbuf})
            b->release();
        h_table.release();
        h_res.release();
        h_out.release();
    }
};

// Device and pinned buffers of the miner, kept by the handle across calls so
// that repeated mining (anytime stages, window services) allocates nothing
// once warm.
struct MinerWorkspace {
    DevBuf arena, pool, q_out, score, cooc, t_out, pdb, pofs, pmask, spool;
    HostBuf hq_out, hscore, ht_out;
    Staged q_ptr, q_items, q_slot, c_ptr, c_items, c_ps, c_cs, p_ptr, p_items, feat, w0, t_ptr, t_items, t_slot,
        p_items_list, s_ptr, s_items, s_cols;
    void release() {
        arena.release(); pool.release(); q_out.release(); score.release(); cooc.release(); t_out.release();
        pdb.release(); pofs.release(); pmask.release(); spool.release();
        hq_out.release(); hscore.release(); ht_out.release();
        for (Staged *s : {&q_ptr, &q_items, &q_slot, &c_ptr, &c_items, &c_ps, &c_cs, &p_ptr, &p_items, &feat, &w0,
                          &t_ptr, &t_items, &t_slot, &p_items_list, &s_ptr, &s_items, &s_cols})
            s->release();
    }
};

// Buffers of sgfim_frequent_extensions, kept by the handle across calls.
struct ExtWorkspace {
    DevBuf list, n_list, out;
    Staged ptr, rows;
    void release() {
        list.release();
        n_list.release();
        out.release();
        ptr.release();
        rows.release();
    }
};

// MLP scorer weights (device) for the learned frontier order.
struct Scorer {
    bool loaded = false;
    uint32_t in_dim = 0, hidden = 0;
    DevBuf w1, b1, w2, b2, w3, b3;
};

}  // namespace sg

struct sgfim_handle {
    int device = 0;
    int n_sm = 0;
    uint64_t hbm_budget = 0;
    uint32_t wave_nodes = 0;
    uint32_t flags = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    sg::Dataset ds;
    sg::Scorer scorer;
    // scratch
    sg::DevBuf support_scratch, cand_ptr_dev, cand_items_dev, out_dev, dev_err;
    sg::DevBuf cooc_scratch;
    sg::MinerWorkspace mws;
    sg::WindowWorkspace wws;
    sg::ExtWorkspace ext;
    sg::SupportPlan plan;
    uint64_t launches = 0;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    cudaEvent_t ev_sync = nullptr;   // blocking-sync event (SGFIM_F_BLOCKING_SYNC)
    // wait for all work queued on the handle's stream
    void sync() {
        if (ev_sync) {
            SG_CUDA_TRY(cudaEventRecord(ev_sync, stream));
            SG_CUDA_TRY(cudaEventSynchronize(ev_sync));
        } else {
            SG_CUDA_TRY(cudaStreamSynchronize(stream));
        }
    }
    // phase timers: event quads recorded by timed calls, resolved by sgfim_phase_stats_get
    struct Quad { cudaEvent_t e[4]; };
    std::vector<Quad> timer_busy, timer_free;
    sgfim_phase_stats pstats{};
    cudaEvent_t *timer_quad();
};

// Body of an exported function: CUDA, engine and host-allocation failures
// become return codes (no exception crosses the C ABI).
#define API_GUARD_BEGIN try {
#define API_GUARD_END(h)                                                   \
    }                                                                      \
    catch (const sg::CudaError &e) {                                       \
        return sg::fail(h, SGFIM_EDEVICE, e.what);                         \
    }                                                                      \
    catch (const sg::EngineError &e) {                                     \
        return sg::fail(h, e.code, e.what);                                \
    }                                                                      \
    catch (const std::bad_alloc &) {                                       \
        return sg::fail(h, SGFIM_ENOMEM, "host allocation failed");        \
    }

namespace sg {
int fail(sgfim_handle *h, int code, const std::string &msg);
int check_device_error(sgfim_handle *h);
// io.cpp
int parse_fimi_file(const char *path, std::vector<uint64_t> &row_ptr, std::vector<uint32_t> &items, std::string &err);
int write_tensorfim_file(const char *path, const sgfim_handle *h, const sgfim_result *r, const sgfim_tf_meta *m);
int write_anyfim_file(const char *path, const sgfim_handle *h, sgfim_result *const *stages, const sgfim_af_meta *m);
// miner.cu
int mine_impl(sgfim_handle *h, const sgfim_mine_params *p, const double *ckpts, uint32_t n_ckpt, sgfim_ckpt_cb cb,
              void *user, sgfim_result **out);
}  // namespace sg
