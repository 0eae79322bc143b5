// miner.cu -- exact MFI search driven from the host in device waves.
//
// Reference counterparts: the engines' task-stack DFS (kernel_bitmap.cu:841-894,
// kernel_bmma.cu:875-910 "wave engine", AnytimeMining/kernel.cu:862-899) and the
// oracle miner mine_mfi (code/pipeline/skab_spike.py:84-135).  The reference
// engines enumerate every frequent itemset; this engine searches the same
// set-enumeration tree with the pruning rules of an exact MFI miner:
//
//   node (H, T):   s_e = sup(H u {e}) for e in T, counted on the device from H's
//                  tidset mask (one batched launch per wave of nodes)
//   PEP:           e with s_e == sup(H) joins H (same tidset)
//   tail order:    the remaining frequent tail F in the order's sequence
//                  (ascending support in H's context by default)
//   leaf:          F empty -> H is a candidate unless a pool member contains it
//   HUT:           H u F contained in a pool member -> no new MFI below
//   FHUT:          sup(H u F) >= thr -> H u F is the subtree's only candidate
//   children:      H u {f_i} with tail f_{i+1..}, masks built on the device,
//                  searched f_0 first
//
// The pool of candidates lives on the device as a vertical bitmap (one bit
// per candidate in every item's row), so "is Q contained in a candidate" is an
// AND-popcount query over the pool rows -- the same kernel as support counting.
// Candidates are tested against the pool as it stood when they were found, so
// the final maximality filter counts, for every candidate, the pool members
// that contain it; exactly one (itself) means the candidate is maximal.
//
// Projection: on large datasets every root subtree (the root child H = {r}
// and all its descendants) is searched on r's projected database -- each
// row restricted to the transactions holding r, packed -- so tidset masks,
// tail counts, FHUT counts and child masks are sup(r)/N as long as on the
// whole database.  Up to kProjSlots projections are resident in one buffer
// (slot p's row e is row p*d + e of it), a projection is built on the device
// when its root child is popped, and its slot is reused once no node of the
// subtree is left; a wave may hold nodes of several resident projections, and
// its queries address rows through the slot of each node's projection.
//
// The order of each node's extensions is a policy that shapes the tree (which
// items each child's tail holds, so how soon HUT and FHUT prune) but never the
// final set: canonical ascending support in the node's context; the
// reference's plain order, one global order of descending item support
// (kernel_bitmap.cu:276-283, exp_e6_cpuvec.py:65-69); or descending score of
// the loaded scoring MLP.  Any order enumerates every frequent superset of H
// inside F exactly once, and the pruning rules hold for any order.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <thread>

#include "common.cuh"
#include "engine.h"
#include "host_pool.h"

namespace sg {

void launch_mlp_forward(const float *X, uint32_t n, uint32_t F, uint32_t H, const uint16_t *W1, const float *b1,
                        const uint16_t *W2, const float *b2, const uint16_t *w3, const float *b3, float *Z1,
                        float *Z2, float *P, cudaStream_t st);

namespace {

using Clock = std::chrono::steady_clock;
constexpr uint32_t kNoNode = 0xffffffffu;
constexpr uint32_t kNoProj = 0xffffffffu;
constexpr uint32_t kProjSlots = 8;
constexpr uint32_t kDim = SGFIM_TRACE_DIM;

struct MNode {
    std::vector<uint32_t> head;  // dense ids
    std::vector<uint32_t> tail;  // dense ids, in the order's sequence
    uint32_t sup = 0;
    uint32_t slot = kNoSlot;     // tidset mask slot; kNoSlot = AND of head rows
    uint32_t id = 0;             // search-tree node id
    uint32_t proj = kNoProj;     // root item whose projected database the node's masks live in
};

struct QuerySet {
    std::vector<uint64_t> ptr{0};
    std::vector<uint32_t> items;
    std::vector<uint32_t> slot;
    void clear() { ptr.assign(1, 0); items.clear(); slot.clear(); }
    size_t size() const { return slot.size(); }
    void add(const uint32_t *it, size_t k, uint32_t s) {
        items.insert(items.end(), it, it + k);
        ptr.push_back(items.size());
        slot.push_back(s);
    }
};

// Runs fn(lo, hi) over [0, n) split into contiguous ranges on the host's cores
// (the result assembly after the search; each range writes only its own slice).
template <class F> void parallel_ranges(uint64_t n, F &&fn) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const uint64_t t = std::min<uint64_t>(std::min<uint64_t>(hw, 32), std::max<uint64_t>(1, n / 4096));
    if (t <= 1) {
        fn((uint64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(t);
    for (uint64_t i = 0; i < t; ++i) th.emplace_back([&, i] { fn(n * i / t, n * (i + 1) / t); });
    for (auto &x : th) x.join();
}

class Miner {
  public:
    Miner(sgfim_handle *h, const sgfim_mine_params &p)
        : h_(h), ds_(h->ds), p_(p), w_(h->mws), arena_(w_.arena), pool_(w_.pool), q_ptr_(w_.q_ptr),
          q_items_(w_.q_items), q_slot_(w_.q_slot), c_ptr_(w_.c_ptr), c_items_(w_.c_items), c_ps_(w_.c_ps),
          c_cs_(w_.c_cs), p_ptr_(w_.p_ptr), p_items_(w_.p_items), feat_(w_.feat), w0_(w_.w0), q_out_(w_.q_out),
          score_(w_.score), hq_out_(w_.hq_out), hscore_(w_.hscore) {}
    // (tail-count staging lives in w_: t_ptr, t_items, t_slot, t_out, ht_out)

    int run(const double *ckpts, uint32_t n_ckpt, sgfim_ckpt_cb cb, void *user, sgfim_result **out);

  private:
    sgfim_handle *h_;
    Dataset &ds_;
    sgfim_mine_params p_;
    MinerWorkspace &w_;
    uint32_t thr_ = 1;
    Clock::time_point t0_;
    // tidset masks (slots of the workspace arena)
    DevBuf &arena_;
    uint64_t slot_words_ = 0;
    std::vector<uint32_t> free_slots_;
    // the bitmap view the wave's queries read: the whole database, or the
    // buffer of resident projections (rows translated per node by prow)
    const uint64_t *vrows_ = nullptr;
    uint64_t vstride_ = 0, vwords_ = 0;
    uint32_t vd_ = 0;                    // rows of the view (queries read item indices below it)
    bool use_proj_ = false;
    uint64_t proj_stride_ = 0;
    uint32_t n_proj_slots_ = 0;
    uint64_t projections_ = 0;
    std::vector<uint32_t> slot_root_;    // projection slot -> root item (kNoProj: free)
    std::vector<int32_t> root_slot_;     // root item -> slot (-1: not resident)
    std::vector<uint32_t> live_;         // root item -> nodes of its subtree on the stack or in the wave
    std::vector<uint64_t> wp_;           // root item -> words of its projection
    void view_global() {
        vrows_ = ds_.bitmaps.as<uint64_t>();
        vstride_ = ds_.stride;
        vwords_ = ds_.n_words;
        vd_ = ds_.d;
    }
    bool make_resident(const MNode &nd);
    // row of item e for queries of node nd under the current view
    uint32_t prow(const MNode &nd, uint32_t e) const {
        return (use_proj_ && nd.proj != kNoProj) ? (uint32_t)root_slot_[nd.proj] * ds_.d + e : e;
    }
    void add_query(QuerySet &q, const MNode &nd, const uint32_t *it, size_t k, uint32_t slot) {
        if (!use_proj_ || nd.proj == kNoProj) {
            q.add(it, k, slot);
            return;
        }
        const uint32_t off = (uint32_t)root_slot_[nd.proj] * ds_.d;
        for (size_t i = 0; i < k; ++i) q.items.push_back(it[i] + off);
        q.ptr.push_back(q.items.size());
        q.slot.push_back(slot);
    }
    // device pool (rows = items, one bit per candidate), in the workspace
    DevBuf &pool_;
    uint64_t pool_words_ = 0;
    uint64_t pool_n_ = 0;
    // slot pools: for each resident projection, the candidates that hold its root
    // item (slot p's row e is row p*d + e).  Every node of a root subtree holds
    // the root item, so only those candidates can contain its HUT and leaf
    // queries, which read the slot pool instead of the whole pool.
    bool use_spool_ = false;
    uint64_t spool_words_ = 0;            // words per row
    std::vector<uint64_t> spool_n_;       // candidates in each slot's pool
    void spool_reserve(uint64_t members);
    std::vector<uint64_t> sp_ptr_, sp_cols_, sp_cnt_, sp_io_;
    std::vector<uint32_t> sp_items_;
    // candidates (host)
    std::vector<uint64_t> cptr_{0};
    std::vector<uint32_t> citems_;
    std::vector<uint32_t> citems_orig_;   // citems_ as original ids, extended at each checkpoint
    std::vector<uint32_t> csup_;
    std::vector<double> ctime_;
    std::vector<uint64_t> cexpanded_;   // nodes expanded when each candidate was emitted
    std::vector<uint32_t> cnode_;
    std::vector<uint64_t> ccheck_;   // pool size when the candidate was tested against the pool
    // search tree and trace
    std::vector<uint32_t> parent_;
    std::vector<float> tfeat_;
    std::vector<uint32_t> tnode_;
    bool need_feat_ = false;
    std::vector<uint32_t> cooc_;
    // staging (workspace)
    Staged &q_ptr_, &q_items_, &q_slot_, &c_ptr_, &c_items_, &c_ps_, &c_cs_, &p_ptr_, &p_items_, &feat_, &w0_;
    DevBuf &q_out_, &score_;
    HostBuf &hq_out_, &hscore_;
    uint64_t nodes_ = 0, waves_ = 0, launches_ = 0;
    // per-node bookkeeping of a wave (PEP, extension order, candidates, children):
    // host threads on large datasets; one (the caller) on small ones, whose waves
    // are small and whose callers may run many miners at once (one per window)
    std::unique_ptr<HostPool> hp_;
    // vectors of finished nodes, reused for new children (no allocation per node once warm)
    std::vector<std::vector<uint32_t>> spare_;
    std::vector<uint64_t> cand_freq_;   // candidates holding each dense item (pool row density)
    double phase_[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // see sgfim_result.phase_s
    // adds the wall time of f() to phase_[i]
    template <class F> void timed(int i, F &&f) {
        const auto a = Clock::now();
        f();
        phase_[i] += std::chrono::duration<double>(Clock::now() - a).count();
    }
    void add_since(int i, Clock::time_point a) { phase_[i] += std::chrono::duration<double>(Clock::now() - a).count(); }

    double elapsed() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }
    uint32_t alloc_slot() {
        if (free_slots_.empty()) return kNoSlot;
        uint32_t s = free_slots_.back();
        free_slots_.pop_back();
        return s;
    }
    void run_queries(const QuerySet &qs, const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t d,
                     int mode, std::vector<uint32_t> &out, const uint64_t *w0 = nullptr);
    void run_tail_counts(const std::vector<uint64_t> &ptr, const std::vector<uint32_t> &items,
                         const std::vector<uint32_t> &slots, std::vector<uint32_t> &out);
    void pool_reserve(uint64_t members);
    void flush_pool(uint64_t from);
    void load_cooc();
    void features(const std::vector<uint32_t> &head, uint32_t head_sup, uint32_t e, uint32_t s, uint32_t pos,
                  uint32_t nf, float *f) const;
    void score(const std::vector<float> &feat, size_t n, std::vector<float> &out);
    int finish(sgfim_result **out);
};

void Miner::run_queries(const QuerySet &qs, const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t d,
                        int mode, std::vector<uint32_t> &out, const uint64_t *w0) {
    const size_t n = qs.size();
    out.assign(n, 0);
    if (n == 0) return;
    cudaStream_t st = h_->stream;
    QueryBatch qb;
    qb.q_ptr = q_ptr_.put(qs.ptr.data(), n + 1, st);
    qb.q_items = q_items_.put(qs.items.data(), qs.items.size(), st);
    qb.mask_slot = q_slot_.put(qs.slot.data(), n, st);
    if (w0) qb.q_w0 = w0_.put(w0, n, st);
    q_out_.reserve(n * 4, st);
    hq_out_.reserve(n * 4);
    qb.rows = rows; qb.row_stride = stride; qb.n_words = n_words; qb.d = d;
    qb.arena = arena_.as<uint64_t>(); qb.arena_stride = slot_words_;
    qb.n_q = n; qb.out = q_out_.as<uint32_t>(); qb.empty_value = ds_.n_txn; qb.mode = mode;
    launch_queries(qb, st, h_->n_sm);
    ++launches_;
    SG_CUDA_TRY(cudaMemcpyAsync(hq_out_.ptr, q_out_.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    h_->sync();
    memcpy(out.data(), hq_out_.ptr, n * 4);
}

// Counts of the tail items of the wave's nodes that hold a mask: one record
// per node (its slot and tail range), one result per tail entry.
void Miner::run_tail_counts(const std::vector<uint64_t> &ptr, const std::vector<uint32_t> &items,
                            const std::vector<uint32_t> &slots, std::vector<uint32_t> &out) {
    const size_t n = items.size();
    out.resize(n);
    if (n == 0) return;
    cudaStream_t st = h_->stream;
    const uint64_t *dptr = w_.t_ptr.put(ptr.data(), ptr.size(), st);
    const uint32_t *ditems = w_.t_items.put(items.data(), n, st);
    const uint32_t *dslot = w_.t_slot.put(slots.data(), slots.size(), st);
    w_.t_out.reserve(n * 4, st);
    w_.ht_out.reserve(n * 4);
    launch_tail_counts(vrows_, vstride_, vwords_, arena_.as<uint64_t>(), slot_words_, dslot,
                       dptr, (uint32_t)slots.size(), n, ditems, w_.t_out.as<uint32_t>(), st, h_->n_sm);
    ++launches_;
    SG_CUDA_TRY(cudaMemcpyAsync(w_.ht_out.ptr, w_.t_out.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    h_->sync();
    memcpy(out.data(), w_.ht_out.ptr, n * 4);
}

// Grow the pool to hold `members` candidates.  The workspace buffer may be
// larger than one row layout needs (left over from an earlier call): the
// layout uses as many words per row as fit.
void Miner::pool_reserve(uint64_t members) {
    const uint64_t need_words = ((members + 63) / 64 + 1) & ~1ull;
    if (need_words <= pool_words_) return;
    const size_t row_bytes_have = pool_.bytes / std::max<uint32_t>(ds_.d, 1);
    uint64_t nw = std::max<uint64_t>(need_words, std::max<uint64_t>(pool_words_ * 2, 1024));
    nw = (nw + 1) & ~1ull;
    if (pool_words_ == 0 && (size_t)nw * 8 <= row_bytes_have) {
        // first use in this call: adopt the existing buffer, cleared
        pool_words_ = (row_bytes_have / 8) & ~1ull;
        SG_CUDA_TRY(cudaMemsetAsync(pool_.ptr, 0, (size_t)ds_.d * pool_words_ * 8, h_->stream));
        return;
    }
    void *np = nullptr;
    SG_CUDA_TRY(cudaMalloc(&np, (size_t)ds_.d * nw * 8));
    SG_CUDA_TRY(cudaMemsetAsync(np, 0, (size_t)ds_.d * nw * 8, h_->stream));
    if (pool_.ptr && pool_words_)
        SG_CUDA_TRY(cudaMemcpy2DAsync(np, nw * 8, pool_.ptr, pool_words_ * 8, pool_words_ * 8, ds_.d,
                                      cudaMemcpyDeviceToDevice, h_->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h_->stream));
    pool_.release();
    pool_.ptr = np;
    pool_.bytes = (size_t)ds_.d * nw * 8;
    pool_words_ = nw;
}

// Grow every slot pool's rows to hold `members` candidates (rows copied over;
// the first use in a call adopts the workspace buffer, whose slots are cleared
// when they are built).
void Miner::spool_reserve(uint64_t members) {
    // at least two words per row, also for no members: a slot is cleared over
    // the row width when it is built, so the width must exist from the first build
    const uint64_t need = std::max<uint64_t>(2, ((members + 63) / 64 + 1) & ~1ull);
    if (need <= spool_words_) return;
    const uint64_t rows = (uint64_t)n_proj_slots_ * ds_.d;
    if (spool_words_ == 0 && w_.spool.bytes >= rows * need * 8) {
        spool_words_ = (w_.spool.bytes / (rows * 8)) & ~1ull;
        return;
    }
    uint64_t nw = std::max<uint64_t>(need, std::max<uint64_t>(spool_words_ * 2, 1024));
    nw = (nw + 1) & ~1ull;
    void *np = nullptr;
    SG_CUDA_TRY(cudaMalloc(&np, rows * nw * 8));
    SG_CUDA_TRY(cudaMemsetAsync(np, 0, rows * nw * 8, h_->stream));
    if (w_.spool.ptr && spool_words_)
        SG_CUDA_TRY(cudaMemcpy2DAsync(np, nw * 8, w_.spool.ptr, spool_words_ * 8, spool_words_ * 8, rows,
                                      cudaMemcpyDeviceToDevice, h_->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h_->stream));
    w_.spool.release();
    w_.spool.ptr = np;
    w_.spool.bytes = rows * nw * 8;
    spool_words_ = nw;
}

// Append candidates [from, n) to the device pool (asynchronous; the next
// query synchronises the stream before the staging buffers are reused).
void Miner::flush_pool(uint64_t from) {
    const uint64_t n = csup_.size();
    if (from >= n) return;
    pool_reserve(n);
    const uint32_t cnt = (uint32_t)(n - from);
    std::vector<uint64_t> lp(cnt + 1);
    for (uint32_t i = 0; i <= cnt; ++i) lp[i] = cptr_[from + i] - cptr_[from];
    const uint64_t *dp = p_ptr_.put(lp.data(), cnt + 1, h_->stream);
    const uint32_t *di = p_items_.put(citems_.data() + cptr_[from], lp[cnt], h_->stream);
    launch_pool_append(pool_.as<uint64_t>(), pool_words_, dp, di, from, cnt, h_->stream);
    ++launches_;
    pool_n_ = n;
    if (!use_spool_) return;
    // each new candidate also joins the pool of every resident slot whose root it
    // holds: entries counted per candidate, positioned, then written in parallel
    // (a slot's columns are taken from its counter, in any order: a slot pool is a set)
    const uint64_t nn = n - from;
    sp_cnt_.assign(nn + 1, 0);
    hp_->run(nn, 2048, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            uint64_t k = 0;
            for (uint64_t j = cptr_[from + i]; j < cptr_[from + i + 1]; ++j) k += root_slot_[citems_[j]] >= 0;
            sp_cnt_[i + 1] = k;
        }
    });
    sp_io_.resize(nn + 1);
    sp_io_[0] = 0;
    for (uint64_t i = 0; i < nn; ++i) {
        sp_io_[i + 1] = sp_io_[i] + sp_cnt_[i + 1] * (cptr_[from + i + 1] - cptr_[from + i]);
        sp_cnt_[i + 1] += sp_cnt_[i];
    }
    const uint64_t n_ent = sp_cnt_[nn];
    if (n_ent == 0) return;
    sp_items_.resize(sp_io_[nn]);
    sp_ptr_.resize(n_ent + 1);
    sp_cols_.resize(n_ent);
    sp_ptr_[n_ent] = sp_io_[nn];
    hp_->run(nn, 2048, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            const uint64_t a = cptr_[from + i], b = cptr_[from + i + 1];
            uint64_t e = sp_cnt_[i], at = sp_io_[i];
            for (uint64_t j = a; j < b; ++j) {
                const int32_t p = root_slot_[citems_[j]];
                if (p < 0) continue;
                const uint32_t off = (uint32_t)p * ds_.d;
                sp_ptr_[e] = at;
                for (uint64_t q = a; q < b; ++q) sp_items_[at++] = citems_[q] + off;
                sp_cols_[e++] = __atomic_fetch_add(&spool_n_[p], (uint64_t)1, __ATOMIC_RELAXED);
            }
        }
    });
    spool_reserve(*std::max_element(spool_n_.begin(), spool_n_.end()));
    launch_pool_append(w_.spool.as<uint64_t>(), spool_words_, w_.s_ptr.put(sp_ptr_.data(), sp_ptr_.size(), h_->stream),
                       w_.s_items.put(sp_items_.data(), sp_items_.size(), h_->stream), 0, (uint32_t)sp_cols_.size(),
                       h_->stream, w_.s_cols.put(sp_cols_.data(), sp_cols_.size(), h_->stream));
    ++launches_;
}

void Miner::load_cooc() {
    const uint32_t d = ds_.d;
    cooc_.assign((size_t)d * d, 0);
    if (d == 0 || d > 8192) return;
    DevBuf &out = w_.cooc;
    out.reserve((size_t)d * d * 4, h_->stream);
    cooc_device(ds_.bitmaps.as<uint64_t>(), d, ds_.n_words, ds_.stride, out.as<uint32_t>(), 1, h_->stream, h_->n_sm,
                nullptr, 0, &launches_);
    SG_CUDA_TRY(cudaMemcpyAsync(cooc_.data(), out.ptr, (size_t)d * d * 4, cudaMemcpyDeviceToHost, h_->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(h_->stream));
}

// Features of the extension H -> H u {e} (the order of sgfim/mlp.py FEATURES):
// prefix support, item support, extension support (fractions of n), the
// conditional density s / sup(H), depth / 16, min and mean over h in H of
// cooc(e, h) / sup(e), and the sibling position pos / nf.
void Miner::features(const std::vector<uint32_t> &head, uint32_t head_sup, uint32_t e, uint32_t s, uint32_t pos,
                     uint32_t nf, float *f) const {
    const double n = (double)std::max<uint64_t>(ds_.n_txn, 1);
    const double se = (double)std::max<uint32_t>(ds_.sup[e], 1);
    double mn = 1.0, mean = 1.0;
    if (!head.empty() && !cooc_.empty()) {
        mn = 1.0;
        double sum = 0;
        for (uint32_t hh : head) {
            const double c = cooc_[(size_t)e * ds_.d + hh] / se;
            mn = std::min(mn, c);
            sum += c;
        }
        mean = sum / head.size();
    }
    f[0] = (float)(head_sup / n);
    f[1] = (float)(ds_.sup[e] / n);
    f[2] = (float)(s / n);
    f[3] = (float)((double)s / std::max<uint32_t>(head_sup, 1));
    f[4] = (float)(head.size() / 16.0);
    f[5] = (float)mn;
    f[6] = (float)mean;
    f[7] = (float)(nf ? (double)pos / nf : 0.0);
}

void Miner::score(const std::vector<float> &feat, size_t n, std::vector<float> &out) {
    out.assign(n, 0.f);
    if (n == 0) return;
    const Scorer &sc = h_->scorer;
    cudaStream_t st = h_->stream;
    const float *X = feat_.put(feat.data(), n * kDim, st);
    score_.reserve(n * 4, st);
    hscore_.reserve(n * 4);
    launch_mlp_forward(X, (uint32_t)n, kDim, sc.hidden, sc.w1.as<uint16_t>(), sc.b1.as<float>(), sc.w2.as<uint16_t>(),
                       sc.b2.as<float>(), sc.w3.as<uint16_t>(), sc.b3.as<float>(), nullptr, nullptr,
                       score_.as<float>(), st);
    ++launches_;
    SG_CUDA_TRY(cudaMemcpyAsync(hscore_.ptr, score_.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    h_->sync();
    memcpy(out.data(), hscore_.ptr, n * 4);
}

// Make `nd`'s root subtree resident: build its projected database (the rows of
// its head and tail items; the root item's own row becomes all ones) in a free
// slot, or in the slot of a subtree with no node left.  False when every slot
// holds a live subtree.
bool Miner::make_resident(const MNode &nd) {
    int32_t slot = -1;
    for (uint32_t p = 0; p < n_proj_slots_ && slot < 0; ++p)
        if (slot_root_[p] == kNoProj || live_[slot_root_[p]] == 0) slot = (int32_t)p;
    if (slot < 0) return false;
    if (slot_root_[slot] != kNoProj) root_slot_[slot_root_[slot]] = -1;
    cudaStream_t st = h_->stream;
    const uint32_t r = nd.proj;
    std::vector<uint32_t> items(nd.head.begin(), nd.head.end());
    items.insert(items.end(), nd.tail.begin(), nd.tail.end());
    const uint32_t *ditems = w_.p_items_list.put(items.data(), items.size(), st);
    // whole rows are cleared: a wave reads up to its widest projection, so every
    // row must be zero past its own projection's words
    launch_projection(ds_.bitmaps.as<uint64_t>(), ds_.stride, ds_.n_words, r, ditems, (uint32_t)items.size(),
                      w_.pofs.as<uint32_t>(), w_.pmask.as<uint64_t>(),
                      w_.pdb.as<uint64_t>() + (uint64_t)slot * ds_.d * proj_stride_,
                      proj_stride_, proj_stride_, ds_.d, st, h_->n_sm);
    launches_ += 3;
    ++projections_;
    if (use_spool_) {
        // the pool projected on r's pool row: every candidate so far (all are in the
        // device pool: the previous wave flushed them) that holds r
        spool_reserve(cand_freq_[r]);
        const uint64_t pw = pool_n_ ? ((pool_n_ + 63) / 64 + 1) & ~1ull : 0;
        w_.pofs.reserve(std::max<uint64_t>(pw, 1) * 4, st);
        w_.pmask.reserve(std::max<uint64_t>(pw, 1) * 6 * 8, st);
        launch_projection(pool_.as<uint64_t>(), pool_words_, pw, r, ditems, (uint32_t)items.size(),
                          w_.pofs.as<uint32_t>(), w_.pmask.as<uint64_t>(),
                          w_.spool.as<uint64_t>() + (uint64_t)slot * ds_.d * spool_words_,
                          spool_words_, spool_words_, ds_.d, st, h_->n_sm);
        launches_ += 3;
        spool_n_[slot] = cand_freq_[r];
    }
    slot_root_[slot] = r;
    root_slot_[r] = slot;
    wp_[r] = ((ds_.sup[r] + 63) / 64 + 1) & ~1ull;
    return true;
}

int Miner::run(const double *ckpts, uint32_t n_ckpt, sgfim_ckpt_cb cb, void *user, sgfim_result **out) {
    *out = nullptr;
    if (!ds_.loaded) return fail(h_, SGFIM_ESTATE, "no dataset loaded");
    if (p_.min_count < 1) return fail(h_, SGFIM_EINVAL, "min_count must be >= 1");
    if (p_.order > SGFIM_ORDER_SUPPORT_DESC) return fail(h_, SGFIM_EINVAL, "unknown order");
    if (p_.order == SGFIM_ORDER_LEARNED && !h_->scorer.loaded)
        return fail(h_, SGFIM_ESTATE, "learned order requested but no scorer loaded");
    if (p_.order == SGFIM_ORDER_LEARNED && h_->scorer.in_dim != kDim)
        return fail(h_, SGFIM_EINVAL, "scorer input width must equal SGFIM_TRACE_DIM");
    thr_ = p_.min_count;
    cand_freq_.assign(ds_.d, 0);
    t0_ = Clock::now();
    cudaStream_t st = h_->stream;
    const uint32_t d = ds_.d;
    need_feat_ = p_.order == SGFIM_ORDER_LEARNED || p_.record_trace;
    if (need_feat_) load_cooc();

    // frequent items, ascending support (ties ascending id)
    std::vector<uint32_t> freq;
    for (uint32_t e = 0; e < d; ++e)
        if (ds_.sup[e] >= thr_) freq.push_back(e);
    std::stable_sort(freq.begin(), freq.end(), [&](uint32_t a, uint32_t b) { return ds_.sup[a] < ds_.sup[b]; });

    hp_ = std::make_unique<HostPool>(
        ds_.n_words >= 2048 ? std::min(16u, std::max(1u, std::thread::hardware_concurrency())) : 1u);
    // projected root subtrees on large datasets (SGFIM_F_NO_PROJECTION / SGFIM_F_PROJECT override)
    view_global();
    use_proj_ = (h_->flags & SGFIM_F_PROJECT) ||
                (!(h_->flags & SGFIM_F_NO_PROJECTION) && ds_.n_words >= 2048 && freq.size() > 1);
    if (use_proj_) {
        uint64_t wmax = 2;
        for (uint32_t e : freq) wmax = std::max<uint64_t>(wmax, ((ds_.sup[e] + 63) / 64 + 1) & ~1ull);
        proj_stride_ = wmax;
        const uint64_t slot_bytes = (uint64_t)d * wmax * 8;
        n_proj_slots_ = (uint32_t)std::max<uint64_t>(
            1, std::min<uint64_t>(kProjSlots, (h_->hbm_budget / 8) / std::max<uint64_t>(slot_bytes, 1)));
        w_.pdb.reserve((size_t)n_proj_slots_ * slot_bytes, st);
        w_.pofs.reserve((size_t)std::max<uint64_t>(ds_.n_words, 1) * 4, st);
        w_.pmask.reserve((size_t)std::max<uint64_t>(ds_.n_words, 1) * 6 * 8, st);
        slot_root_.assign(n_proj_slots_, kNoProj);
        root_slot_.assign(d, -1);
        live_.assign(d, 0);
        wp_.assign(d, 0);
        use_spool_ = true;
        spool_n_.assign(n_proj_slots_, 0);
    }
    // mask arena
    slot_words_ = use_proj_ ? proj_stride_ : ds_.stride;
    const uint64_t slot_bytes = slot_words_ * 8;
    const uint64_t budget = h_->hbm_budget / 4;
    uint64_t max_slots = std::min<uint64_t>(1u << 20, budget / std::max<uint64_t>(slot_bytes, 1));
    // up to 256 masks per frequent item: the stack's pending children keep their
    // masks (at 64 per item, 35k children of the 2% anytime-2m search had to
    // rebuild theirs from head rows later)
    max_slots = std::min<uint64_t>(max_slots, std::max<uint64_t>(4096, (uint64_t)freq.size() * 256));
    if (max_slots < 64) max_slots = 64;
    arena_.reserve(max_slots * slot_bytes, st);
    free_slots_.resize(max_slots);
    for (uint64_t i = 0; i < max_slots; ++i) free_slots_[i] = (uint32_t)(max_slots - 1 - i);
    pool_reserve(65536);

    // nodes per wave, and tail entries per wave (16 per node); wider waves mean
    // fewer round trips and the same tree (node counts equal at 32 ... 32,768)
    const uint64_t nmax = h_->wave_nodes ? h_->wave_nodes : 32768;
    const uint64_t qmax = std::max<uint64_t>(1u << 17, nmax * 16);
    std::vector<MNode> stack;
    if (!freq.empty()) {
        MNode root;
        root.tail = freq;
        root.sup = (uint32_t)ds_.n_txn;
        root.id = 0;
        parent_.push_back(kNoNode);
        stack.push_back(std::move(root));
    }
    uint32_t next_ck = 0;
    std::vector<MNode> wave;
    QuerySet qs, qpool, qfhut, qchild;
    std::vector<uint32_t> counts, counts_q, pool_hit, fhut_cnt, tmp;
    // tail counts of nodes with a mask: concatenated tails, per-node ranges and slots
    std::vector<uint64_t> t_ptr;
    std::vector<uint32_t> t_items, t_slot;
    std::vector<std::pair<uint8_t, uint64_t>> count_src;   // per wave node: (0 tail path | 1 query path, offset)
    std::vector<float> wfeat, wscore;
    int status = SGFIM_OK;

    struct Work {
        std::vector<uint32_t> head;                    // after PEP
        std::vector<std::pair<uint32_t, uint32_t>> f;  // (support, item), ascending
        std::vector<uint32_t> pq, fq;                  // pool query (rarest row first), FHUT query rows
        int kind = 0;                                  // 0 leaf, 1 internal, 2 pruned or FHUT, 3 expands
        int emit = 0;                                  // a candidate: head (leaf) or head u F (FHUT)
        size_t pool_q = 0, fhut_q = 0, fi0 = 0;        // its queries; fi0: its FHUT rows' offset
        size_t e0 = 0, ei0 = 0;                        // its candidate's index and item offset in the wave
        size_t feat0 = 0;                              // first feature row of its extensions
        size_t kid0 = 0, nkids = 0;                    // range in the wave's kid list
    };
    std::vector<Work> work;
    std::vector<MNode> kids;
    std::vector<std::pair<uint32_t, uint32_t>> kid_src;  // (parent slot, added item)
    std::vector<uint32_t> child_slot;

    while (!stack.empty()) {
        // ---- pop a wave
        // the previous wave's nodes are done: keep their vectors for the next children
        {
            const size_t s0 = spare_.size();
            spare_.resize(s0 + 2 * wave.size());
            hp_->run(wave.size(), 2048, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t i = lo; i < hi; ++i) {
                    wave[i].head.clear();
                    wave[i].tail.clear();
                    spare_[s0 + 2 * i] = std::move(wave[i].head);
                    spare_[s0 + 2 * i + 1] = std::move(wave[i].tail);
                }
            });
        }
        wave.clear();
        uint64_t nq = 0;
        bool wave_global = !use_proj_;
        uint64_t wave_words = 0;
        while (!stack.empty() && wave.size() < nmax) {
            if (use_proj_) {
                const MNode &top = stack.back();
                if (top.proj == kNoProj) {   // the root node: the whole database
                    if (!wave.empty() && !wave_global) break;
                    wave_global = true;
                } else {
                    if (wave_global && !wave.empty()) break;
                    wave_global = false;
                    if (root_slot_[top.proj] < 0 && !make_resident(top)) break;
                    wave_words = std::max(wave_words, wp_[top.proj]);
                }
            }
            const uint64_t w = stack.back().tail.size();
            if (!wave.empty() && nq + w > qmax) break;
            nq += w;
            wave.push_back(std::move(stack.back()));
            stack.pop_back();
        }
        if (wave_global) {
            view_global();
        } else {
            vrows_ = w_.pdb.as<uint64_t>();
            vstride_ = proj_stride_;
            vwords_ = wave_words;
            vd_ = n_proj_slots_ * d;   // slot p's row e is row p * d + e
        }
        ++waves_;
        nodes_ += wave.size();
        // nodes without a mask (created when the arena was full) get
        // one rebuilt from their head rows when a slot is free
        qchild.clear();
        child_slot.clear();
        for (MNode &nd : wave) {
            if (nd.slot != kNoSlot || nd.head.empty() || nd.tail.size() < 2) continue;
            const uint32_t s = alloc_slot();
            if (s == kNoSlot) break;
            add_query(qchild, nd, nd.head.data(), nd.head.size(), kNoSlot);
            child_slot.push_back(s);
            nd.slot = s;
        }
        if (qchild.size()) {
            const size_t n = qchild.size();
            launch_child_masks(arena_.as<uint64_t>(), slot_words_, vwords_, vrows_, vstride_,
                               c_ptr_.put(qchild.ptr.data(), n + 1, st),
                               c_items_.put(qchild.items.data(), qchild.items.size(), st),
                               c_ps_.put(qchild.slot.data(), n, st), c_cs_.put(child_slot.data(), n, st), (uint32_t)n,
                               st, h_->n_sm);
            ++launches_;
        }
        // ---- phase A: s_e for every tail item (nodes with a mask: one record per node;
        // nodes without one, created while the arena was full: a query per item)
        // (positions in wave order here, the masked nodes' tail rows copied in parallel below)
        qs.clear();
        t_ptr.assign(1, 0);
        t_slot.clear();
        count_src.resize(wave.size());
        uint64_t n_ti = 0;
        for (size_t i = 0; i < wave.size(); ++i) {
            const MNode &nd = wave[i];
            if (nd.slot != kNoSlot) {
                count_src[i] = {0, n_ti};
                if (nd.tail.empty()) continue;
                n_ti += nd.tail.size();
                t_ptr.push_back(n_ti);
                t_slot.push_back(nd.slot);
            } else {
                count_src[i] = {1, qs.size()};
                for (uint32_t e : nd.tail) {
                    tmp.assign(nd.head.begin(), nd.head.end());
                    tmp.push_back(e);
                    add_query(qs, nd, tmp.data(), tmp.size(), kNoSlot);
                }
            }
        }
        t_items.resize(n_ti);
        hp_->run(wave.size(), 1024, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                const MNode &nd = wave[i];
                if (nd.slot == kNoSlot || nd.tail.empty()) continue;
                const uint32_t off = (use_proj_ && nd.proj != kNoProj) ? (uint32_t)root_slot_[nd.proj] * d : 0u;
                uint32_t *dst = t_items.data() + count_src[i].second;
                for (size_t j = 0; j < nd.tail.size(); ++j) dst[j] = nd.tail[j] + off;
            }
        });
        timed(0, [&] {
            run_tail_counts(t_ptr, t_items, t_slot, counts);
            run_queries(qs, vrows_, vstride_, vwords_, vd_, QUERY_COUNT, counts_q);
        });
        // ---- phase B: PEP, extension order, pool and FHUT queries; each node on
        // the host pool, then the query lists concatenated in wave order
        auto t_exp = Clock::now();
        if (work.size() < wave.size()) work.resize(wave.size());
        hp_->run(wave.size(), 256, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                const MNode &nd = wave[i];
                Work &wk = work[i];
                wk.head.assign(nd.head.begin(), nd.head.end());
                wk.f.clear();
                wk.emit = 0;
                wk.pool_q = wk.fhut_q = wk.feat0 = wk.kid0 = wk.nkids = 0;
                const uint32_t *cs =
                    (count_src[i].first == 0 ? counts.data() : counts_q.data()) + count_src[i].second;
                for (size_t j = 0; j < nd.tail.size(); ++j) {
                    const uint32_t s = cs[j];
                    if (s < thr_) continue;
                    if (s == nd.sup) wk.head.push_back(nd.tail[j]);
                    else wk.f.emplace_back(s, nd.tail[j]);
                }
                std::sort(wk.f.begin(), wk.f.end());
                wk.kind = wk.f.empty() ? 0 : 1;
                // FHUT: the AND of F over a masked node's mask, else of head and F
                wk.fq.clear();
                if (wk.kind == 1) {
                    const uint32_t off =
                        (use_proj_ && nd.proj != kNoProj) ? (uint32_t)root_slot_[nd.proj] * ds_.d : 0u;
                    if (nd.slot == kNoSlot)
                        for (uint32_t h : wk.head) wk.fq.push_back(h + off);
                    for (auto &pr : wk.f) wk.fq.push_back(pr.second + off);
                }
                // the pool query lists the rarest pool rows first: the device AND empties
                // sooner and stops reading rows
                wk.pq.assign(wk.head.begin(), wk.head.end());
                for (auto &pr : wk.f) wk.pq.push_back(pr.second);
                std::sort(wk.pq.begin(), wk.pq.end(),
                          [&](uint32_t x, uint32_t y) { return cand_freq_[x] < cand_freq_[y]; });
                if (use_spool_ && nd.proj != kNoProj) {
                    const uint32_t off = (uint32_t)root_slot_[nd.proj] * ds_.d;
                    for (uint32_t &x : wk.pq) x += off;
                }
            }
        });
        const bool slot_pools = use_spool_ && !wave_global;
        uint64_t spool_max = 0;   // candidates in the largest slot pool the wave reads
        uint64_t n_pi = 0, n_fi = 0;
        qpool.ptr.resize(wave.size() + 1);
        qpool.ptr[0] = 0;
        qpool.slot.assign(wave.size(), kNoSlot);
        qfhut.ptr.assign(1, 0);
        qfhut.slot.clear();
        for (size_t i = 0; i < wave.size(); ++i) {
            Work &wk = work[i];
            wk.pool_q = i;
            n_pi += wk.pq.size();
            qpool.ptr[i + 1] = n_pi;
            if (wk.kind == 1) {
                wk.fhut_q = qfhut.slot.size();
                wk.fi0 = n_fi;
                n_fi += wk.fq.size();
                qfhut.ptr.push_back(n_fi);
                qfhut.slot.push_back(wave[i].slot);
            }
            if (slot_pools) spool_max = std::max(spool_max, spool_n_[root_slot_[wave[i].proj]]);
        }
        qpool.items.resize(n_pi);
        qfhut.items.resize(n_fi);
        hp_->run(wave.size(), 1024, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                const Work &wk = work[i];
                std::copy(wk.pq.begin(), wk.pq.end(), qpool.items.begin() + qpool.ptr[i]);
                if (wk.kind == 1) std::copy(wk.fq.begin(), wk.fq.end(), qfhut.items.begin() + wk.fi0);
            }
        });
        add_since(6, t_exp);
        if (slot_pools && spool_max > 0) {
            const uint64_t pw = ((spool_max + 63) / 64 + 1) & ~1ull;
            timed(1, [&] {
                run_queries(qpool, w_.spool.as<uint64_t>(), spool_words_, pw, n_proj_slots_ * d, QUERY_ANY, pool_hit);
            });
        } else if (!slot_pools && pool_n_ > 0) {
            const uint64_t pw = ((pool_n_ + 63) / 64 + 1) & ~1ull;
            timed(1, [&] { run_queries(qpool, pool_.as<uint64_t>(), pool_words_, pw, d, QUERY_ANY, pool_hit); });
        } else {
            pool_hit.assign(qpool.size(), 0);
        }
        timed(2, [&] { run_queries(qfhut, vrows_, vstride_, vwords_, vd_, QUERY_COUNT, fhut_cnt); });
        // ---- phase C: leaf and FHUT candidates, HUT, expanding nodes
        t_exp = Clock::now();
        const uint64_t pool_before = csup_.size();
        hp_->run(wave.size(), 1024, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                Work &wk = work[i];
                if (wk.kind == 0) {
                    wk.emit = !wk.head.empty() && pool_hit[wk.pool_q] == 0;
                    continue;
                }
                wk.kind = 2;
                if (pool_hit[wk.pool_q] != 0) continue;  // HUT
                if (fhut_cnt[wk.fhut_q] >= thr_) {       // FHUT: head u F is the subtree's candidate
                    wk.emit = 1;
                    continue;
                }
                wk.kind = 3;
            }
        });
        // positions (wave order): candidates, their items, extensions (= children)
        uint64_t n_emit = 0, n_emit_items = 0, n_ext = 0;
        for (size_t i = 0; i < wave.size(); ++i) {
            Work &wk = work[i];
            if (wk.emit) {
                wk.e0 = n_emit++;
                wk.ei0 = n_emit_items;
                n_emit_items += wk.head.size() + (wk.kind == 2 ? wk.f.size() : 0);
            }
            if (wk.kind == 3) {
                wk.feat0 = wk.kid0 = n_ext;
                wk.nkids = wk.f.size();
                n_ext += wk.f.size();
            }
        }
        if (n_emit) {
            const uint64_t c0 = csup_.size(), it0 = citems_.size();
            citems_.resize(it0 + n_emit_items);
            cptr_.resize(c0 + 1 + n_emit);
            csup_.resize(c0 + n_emit);
            cnode_.resize(c0 + n_emit);
            hp_->run(wave.size(), 1024, [&](uint64_t lo, uint64_t hi) {
                std::vector<uint32_t> freq(d, 0);   // this chunk's candidates per item
                for (uint64_t i = lo; i < hi; ++i) {
                    const Work &wk = work[i];
                    if (!wk.emit) continue;
                    uint32_t *dst = citems_.data() + it0 + wk.ei0;
                    uint32_t *e = std::copy(wk.head.begin(), wk.head.end(), dst);
                    if (wk.kind == 2)
                        for (auto &pr : wk.f) *e++ = pr.second;
                    std::sort(dst, e);
                    for (const uint32_t *x = dst; x < e; ++x) ++freq[*x];
                    cptr_[c0 + 1 + wk.e0] = (uint64_t)(e - citems_.data());
                    csup_[c0 + wk.e0] = wk.kind == 2 ? fhut_cnt[wk.fhut_q] : wave[i].sup;
                    cnode_[c0 + wk.e0] = wave[i].id;
                }
                for (uint32_t x = 0; x < d; ++x)
                    if (freq[x]) __atomic_fetch_add(&cand_freq_[x], (uint64_t)freq[x], __ATOMIC_RELAXED);
            });
            ctime_.resize(c0 + n_emit, elapsed());
            cexpanded_.resize(c0 + n_emit, nodes_);
            ccheck_.resize(c0 + n_emit, pool_n_);
        }
        // features of the expanding nodes' extensions (F in ascending support; the
        // position feature is that rank)
        if (need_feat_) {
            wfeat.resize(n_ext * kDim);
            hp_->run(wave.size(), 256, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t i = lo; i < hi; ++i) {
                    const Work &wk = work[i];
                    if (wk.kind != 3) continue;
                    const size_t nf = wk.f.size();
                    for (size_t j = 0; j < nf; ++j)
                        features(wk.head, wave[i].sup, wk.f[j].second, wk.f[j].first, (uint32_t)j, (uint32_t)nf,
                                 wfeat.data() + (wk.feat0 + j) * kDim);
                }
            });
        }
        add_since(6, t_exp);
        // learned order: score every extension of the wave in one launch
        if (p_.order == SGFIM_ORDER_LEARNED) timed(4, [&] { score(wfeat, n_ext, wscore); });
        t_exp = Clock::now();
        // children in the order's sequence: the p-th extension's tail is the
        // extensions after it, and the first is searched first
        // (kids keeps its elements from wave to wave: they were moved to the stack, so
        // each is reset below; the spare vectors are handed out by position)
        if (kids.size() < n_ext) kids.resize(n_ext);
        kid_src.resize(n_ext);
        const uint64_t n_spare = std::min<uint64_t>(spare_.size() / 2, n_ext), sp0 = spare_.size() - 2 * n_spare;
        const uint64_t id0 = parent_.size(), tr0 = tnode_.size();
        parent_.resize(id0 + n_ext);
        if (p_.record_trace) {
            tfeat_.resize((tr0 + n_ext) * kDim);
            tnode_.resize(tr0 + n_ext);
        }
        hp_->run(wave.size(), 256, [&](uint64_t lo, uint64_t hi) {
            std::vector<uint32_t> rank;
            for (uint64_t i = lo; i < hi; ++i) {
                const MNode &nd = wave[i];
                const Work &wk = work[i];
                if (wk.kind != 3) continue;
                const size_t nf = wk.f.size();
                rank.resize(nf);
                std::iota(rank.begin(), rank.end(), (uint32_t)0);
                if (p_.order == SGFIM_ORDER_SUPPORT_DESC) {
                    std::sort(rank.begin(), rank.end(), [&](uint32_t a, uint32_t b) {
                        const uint32_t x = wk.f[a].second, y = wk.f[b].second;
                        return ds_.sup[x] != ds_.sup[y] ? ds_.sup[x] > ds_.sup[y] : x < y;
                    });
                } else if (p_.order == SGFIM_ORDER_LEARNED) {
                    const float *sc = wscore.data() + wk.feat0;
                    std::stable_sort(rank.begin(), rank.end(), [&](uint32_t a, uint32_t b) { return sc[a] > sc[b]; });
                }
                for (size_t p = 0; p < nf; ++p) {
                    const uint32_t j = rank[p];
                    const uint64_t k = wk.kid0 + p;
                    MNode &c = kids[k];
                    if (k < n_spare) {
                        c.head = std::move(spare_[sp0 + 2 * k]);
                        c.tail = std::move(spare_[sp0 + 2 * k + 1]);
                    }
                    c.slot = kNoSlot;
                    c.head.assign(wk.head.begin(), wk.head.end());
                    c.head.push_back(wk.f[j].second);
                    c.sup = wk.f[j].first;
                    c.tail.resize(nf - p - 1);
                    for (size_t q = p + 1; q < nf; ++q) c.tail[q - p - 1] = wk.f[rank[q]].second;
                    c.id = (uint32_t)(id0 + k);
                    c.proj = (use_proj_ && nd.proj == kNoProj) ? wk.f[j].second : nd.proj;
                    parent_[id0 + k] = nd.id;
                    if (p_.record_trace) {
                        std::copy_n(wfeat.data() + (wk.feat0 + j) * kDim, kDim, tfeat_.data() + (tr0 + k) * kDim);
                        tnode_[tr0 + k] = c.id;
                    }
                    kid_src[k] = {nd.slot, wk.f[j].second};
                }
            }
        });
        spare_.resize(sp0);
        add_since(6, t_exp);
        // child masks for the children searched next: mask(child) = mask(parent) & row(e)
        qchild.clear();
        child_slot.clear();
        for (size_t k = 0; k < n_ext; ++k) {
            MNode &c = kids[k];
            // leaves need no mask; a root child gets its mask once its projection is resident
            if (c.tail.empty() || (use_proj_ && (c.proj == kNoProj || root_slot_[c.proj] < 0))) continue;
            c.slot = alloc_slot();
            if (c.slot == kNoSlot) continue;
            if (kid_src[k].first != kNoSlot) {
                const uint32_t e = prow(c, kid_src[k].second);
                qchild.add(&e, 1, kid_src[k].first);
            } else {
                add_query(qchild, c, c.head.data(), c.head.size(), kNoSlot);
            }
            child_slot.push_back(c.slot);
        }
        if (qchild.size()) {
            const size_t n = qchild.size();
            const uint64_t *dptr = c_ptr_.put(qchild.ptr.data(), n + 1, st);
            const uint32_t *ditems = c_items_.put(qchild.items.data(), qchild.items.size(), st);
            const uint32_t *dps = c_ps_.put(qchild.slot.data(), n, st);
            const uint32_t *dcs = c_cs_.put(child_slot.data(), n, st);
            launch_child_masks(arena_.as<uint64_t>(), slot_words_, vwords_, vrows_, vstride_, dptr, ditems, dps,
                               dcs, (uint32_t)n, st, h_->n_sm);
            ++launches_;
        }
        // the stack is LIFO: push in reverse so that the wave's first node's first
        // child is popped first
        t_exp = Clock::now();
        // (the expanding nodes' kid ranges ascend in wave order, so this is the kid
        // list reversed)
        {
            const size_t sb = stack.size();
            stack.resize(sb + n_ext);
            hp_->run(n_ext, 4096, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t k = lo; k < hi; ++k) {
                    if (use_proj_ && kids[k].proj != kNoProj)
                        __atomic_fetch_add(&live_[kids[k].proj], 1u, __ATOMIC_RELAXED);
                    stack[sb + n_ext - 1 - k] = std::move(kids[k]);
                }
            });
        }
        // parents' masks are no longer needed once the child-mask kernel ran (stream order)
        for (MNode &nd : wave) {
            if (nd.slot != kNoSlot) free_slots_.push_back(nd.slot);
            if (use_proj_ && nd.proj != kNoProj) --live_[nd.proj];
        }
        add_since(6, t_exp);
        flush_pool(pool_before);
        // ---- checkpoints, limits
        const double el = elapsed();
        while (next_ck < n_ckpt && el >= ckpts[next_ck]) {
            if (cb) {
                for (size_t k = citems_orig_.size(); k < citems_.size(); ++k) citems_orig_.push_back(ds_.d2o[citems_[k]]);
                const std::vector<uint32_t> &oi = citems_orig_;
                sgfim_checkpoint ck;
                ck.t_s = ckpts[next_ck];
                ck.elapsed_s = el;
                ck.n_emitted = csup_.size();
                ck.set_ptr = cptr_.data();
                ck.items = oi.data();
                ck.support = csup_.data();
                ck.nodes = nodes_;
                if (cb(user, &ck) != 0) {
                    status = SGFIM_ECANCELED;
                    break;
                }
            }
            ++next_ck;
        }
        if (status != SGFIM_OK) break;
        if (p_.time_limit_s > 0 && el > p_.time_limit_s) {
            status = SGFIM_ETIMEDOUT;
            break;
        }
        if (p_.node_limit && nodes_ > p_.node_limit) {
            status = SGFIM_ENOMEM;
            break;
        }
    }
    SG_CUDA_TRY(cudaStreamSynchronize(st));
    if (status != SGFIM_OK) {
        h_->launches += launches_;
        return fail(h_, status, status == SGFIM_ECANCELED    ? "stopped by checkpoint callback"
                                : status == SGFIM_ETIMEDOUT ? "time limit expired"
                                                            : "node limit exceeded");
    }
    // remaining checkpoints fire once the search is complete
    if (cb && next_ck < n_ckpt) {
        const double el = elapsed();
        for (size_t k = citems_orig_.size(); k < citems_.size(); ++k) citems_orig_.push_back(ds_.d2o[citems_[k]]);
        const std::vector<uint32_t> &oi = citems_orig_;
        for (; next_ck < n_ckpt; ++next_ck) {
            sgfim_checkpoint ck;
            ck.t_s = ckpts[next_ck];
            ck.elapsed_s = el;
            ck.n_emitted = csup_.size();
            ck.set_ptr = cptr_.data();
            ck.items = oi.data();
            ck.support = csup_.data();
            ck.nodes = nodes_;
            if (cb(user, &ck) != 0) break;
        }
    }
    int rc = finish(out);
    h_->launches += launches_;
    return rc;
}

int Miner::finish(sgfim_result **out) {
    const auto t_fin = Clock::now();
    const double filter0 = phase_[3];
    const uint64_t n = csup_.size();
    // maximality filter: a candidate was already tested against every member
    // that existed when it was found, so only later members (its own bit
    // included) can contain it; two hits mean a proper superset exists
    std::vector<uint8_t> keep(n, 1);
    if (n > 1) {
        const uint64_t pw = ((pool_n_ + 63) / 64 + 1) & ~1ull;
        const uint64_t chunk = 1u << 20;
        QuerySet qs;
        std::vector<uint32_t> cnt;
        std::vector<uint64_t> w0;
        for (uint64_t a = 0; a < n; a += chunk) {
            const uint64_t b = std::min(n, a + chunk);
            // each candidate's items, rarest pool row first, built in parallel ranges
            qs.ptr.resize(b - a + 1);
            for (uint64_t c = a; c <= b; ++c) qs.ptr[c - a] = cptr_[c] - cptr_[a];
            qs.items.resize(cptr_[b] - cptr_[a]);
            qs.slot.assign(b - a, kNoSlot);
            w0.resize(b - a);
            parallel_ranges(b - a, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t c = a + lo; c < a + hi; ++c) {
                    uint32_t *dst = qs.items.data() + (cptr_[c] - cptr_[a]);
                    std::copy(citems_.begin() + cptr_[c], citems_.begin() + cptr_[c + 1], dst);
                    std::sort(dst, dst + (cptr_[c + 1] - cptr_[c]),
                              [&](uint32_t x, uint32_t y) { return cand_freq_[x] < cand_freq_[y]; });
                    w0[c - a] = ccheck_[c] / 64;
                }
            });
            timed(3, [&] { run_queries(qs, pool_.as<uint64_t>(), pool_words_, pw, ds_.d, QUERY_ANY2, cnt, w0.data()); });
            for (uint64_t c = a; c < b; ++c) keep[c] = cnt[c - a] <= 1;
        }
    }
    // trace labels: every ancestor of a node that emitted a final MFI
    std::vector<uint8_t> pos;
    if (p_.record_trace) {
        pos.assign(parent_.size(), 0);
        for (uint64_t c = 0; c < n; ++c) {
            if (!keep[c]) continue;
            for (uint32_t v = cnode_[c]; v != kNoNode && !pos[v]; v = parent_[v]) pos[v] = 1;
        }
    }
    // root rule: the highest original id of the set must be a root
    std::vector<uint8_t> is_root;
    if (p_.root_rule == SGFIM_ROOTS_LIST) {
        is_root.assign(ds_.d, 0);
        for (uint32_t i = 0; i < p_.n_roots; ++i) {
            const uint32_t id = p_.roots[i];
            if (id < ds_.n_ids && ds_.o2d[id] >= 0) is_root[ds_.o2d[id]] = 1;
        }
    } else if (p_.root_rule == SGFIM_ROOTS_MINCOUNT) {
        is_root.assign(ds_.d, 0);
        for (uint32_t e = 0; e < ds_.d; ++e) is_root[e] = ds_.occ[ds_.d2o[e]] >= p_.root_min_count;
    }
    std::vector<uint64_t> order;
    for (uint64_t c = 0; c < n; ++c) {
        if (!keep[c]) continue;
        if (!is_root.empty()) {
            const uint32_t top = citems_[cptr_[c + 1] - 1];  // dense ids ascend with original ids
            if (!is_root[top]) continue;
        }
        order.push_back(c);
    }
    // deterministic order: support descending, then items lexicographic.  A stable LSD
    // radix sort on the complemented support (four byte passes) makes runs of equal
    // support; the runs are then sorted by items, in parallel ranges of runs.
    if (n >= (1ull << 32)) {
        std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
            if (csup_[a] != csup_[b]) return csup_[a] > csup_[b];
            return std::lexicographical_compare(citems_.begin() + cptr_[a], citems_.begin() + cptr_[a + 1],
                                                citems_.begin() + cptr_[b], citems_.begin() + cptr_[b + 1]);
        });
    } else {
        // keys: complemented support above the candidate index (both 32 bits)
        const uint64_t m0 = order.size();
        std::vector<uint64_t> key(m0), tmp_k(m0);
        for (uint64_t i = 0; i < m0; ++i) key[i] = ((uint64_t)(~csup_[order[i]]) << 32) | order[i];
        uint64_t *src = key.data(), *dst = tmp_k.data();
        for (int pass = 0; pass < 4; ++pass) {
            const int sh = 32 + 8 * pass;
            uint64_t cnt[257] = {0};
            for (uint64_t i = 0; i < m0; ++i) ++cnt[(src[i] >> sh & 255u) + 1];
            for (int k = 0; k < 256; ++k) cnt[k + 1] += cnt[k];
            for (uint64_t i = 0; i < m0; ++i) dst[cnt[src[i] >> sh & 255u]++] = src[i];
            std::swap(src, dst);
        }
        // four passes: the sorted keys are back in key[]
        std::vector<uint64_t> runs{0};
        for (uint64_t i = 0; i < m0; ++i) {
            order[i] = key[i] & 0xffffffffull;
            if (i && (key[i] >> 32) != (key[i - 1] >> 32)) runs.push_back(i);
        }
        runs.push_back(m0);
        const uint64_t n_runs = runs.size() - 1;
        auto lex = [&](uint64_t a, uint64_t b) {
            return std::lexicographical_compare(citems_.begin() + cptr_[a], citems_.begin() + cptr_[a + 1],
                                                citems_.begin() + cptr_[b], citems_.begin() + cptr_[b + 1]);
        };
        // ranges of elements, each sorting the runs that start inside it (runs of low
        // supports are the long ones: splitting by run count would load one range)
        parallel_ranges(m0, [&](uint64_t lo, uint64_t hi) {
            uint64_t r = std::lower_bound(runs.begin(), runs.begin() + n_runs, lo) - runs.begin();
            for (; r < n_runs && runs[r] < hi; ++r)
                if (runs[r + 1] - runs[r] > 1) std::sort(order.begin() + runs[r], order.begin() + runs[r + 1], lex);
        });
    }
    sgfim_result *r = static_cast<sgfim_result *>(calloc(1, sizeof(sgfim_result)));
    if (!r) return fail(h_, SGFIM_ENOMEM, "result allocation failed");
    const uint64_t m = order.size();
    uint64_t total = 0;
    for (uint64_t c : order) total += cptr_[c + 1] - cptr_[c];
    r->n_sets = m;
    r->set_ptr = static_cast<uint64_t *>(malloc((m + 1) * 8));
    r->items = static_cast<uint32_t *>(malloc(std::max<uint64_t>(total, 1) * 4));
    r->support = static_cast<uint32_t *>(malloc(std::max<uint64_t>(m, 1) * 4));
    r->emit_time_s = static_cast<double *>(malloc(std::max<uint64_t>(m, 1) * 8));
    r->emit_node = static_cast<uint64_t *>(malloc(std::max<uint64_t>(m, 1) * 8));
    const uint64_t tn = p_.record_trace ? tnode_.size() : 0;
    r->trace_n = tn;
    r->trace_dim = kDim;
    r->trace_features = static_cast<float *>(malloc(std::max<uint64_t>(tn * kDim, 1) * 4));
    r->trace_labels = static_cast<uint8_t *>(malloc(std::max<uint64_t>(tn, 1)));
    if (!r->set_ptr || !r->items || !r->support || !r->emit_time_s || !r->emit_node || !r->trace_features ||
        !r->trace_labels) {
        sgfim_result_free(r);
        return fail(h_, SGFIM_ENOMEM, "result allocation failed");
    }
    r->set_ptr[0] = 0;
    for (uint64_t i = 0; i < m; ++i) r->set_ptr[i + 1] = r->set_ptr[i] + (cptr_[order[i] + 1] - cptr_[order[i]]);
    parallel_ranges(m, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            const uint64_t c = order[i];
            uint64_t at = r->set_ptr[i];
            for (uint64_t k = cptr_[c]; k < cptr_[c + 1]; ++k) r->items[at++] = ds_.d2o[citems_[k]];
            r->support[i] = csup_[c];
            r->emit_time_s[i] = ctime_[c];
            r->emit_node[i] = cexpanded_[c];
        }
    });
    if (tn) {
        memcpy(r->trace_features, tfeat_.data(), tn * kDim * 4);
        for (uint64_t t = 0; t < tn; ++t) r->trace_labels[t] = pos[tnode_[t]];
    }
    r->n_txn = ds_.n_txn;
    r->min_count = thr_;
    r->elapsed_s = elapsed();
    r->nodes = nodes_;
    r->waves = waves_;
    r->kernel_launches = launches_;
    r->candidates = n;
    add_since(7, t_fin);
    phase_[7] -= phase_[3] - filter0;
    phase_[5] = r->elapsed_s - (phase_[0] + phase_[1] + phase_[2] + phase_[3] + phase_[4] + phase_[6] + phase_[7]);
    for (int i = 0; i < 8; ++i) r->phase_s[i] = phase_[i];
    *out = r;
    return SGFIM_OK;
}

}  // namespace

int mine_impl(sgfim_handle *h, const sgfim_mine_params *p, const double *ckpts, uint32_t n_ckpt, sgfim_ckpt_cb cb,
              void *user, sgfim_result **out) {
    *out = nullptr;
    if (p->root_rule > SGFIM_ROOTS_MINCOUNT) return fail(h, SGFIM_EINVAL, "unknown root rule");
    if (p->root_rule == SGFIM_ROOTS_LIST && p->n_roots && !p->roots) return fail(h, SGFIM_EINVAL, "null roots");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    if (h->ds.n_txn == 0 || h->ds.d == 0) {
        // nothing to mine: an empty, valid result
        sgfim_result *r = static_cast<sgfim_result *>(calloc(1, sizeof(sgfim_result)));
        if (!r) return fail(h, SGFIM_ENOMEM, "result allocation failed");
        r->set_ptr = static_cast<uint64_t *>(calloc(1, 8));
        r->items = static_cast<uint32_t *>(calloc(1, 4));
        r->support = static_cast<uint32_t *>(calloc(1, 4));
        r->emit_time_s = static_cast<double *>(calloc(1, 8));
        r->emit_node = static_cast<uint64_t *>(calloc(1, 8));
        r->trace_features = static_cast<float *>(calloc(1, 4));
        r->trace_labels = static_cast<uint8_t *>(calloc(1, 1));
        r->trace_dim = kDim;
        r->n_txn = h->ds.n_txn;
        r->min_count = p->min_count;
        *out = r;
        return SGFIM_OK;
    }
    Miner m(h, *p);
    int rc = m.run(ckpts, n_ckpt, cb, user, out);
    if (rc != SGFIM_OK) return rc;
    return check_device_error(h);
}

}  // namespace sg
