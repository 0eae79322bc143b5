// kernels.h -- host-side launchers of the sgfim CUDA kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

constexpr uint32_t kNoSlot = 0xffffffffu;

// Counting modes of the streaming query kernel.  QUERY_ANY stops at the first
// set bit (result 0 / non-zero); QUERY_ANY2 stops once two bits are counted
// (result 0, 1 or >= 2).
enum QueryMode : int { QUERY_COUNT = 0, QUERY_ANY = 1, QUERY_ANY2 = 2 };

// A batch of AND-popcount queries over row-major uint64 bitmaps.
// Query q: popc(mask_q & AND_{i in items[ptr[q]..ptr[q+1])} rows[i]) over
// words [0, n_words).  mask_q is arena + mask_slot[q] * arena_stride when
// mask_slot is non-null and mask_slot[q] != kNoSlot, otherwise all ones.
// In QUERY_ANY mode the result is only guaranteed to be 0 / non-zero.
struct QueryBatch {
    const uint64_t *rows = nullptr;
    uint64_t row_stride = 0;        // words, even
    uint64_t n_words = 0;           // valid words, even (padding words are zero)
    uint32_t d = 0;                 // number of rows
    const uint64_t *q_ptr = nullptr;   // n_q + 1
    const uint32_t *q_items = nullptr;
    const uint32_t *mask_slot = nullptr;  // optional, n_q
    const uint64_t *arena = nullptr;
    uint64_t arena_stride = 0;
    uint64_t n_q = 0;
    const uint64_t *n_q_device = nullptr;  // when set, the query count is read on the device
    const uint32_t *q_index = nullptr;     // optional indirection: query j is q_index[j]
    const uint64_t *q_w0 = nullptr;        // optional first word of each query (words before it are skipped)
    uint32_t *out = nullptr;
    uint64_t empty_value = 0;       // result of an empty query without mask
    int mode = QUERY_COUNT;
};

// Launchers (all asynchronous on `st`).
void launch_transpose(const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn, const int32_t *remap,
                      uint32_t d, uint64_t *bitmaps, uint64_t stride, uint32_t *counts, cudaStream_t st,
                      int n_sm);
// host candidate CSR on the device: monotonicity check (bad |= 1) and id -> row mapping in place
void launch_cand_prep(const uint64_t *cand_ptr, uint64_t n_cand, uint32_t *items, uint64_t n_items,
                      const int32_t *remap, uint32_t n_ids, uint32_t *bad, cudaStream_t st, int n_sm);
void launch_row_popc(const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t d, uint32_t *counts,
                     cudaStream_t st);
void launch_queries(const QueryBatch &qb, cudaStream_t st, int n_sm);
// Counts of every (node, tail item) of a wave whose nodes hold a mask slot:
// out[j] = popc(arena[slot[i]] AND rows[items[j]]) for tail_ptr[i] <= j < tail_ptr[i+1].
void launch_tail_counts(const uint64_t *rows, uint64_t row_stride, uint64_t n_words, const uint64_t *arena,
                        uint64_t arena_stride, const uint32_t *slot, const uint64_t *tail_ptr, uint32_t n_nodes,
                        uint64_t n_entries, const uint32_t *items, uint32_t *out, cudaStream_t st, int n_sm);

// Batched candidate supports (config "support-1m" path).  Packs CSR candidates
// into 16-byte records when every item fits 16 bits and k <= 8, runs the
// shared-memory staged kernel on those and the streaming kernel on the rest.
enum SupportKernel : int {
    SUPPORT_AUTO = 0, SUPPORT_STAGED = 1, SUPPORT_SORTED = 2, SUPPORT_STREAM = 3, SUPPORT_STAGED4 = 4,
    SUPPORT_LANE = 5, SUPPORT_LANE_TM = 6
};
struct SupportPlan {
    int kernel = SUPPORT_AUTO;
    uint32_t cands_per_cta = 0;    // 0 = derived from the SM count
    uint32_t waves = 0;            // CTAs per SM over the grid when cands_per_cta == 0 (0 = kernel default)
};

// Scratch layout of the support path: records (16 B per candidate), the
// >8-item list, the sort permutation, the sort bins and a counter word.
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kSupportSortBins = 8 * 4096;
constexpr size_t support_scratch_bytes_for(uint64_t n) {
    return align256(n * 16) + 2 * align256(n * 4) + align256(kSupportSortBins * 4) + 256;
}
struct SupportScratch {
    // device scratch; sized by support_scratch_bytes()
    void *base = nullptr;
    size_t bytes = 0;
};
size_t support_scratch_bytes(uint64_t n_cand);
// ev (optional, 4 events): recorded before prep, before the counting kernel,
// after it, and after the >8-item tail.
int support_batch_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride,
                         uint64_t n_txn, const uint64_t *cand_ptr, const uint32_t *cand_items, uint64_t n_cand,
                         uint32_t *out, const SupportScratch &scratch, const SupportPlan &plan,
                         const CUtensorMap *map, uint32_t *dev_err, cudaStream_t st, int n_sm,
                         uint64_t *launches, cudaEvent_t *ev = nullptr);
// One lane per candidate (kernels_lane.cu): k-sorted records, chunks staged by
// TMA.  Returns -1 when d or the shared-memory layout does not fit (the caller
// then takes another kernel); otherwise the >8-item candidates are left in
// *ovf_list / *ovf_count (device) for the streaming kernel.  ev (optional):
// ev[1] and ev[2] are recorded around the counting kernel.
bool lane_supported(uint32_t d);
// The same counting with the records and totals in tensor memory and a ring of
// shared-memory box slots that loads the next chunk during the current one.
int lane_tm_supports_device(const CUtensorMap *map, uint32_t d, uint64_t n_words, const uint64_t *cand_ptr,
                            const uint32_t *cand_items, uint64_t n_cand, uint64_t n_txn, uint32_t *out, void *scratch,
                            size_t scratch_bytes, uint32_t waves, uint32_t *dev_err, cudaStream_t st, int n_sm,
                            uint32_t **ovf_list, unsigned long long **ovf_count, uint64_t *launches,
                            cudaEvent_t *ev);
int lane_supports_device(const CUtensorMap *map, uint32_t d, uint64_t n_words, const uint64_t *cand_ptr,
                         const uint32_t *cand_items, uint64_t n_cand, uint64_t n_txn, uint32_t *out, void *scratch,
                         size_t scratch_bytes, uint32_t waves, uint32_t *dev_err, cudaStream_t st, int n_sm,
                         uint32_t **ovf_list, unsigned long long **ovf_count, uint64_t *launches,
                         cudaEvent_t *ev);
// Encode the 2-D tensor map used by the staged kernel (rows x words, u64).
bool encode_bitmap_map(CUtensorMap *map, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                       uint64_t row_stride);
size_t staged_smem_bytes(uint32_t d, uint32_t cands_per_cta);

// A kernel whose mbarrier never completes: its bounded wait runs out and
// records DEVERR_MBAR_TIMEOUT in err (the wait self-test).
void launch_wait_probe(uint32_t *err, cudaStream_t st);

// Projected database of one item (the miner's root subtrees): out row e (for
// every e in items, out_words <= out_stride words, all d rows zeroed first)
// holds the bits of row e at the transactions of row root_row, packed in order.
// Scratch: ofs n_words x 4 B, masks 6 x n_words x 8 B.
void launch_projection(const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t root_row,
                       const uint32_t *items, uint32_t n_items, uint32_t *ofs, uint64_t *masks, uint64_t *out,
                       uint64_t out_stride, uint64_t out_words, uint32_t d, cudaStream_t st, int n_sm);

// Miner helpers.
// mask(child c) = (parent_slot[c] != kNoSlot ? arena[parent_slot[c]] : ones) & AND rows(items[ptr[c]..ptr[c+1]))
void launch_child_masks(uint64_t *arena, uint64_t arena_stride, uint64_t n_words, const uint64_t *rows,
                        uint64_t row_stride, const uint64_t *ptr, const uint32_t *items, const uint32_t *parent_slot,
                        const uint32_t *child_slot, uint32_t n, cudaStream_t st, int n_sm);
// Sets the bit of member m (first_member + s, or set_col[s] when given) in the
// pool row of every item of set s.
void launch_pool_append(uint64_t *pool_rows, uint64_t pool_stride, const uint64_t *set_ptr,
                        const uint32_t *set_items, uint64_t first_member, uint32_t n_sets, cudaStream_t st,
                        const uint64_t *set_col = nullptr);

// Co-occurrence (d x d) over the bitmap rows.
int cooc_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out,
                int kind, cudaStream_t st, int n_sm, void *scratch, size_t scratch_bytes, uint64_t *launches,
                uint32_t *dev_err = nullptr);
// tcgen05 e4m3 GEMM form (kernels_tc.cu); returns -1 when the layout is unusable.
// 256 x 256 blocks (two M = 128, N = 256 MMAs per K step), the AUTO form.
int cooc_tc256_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out,
                      cudaStream_t st, int n_sm, uint32_t *dev_err, uint64_t *launches);
int cooc_tc_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out,
                   cudaStream_t st, int n_sm, uint32_t *dev_err, uint64_t *launches);
size_t cooc_scratch_bytes(uint32_t d, uint64_t n_words, int kind);

// Batched window miner (kernels_wmine.cu).  A task is a whole window
// (child == kWholeWindow) or one subtree of a split window's root (child =
// index into the root's sorted frequent tail; wroot_kernel fills the root
// records first).  Per-warp workspaces are warp-major: lists list_cap x MW
// words, lmfi lmfi_cap, pool pool_cap x MW words + pool_cap supports, levels
// wmine_level_bytes(MW).  task_status: 0 done, 1 workspace overflow (mine the
// window elsewhere), 2 output arena full (retry the task).
constexpr uint32_t kWholeWindow = 0xffffffffu;
struct WMineParams {
    const uint64_t *hm = nullptr;   // ring horizontal masks [capacity][MW]
    uint64_t cap_mask = 0;          // ring capacity (transactions, power of two) - 1
    const uint64_t *ring_rows = nullptr;  // ring vertical rows [d][ring_words]
    uint64_t ring_words = 0;              // capacity / 64
    uint32_t d = 0;
    const uint64_t *starts = nullptr;   // per window
    const uint32_t *lens = nullptr;
    const uint32_t *thrs = nullptr;
    void *roots = nullptr;              // per window, wmine_root_bytes(MW) each
    const uint32_t *split_win = nullptr;
    uint32_t n_split = 0;
    void *subs = nullptr;               // split root children, wmine_root_bytes(MW) each
    const uint32_t *sub_win = nullptr;
    const uint32_t *sub_child = nullptr;
    uint32_t n_sub = 0;
    const uint32_t *task_win = nullptr;
    const uint32_t *task_child = nullptr;
    const uint32_t *task_sub = nullptr;     // null or per task: split-child record, kWholeWindow = none
    const uint32_t *task_gchild = nullptr;  // per task with a record: grandchild index, kWholeWindow = the
                                            // record's own candidate (a terminal child)
    const uint32_t *task_order = nullptr;
    uint32_t n_tasks = 0;
    uint32_t *next = nullptr;           // [0] task counter, [1] root counter, [2] split-child counter
    uint64_t *lists = nullptr;
    uint32_t list_cap = 0;
    uint32_t *lmfi = nullptr;
    uint32_t lmfi_cap = 0;
    uint64_t *pool_m = nullptr;
    uint32_t *pool_s = nullptr;
    uint32_t pool_cap = 0;
    void *levels = nullptr;
    uint64_t *out_m = nullptr;
    uint32_t *out_s = nullptr;
    unsigned long long *out_pos = nullptr;
    uint64_t out_cap = 0;
    uint64_t *task_off = nullptr;
    uint32_t *task_cnt = nullptr;
    int32_t *task_status = nullptr;
    uint64_t *task_nodes = nullptr;
    uint64_t *task_ns = nullptr;        // optional: device-clock duration of each task
    // vertical search (when set): per warp (128 + wmine_depth()) x v_words u32 -- 128 item rows over
    // the task database's entries, then one tidset per search level
    uint32_t *vbuf = nullptr;
    uint32_t v_words = 0;
};
int wmine_depth();
// resident 128-thread blocks of the task kernel per SM (registers bound it)
int wtask_blocks_per_sm(bool vertical);
// Cross-subtree maximality filter of split windows: window wi's tasks, in
// depth-first subtree order, are entries win_task0[wi] .. win_task0[wi+1]-1
// of task_of[]; task_first[entry] is the window-relative index of the task's
// first candidate and win_total[wi] the window's candidate count.
struct WFilterParams {
    uint32_t d = 0;
    uint32_t n_win = 0;
    const uint32_t *win_task0 = nullptr;
    const uint32_t *task_of = nullptr;
    const uint64_t *task_first = nullptr;
    const uint64_t *win_total = nullptr;
    const uint64_t *task_off = nullptr;
    const uint32_t *task_cnt = nullptr;
    uint32_t *task_kept = nullptr;      // in: task_cnt; out: kept
    const uint64_t *out_m = nullptr;
    uint8_t *keep = nullptr;            // per arena slot (in: 1)
    uint64_t *scratch = nullptr;        // per CTA scratch_words words
    uint64_t scratch_words = 0;
    int32_t *win_status = nullptr;      // per split window: 1 = scratch too small
    uint32_t *next = nullptr;
};
struct WGatherParams {
    uint64_t n_tasks = 0;
    const uint64_t *task_off = nullptr;
    const uint32_t *task_cnt = nullptr;
    const uint64_t *task_dst = nullptr; // ~0 = skip
    const uint8_t *keep = nullptr;      // null = keep all
    const uint64_t *out_m = nullptr;
    const uint32_t *out_s = nullptr;
    uint64_t *dst_m = nullptr;
    uint32_t *dst_s = nullptr;
};
size_t wmine_level_bytes(int mw);
size_t wmine_root_bytes(int mw);
// blocks of 128 threads (4 warps; wfilter: 256 or 1,024 threads)
void launch_wroot(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st);
void launch_wsub(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st);
void launch_wtask(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st);
void launch_wfilter(const WFilterParams &p, int mw, unsigned blocks, unsigned threads, cudaStream_t st);
void launch_wgather(const WGatherParams &p, int mw, unsigned blocks, cudaStream_t st);

}  // namespace sg
