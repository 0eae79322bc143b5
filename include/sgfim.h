/*
 * sgfim.h -- C ABI of the GB300 maximal-frequent-itemset (MFI) engine.
 *
 * The reference drives its engines as executables
 * (code/pipeline/engine_adapter.py:70-100 runs `CoParaCG_{baseline,bmma}.exe
 * <fimi> <rel_thr>`, :115-131 runs `AnytimeMining.exe <fimi> <upto_stage>`)
 * and reads their `*=Results.txt` files back.  This library offers the same
 * path as plain C calls: a caller binds it with ctypes (or cgo/JNI/N-API)
 * and never sees a CUDA or PyTorch type.  The CLI shims built on top of it
 * write byte-compatible Results.txt files, so engine_adapter.py keeps working.
 *
 * Conventions
 *   - Return codes: SGFIM_OK (0) or a negative SGFIM_E* code; no call exits
 *     the process.  sgfim_last_error() gives the message of the last failure
 *     on a handle.
 *   - Item ids at the ABI are ORIGINAL ids (the integers of the FIMI file or
 *     the rows of a bitmap matrix).  Internally items are remapped to dense
 *     ids in ascending original-id order.
 *   - Results are allocated by the engine and released with
 *     sgfim_result_free().  Itemsets come back as CSR arrays of original ids,
 *     ascending inside each set, with uint32 supports (absolute counts).
 *   - One handle per host thread; a handle is not reentrant.  Callbacks run
 *     on the calling thread.
 *   - Every device wait inside the engine's kernels is bounded; a wait that
 *     runs out makes the call return SGFIM_EDEVICE without hanging the GPU.
 */
#ifndef SGFIM_H
#define SGFIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGFIM_ABI_VERSION 3

enum {
    SGFIM_OK = 0,
    SGFIM_EINVAL = -1,     /* bad argument */
    SGFIM_ENOMEM = -2,     /* host or device allocation failed / budget exceeded */
    SGFIM_EIO = -3,        /* file could not be read or written */
    SGFIM_EDEVICE = -4,    /* CUDA error or bounded device wait ran out */
    SGFIM_ESTATE = -5,     /* call out of order (e.g. mining before loading) */
    SGFIM_ETIMEDOUT = -6,  /* the caller's time limit expired */
    SGFIM_ECANCELED = -7,  /* a checkpoint callback asked to stop */
    SGFIM_ENODATA = -8,    /* no transactions loaded */
    SGFIM_ECAPACITY = -9   /* input larger than sgfim_support_batch_noalloc's fixed scratch */
};

typedef struct sgfim_handle sgfim_handle;

typedef struct {
    int device;               /* CUDA device ordinal */
    uint64_t hbm_budget;      /* bytes of device memory the engine may use; 0 = 90% of free */
    uint32_t wave_nodes;      /* search nodes expanded per wave; 0 = engine default */
    uint32_t flags;           /* SGFIM_F_* */
    const char *tune_cache;   /* autotuner cache file (JSON); NULL = none */
    uint32_t wait_limit_us;   /* bound of every device-side wait (an mbarrier that a TMA copy or an
                                 MMA completes), in microseconds of the GPU's global timer; a wait
                                 that runs out ends its kernel and the call returns SGFIM_EDEVICE.
                                 0 = 4,000,000 (4 s) */
} sgfim_config;

#define SGFIM_F_VERBOSE 0x1u   /* print phase timers to stderr */
#define SGFIM_F_IGNORE_ID0 0x2u /* loads drop item id 0: the TensorFIM and AnyFIM engines never
                                   use id 0 as a candidate (kernel_bitmap.cu:354-356,
                                   AnytimeMining/kernel.cu:338-341) */
#define SGFIM_F_PHASE_TIMERS 0x4u /* record per-kernel CUDA events in support-batch calls */
#define SGFIM_F_BLOCKING_SYNC 0x8u /* the miner waits for the device by sleeping, not spinning
                                      (many concurrent handles on few host cores) */
#define SGFIM_F_WINDOWS_HORIZONTAL 0x10u /* sgfim_ring_mine_windows searches each task on horizontal
                                            item masks instead of vertical rows (slower; kept for
                                            comparison) */
#define SGFIM_F_NO_PROJECTION 0x20u /* the miner searches every node on the whole database; by
                                       default a root subtree is searched on its root item's
                                       projected database once the data hold 131,072+ transactions */
#define SGFIM_F_PROJECT 0x40u      /* project root subtrees whatever the size */

/* Open a handle on a device.  Replaces the engines' process start-up
 * (kernel_bitmap.cu:796-800, AnytimeMining/kernel.cu:798-805). */
int sgfim_open(const sgfim_config *cfg, sgfim_handle **out);
void sgfim_close(sgfim_handle *h);
const char *sgfim_last_error(const sgfim_handle *h);
int sgfim_abi_version(void);

/* Device status of the asynchronous device-pointer calls
 * (sgfim_support_batch_device, sgfim_cooccurrence_device): waits for
 * `stream`, then reads and clears the handle's device error word.  Returns
 * SGFIM_OK, or SGFIM_EDEVICE when a kernel launched since the last check gave
 * up (a bounded wait ran out): the outputs of those calls are then
 * incomplete.  The calls with host buffers check it themselves.  The
 * reference has no counterpart: its kernels never wait on the device. */
int sgfim_device_status(sgfim_handle *h, void *stream);

/* Self-test of the bounded waits (no reference counterpart): launches one
 * small kernel whose mbarrier nothing ever completes, so its wait runs out
 * after the handle's wait_limit_us and records a device error.  Returns
 * SGFIM_EDEVICE (the expected result) and leaves the handle usable; use a
 * short wait_limit_us (milliseconds) for it. */
int sgfim_selftest_wait(sgfim_handle *h);

/* ---------------------------------------------------------------- loading */

/* Parse a FIMI file: one transaction per '\n', whitespace-separated
 * non-negative integers; a '-' and the digits after it are dropped; a final
 * line without '\n' counts when it holds an item.  Replaces readTransSetFile
 * (code/engine_tensorfim/code/engine/src/kernel_bitmap.cu:205-267). */
int sgfim_load_fimi(sgfim_handle *h, const char *path);

/* Load transactions from CSR host arrays of original ids:
 * transaction t holds items[row_ptr[t] .. row_ptr[t+1]).  Duplicate ids in
 * a row count once in the bitmap (the bitmap ORs bits, kernel_bitmap.cu:374-379). */
int sgfim_load_csr(sgfim_handle *h, const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn);

/* Load vertical bitmaps directly (host memory): row e (original id e,
 * 0 <= e < d) holds n_words uint64 words; bit t&63 of word t>>6 is
 * transaction t; bits at t >= n_txn must be zero. */
int sgfim_load_bitmaps(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_txn,
                       uint64_t n_words);

typedef struct {
    uint64_t n_txn;          /* transNum */
    uint32_t n_ids;          /* itemIDmax + 1 */
    uint32_t n_present;      /* distinct ids that occur (the reference's "dimension") */
    uint32_t id_min, id_max; /* itemIDmin / itemIDmax over present ids */
    uint64_t len_min, len_max; /* transaction length extremes */
    double len_mean;
    uint64_t words;          /* uint64 words per item bitmap row (padded) */
    uint32_t rows;           /* bitmap rows: present ids in ascending order (FIMI/CSR
                                loads) or every row (bitmap loads) */
} sgfim_dataset_info;

int sgfim_dataset_info_get(sgfim_handle *h, sgfim_dataset_info *out);

/* Singleton supports of ids 0..n-1 (getItemsFrequenc, kernel_bitmap.cu:269-275). */
int sgfim_item_counts(sgfim_handle *h, uint32_t *out, uint32_t n);

/* ---------------------------------------------------------------- counting */

/* Supports of n_cand itemsets given as CSR over original ids:
 * out[c] = |{t : items[cand_ptr[c]..cand_ptr[c+1]) all in t}|.
 * The batched form of getResFrequencyCuda (kernel_bitmap.cu:412-536) and of
 * the wave engine's batchCountBMMA (kernel_bmma.cu:772-872).  An empty
 * itemset has support n_txn; an id that never occurs gives 0. */
int sgfim_support_batch(sgfim_handle *h, const uint64_t *cand_ptr, const uint32_t *cand_items,
                        uint64_t n_cand, uint32_t *out);

/* Device-pointer form for callers whose data already sits in HBM.
 * bitmaps: d rows of row_stride uint64 words (row_stride even, base 16-byte
 * aligned), n_words valid words per row; cand_ptr/cand_items: CSR in device
 * memory (items are row indices); out: n_cand uint32 in device memory.
 * stream: a cudaStream_t passed as void* (NULL = legacy default stream).
 * Asynchronous: returns after enqueueing the work. */
int sgfim_support_batch_device(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                               uint64_t row_stride, const uint64_t *cand_ptr, const uint32_t *cand_items,
                               uint64_t n_cand, uint32_t *out, void *stream);

/* Pairwise co-occurrence C[i][j] = |{t : i in t and j in t}| of the loaded
 * bitmap rows (d x d uint32, row-major, host memory; d = info.rows, row i is
 * the i-th present id in ascending order for FIMI/CSR loads).  The reference's
 * equivalent is the b1 AND-POPC GEMM of bmma_bench.cu:99-152 with A = B =
 * the item bitmaps. */
int sgfim_cooccurrence(sgfim_handle *h, uint32_t *out, uint32_t d);

/* Kernel plan of the support-batch entry points (the tuning knobs; the
 * reference tunes its wave engine with environment variables instead,
 * BMMA_WAVE_CAP / BMMA_SPLITK_OFF / BMMA_MASK_WPB, kernel_bmma.cu:351-368).
 * kernel: SGFIM_KERNEL_*; cands_per_cta: candidates a CTA owns (0 = derived);
 * waves: CTAs per SM over the grid when cands_per_cta is 0 (0 = the kernel's
 * default: 1 for SORTED, 2 for STAGED). */
#define SGFIM_KERNEL_AUTO 0    /* LANE_TM when the rows fit shared memory (d <= 1,792), else STAGED4 or streaming */
#define SGFIM_KERNEL_STAGED 1  /* TMA-staged chunks, candidates in input order */
#define SGFIM_KERNEL_SORTED 2  /* TMA-staged chunks, candidates sorted by (k, first item); ids < 1024 */
#define SGFIM_KERNEL_STREAM 3  /* one warp per candidate, rows streamed from L2/HBM */
#define SGFIM_KERNEL_STAGED4 4 /* TMA-staged chunks, 4-lane groups (32 bytes of a row per lane) */
#define SGFIM_KERNEL_LANE 5    /* TMA-staged chunks, one lane per candidate, candidates sorted by k
                                  on the device; waves = CTAs per SM (default 2) */
#define SGFIM_KERNEL_LANE_TM 6 /* LANE with the candidates in tensor memory and the next chunk
                                  loaded during the current one; waves default 1 */
int sgfim_support_plan_set(sgfim_handle *h, int kernel, uint32_t cands_per_cta, uint32_t waves);

/* Allocation-free form of sgfim_support_batch_device.  It has no counterpart
 * in the reference; it exists for callers that must not allocate device
 * memory: applications whose own memory pool owns the GPU and forbids other
 * code to call cudaMalloc/cudaFree (for example a serving process that plans
 * all of its HBM at start-up), or hot loops that cannot afford cudaMalloc's
 * implicit synchronisation.  It needs no handle and allocates nothing; its
 * scratch is a fixed array in the library's device memory (about 25 MB, kept
 * by every GPU that loads the library until the process exits).
 *   - Arguments and results are those of sgfim_support_batch_device
 *     (device pointers, asynchronous on `stream`, the current CUDA device).
 *   - n_cand above SGFIM_NOALLOC_MAX_CAND returns SGFIM_ECAPACITY and does nothing.
 *   - The first call on a device looks up the array's device address with that
 *     device current; make that first call before any stream capture.
 *   - All calls share the one scratch array and it keeps the previous call's
 *     contents (the kernels clear what they need).  Calls that overlap on the
 *     GPU -- on different streams or from different host threads -- race on
 *     it and must be serialised by the caller. */
#define SGFIM_NOALLOC_MAX_CAND 1048576u
int sgfim_support_batch_noalloc(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride,
                                const uint64_t *cand_ptr, const uint32_t *cand_items, uint64_t n_cand,
                                uint32_t *out, void *stream);

/* Device status of sgfim_support_batch_noalloc on the current device: waits
 * for `stream`, reads the library's fixed device error word and clears it.
 * SGFIM_OK, or SGFIM_EDEVICE when one of the calls since the last check gave
 * up on a bounded wait (its supports are then incomplete).  The word is shared
 * by every call on the device and stays set until this call reads it.  It
 * allocates nothing.  A device reset (cudaDeviceReset) unloads the library's
 * device arrays: after one, neither no-alloc call may be used again in the
 * process. */
int sgfim_noalloc_status(void *stream);

/* Phase timers (CUDA events on the launching stream) of the batched support
 * path, enabled by SGFIM_F_PHASE_TIMERS; the counterpart of the wave engine's
 * g_tMask / g_tBmma / g_tCopy timers (kernel_bmma.cu:385,817-869).
 * sgfim_phase_stats_get waits for the recorded events, sums them over every
 * call since the last reset and optionally resets. */
typedef struct {
    uint64_t calls;          /* timed support-batch calls */
    uint64_t launches;       /* kernels launched by those calls */
    double prep_ms;          /* candidate packing */
    double count_ms;         /* the staged (or streaming) counting kernel */
    double tail_ms;          /* candidates with more than 8 items */
} sgfim_phase_stats;
int sgfim_phase_stats_get(sgfim_handle *h, sgfim_phase_stats *out, int reset);

/* Device-pointer form: bitmaps as in sgfim_support_batch_device, out d*d
 * uint32 in device memory.  kind: SGFIM_COOC_* (AUTO: the tcgen05 kernel with 256 x 256
 * blocks, or the popcount kernel when the bitmaps are not 16-byte aligned). */
#define SGFIM_COOC_AUTO 0
#define SGFIM_COOC_POPC 1     /* CUDA-core AND + popc, register tiled */
#define SGFIM_COOC_BMMA 2     /* b1 mma.sync AND-POPC on the tensor pipe */
#define SGFIM_COOC_TC_F8 3    /* tcgen05 e4m3 GEMM of 0/1 bytes, fp32 accumulate, 128 x 128 tiles */
#define SGFIM_COOC_TC_F8_256 4 /* the same with 256 x 256 blocks (two M=128, N=256 MMAs per K step) */
int sgfim_cooccurrence_device(sgfim_handle *h, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                              uint64_t row_stride, uint32_t *out, int kind, void *stream);

/* Frequent single-item extensions of n_sets itemsets (CSR over original ids):
 * bit (id & 63) of masks[s * mask_words + (id >> 6)] is set when id is not in
 * set s and sup(set s u {id}) >= min_count (0 is taken as 1).  mask_words >=
 * ceil(n_ids / 64).  An all-zero mask means the set is maximal at min_count:
 * the maximality rule of mine_mfi (code/pipeline/skab_spike.py:129-135) and
 * of the engines' leaf test (kernel_bitmap.cu:870), for any batch of sets.
 * Exact: each candidate item is first bounded by the minimum pairwise
 * co-occurrence with the set's items (computed once per dataset), and the
 * items whose bound reaches min_count are counted exactly against the set's
 * rows.  A set holding an id that never occurs has support 0 and no
 * frequent extension. */
int sgfim_frequent_extensions(sgfim_handle *h, const uint64_t *set_ptr, const uint32_t *set_items,
                              uint64_t n_sets, uint32_t min_count, uint64_t *masks, uint32_t mask_words);

/* ---------------------------------------------------------------- mining */

typedef struct {
    uint64_t n_sets;
    uint64_t *set_ptr;       /* n_sets + 1 offsets into items */
    uint32_t *items;         /* original ids, ascending inside a set */
    uint32_t *support;       /* absolute supports */
    double *emit_time_s;     /* seconds from the start of the call when each set was emitted */
    uint64_t n_txn;          /* transactions in the loaded database */
    uint32_t min_count;      /* absolute threshold used */
    double elapsed_s;        /* wall time of the mining call */
    double preprocess_s;     /* part of elapsed_s spent building bitmaps */
    uint64_t nodes;          /* search nodes expanded */
    uint64_t waves;          /* device waves */
    uint64_t kernel_launches;
    uint64_t candidates;     /* candidate MFIs emitted before the final maximality filter */
    /* search trace (sgfim_mine_params.record_trace): one row per created child
     * node -- trace_dim features (SGFIM_TRACE_DIM, see sgfim/mlp.py FEATURES) and
     * label 1 when a final MFI was emitted inside that child's subtree */
    uint64_t trace_n;
    uint32_t trace_dim;
    float *trace_features;   /* trace_n * trace_dim */
    uint8_t *trace_labels;   /* trace_n */
    /* wall time of the search phases (each device phase ends in a stream
     * synchronisation, so device time of asynchronous launches is charged to
     * the next phase): [0] extension counts, [1] pool (HUT / leaf) queries,
     * [2] FHUT counts, [3] final maximality filter, [4] scoring, [5] the rest
     * (wave assembly, staging, launches, checkpoints), [6] host expansion (PEP,
     * extension order, candidates, children), [7] result assembly after the
     * search */
    double phase_s[8];
    uint64_t *emit_node;     /* search nodes expanded when each set was emitted (a clock-free
                                measure of how early the search order reaches it) */
} sgfim_result;

#define SGFIM_TRACE_DIM 8

/* Root rules: which items may be the highest-id item of a reported MFI. */
#define SGFIM_ROOTS_ALL 0     /* every frequent item: the complete MFI set (mine_mfi, skab_spike.py:84-135) */
#define SGFIM_ROOTS_LIST 1    /* the ids in `roots` (AnyFIM stage k: the top-k ids, AnytimeMining/kernel.cu:850-859) */
#define SGFIM_ROOTS_MINCOUNT 2 /* ids with count >= root_min_count (TensorFIM: count/n > thr, kernel_bmma.cu:1199,1224-1233) */

/* Extension orders: the sequence of each search node's frequent extensions
 * f_0, f_1, ...  Child H u {f_i} gets the tail f_{i+1..} and f_0 is searched
 * first, so the order shapes the tree (how soon HUT/FHUT prune) and the
 * emission times; the final result never changes. */
#define SGFIM_ORDER_SUPPORT 0      /* canonical: ascending support in the node's context (ties: id) */
#define SGFIM_ORDER_LEARNED 1      /* descending score of the loaded scoring MLP (ties: canonical) */
#define SGFIM_ORDER_SUPPORT_DESC 2 /* plain: one global order, descending item support, ties ascending id
                                      (the reference's frequency order, kernel_bitmap.cu:276-283) */

typedef struct {
    uint32_t min_count;       /* absolute support threshold (>= 1) */
    uint32_t root_rule;       /* SGFIM_ROOTS_* */
    const uint32_t *roots;    /* SGFIM_ROOTS_LIST: original ids */
    uint32_t n_roots;
    uint32_t root_min_count;  /* SGFIM_ROOTS_MINCOUNT */
    uint32_t order;           /* SGFIM_ORDER_* */
    double time_limit_s;      /* 0 = none; expiry returns SGFIM_ETIMEDOUT */
    uint64_t node_limit;      /* 0 = none; exceeding it returns SGFIM_ENOMEM */
    uint32_t record_trace;    /* non-zero: fill the result's trace arrays */
} sgfim_mine_params;

/* Exact MFI set {M in MFI(min_count) : max(M) in roots}.  With
 * SGFIM_ROOTS_ALL this equals mine_mfi(txns, min_count=...) of
 * code/pipeline/skab_spike.py:84-135 as a set of (itemset, support). */
int sgfim_mine(sgfim_handle *h, const sgfim_mine_params *p, sgfim_result **out);

/* Anytime mining at a support floor with wall-clock checkpoints.  The
 * callback runs at each checkpoint (seconds from the call's start) with the
 * candidate MFIs emitted so far; returning non-zero stops the search
 * (SGFIM_ECANCELED).  The final result is exact; checkpoint pools hold every
 * emitted candidate, which the final maximality filter may still drop. */
typedef struct {
    double t_s;               /* checkpoint time requested */
    double elapsed_s;         /* actual time of the callback */
    uint64_t n_emitted;       /* candidates emitted so far */
    const uint64_t *set_ptr;  /* CSR of the emitted candidates (valid during the callback) */
    const uint32_t *items;
    const uint32_t *support;
    uint64_t nodes;
} sgfim_checkpoint;
typedef int (*sgfim_ckpt_cb)(void *user, const sgfim_checkpoint *ck);

int sgfim_mine_anytime(sgfim_handle *h, const sgfim_mine_params *p, const double *checkpoints_s,
                       uint32_t n_checkpoints, sgfim_ckpt_cb cb, void *user, sgfim_result **out);

void sgfim_result_free(sgfim_result *r);

/* ---------------------------------------------------------------- output */

/* Results.txt writers.  TENSORFIM: header + "List of MFIs" records sorted by
 * frequency descending (kernel_bitmap.cu:651-690), parsed by
 * engine_adapter.parse_tensorfim_results (engine_adapter.py:103-111). */
typedef struct {
    const char *trans_set_file;   /* echoed as transSetFile */
    double support_threshold;     /* relative threshold echoed in the header */
    double computation_time_s;
    double preprocessing_time_s;
    uint32_t dimension_reduced;
} sgfim_tf_meta;
int sgfim_write_tensorfim(sgfim_handle *h, const sgfim_result *r, const sgfim_tf_meta *meta, const char *path);

/* ANYFIM: per-stage sections "==== <k>th stage MFIs Number: <m> ====" and the
 * header arrays of AnytimeMining/kernel.cu:615-659, parsed by
 * engine_adapter.parse_anyfim_results (engine_adapter.py:134-166). */
typedef struct {
    const char *trans_set_file;
    uint32_t upto_stage;
    double preprocessing_time_s;
    const double *runtime_per_stage_s;    /* upto_stage values */
    const uint32_t *frequency_thr_per_stage; /* upto_stage values */
} sgfim_af_meta;
int sgfim_write_anyfim(sgfim_handle *h, sgfim_result *const *stages, const sgfim_af_meta *meta,
                       const char *path);

/* ---------------------------------------------------------------- windows */

/* Device-resident transaction ring for sliding-window mining (no reference
 * counterpart; the reference transactionises windows on the host,
 * code/pipeline/skab_spike.py:61-80, and runs one engine process per file).
 * Items are ids 0..n_items-1; the ring keeps the newest `capacity` (rounded up
 * to a power of two of 64) transactions as vertical bitmap rows on the GPU.
 * Appending a batch evicts the oldest transactions it overwrites.  Thread
 * safe: appends and window loads may come from different host threads. */
typedef struct sgfim_ring sgfim_ring;
int sgfim_ring_open(int device, uint32_t n_items, uint64_t capacity_txn, sgfim_ring **out);
void sgfim_ring_close(sgfim_ring *r);
/* Stream position of the next transaction (= transactions appended so far). */
uint64_t sgfim_ring_head(sgfim_ring *r);
uint64_t sgfim_ring_capacity(const sgfim_ring *r);
/* Append n_txn transactions (CSR over item ids; ids >= n_items are ignored). */
int sgfim_ring_append(sgfim_ring *r, const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn);
/* Make the window [start, start+len) of the stream the handle's dataset
 * (bitmaps copied on the device; rows = item ids).  The window must still be
 * in the ring: head - start <= capacity and start + len <= head. */
int sgfim_ring_window_load(sgfim_ring *r, sgfim_handle *h, uint64_t start, uint64_t len);

/* MFIs of many windows of the ring in a few batched launches (no reference
 * counterpart: the reference runs one engine process per window file).
 * Window w is [starts[w], starts[w] + lens[w]) at absolute floor
 * min_counts[w] (0 is taken as 1); its result (as a set) equals sgfim_mine on
 * sgfim_ring_window_load of the same window.  Rings of at most 128 items:
 * each window's root is expanded on the device and every root subtree (the
 * costliest ones split once more) is searched by one warp, all tasks of all
 * windows in one persistent launch; a cross-subtree filter and a device
 * gather then produce each window's MFIs, listed in depth-first order.  A
 * window whose task outgrows its warp's workspace, and every window of a
 * wider ring, is mined by the wave miner on `h` instead, so `h`'s dataset is
 * replaced.  The handle's HBM budget bounds the per-warp workspaces (half)
 * and the output arena (a quarter).  Appends from other threads may proceed
 * meanwhile; an append that would overwrite a window still being mined waits
 * for it. */
typedef struct sgfim_windows_result {
    uint64_t n_windows;
    uint32_t mask_words;   /* 64-bit words per itemset mask; bit e = item e */
    uint64_t *offset;      /* n_windows + 1: window w's MFIs are [offset[w], offset[w+1]) */
    uint64_t *masks;       /* offset[n_windows] * mask_words words */
    uint32_t *support;     /* offset[n_windows] */
    int32_t *status;       /* per window, SGFIM_OK or the wave miner's error */
    uint64_t *nodes;       /* search-tree nodes per window */
    uint8_t *batched;      /* 1 = mined by the batched kernel, 0 = by the wave miner */
    double elapsed_s;      /* whole call */
    double kernel_ms;      /* batched kernel(s), device time */
    uint32_t launches;     /* batched kernel launches */
    uint32_t warps;        /* warps of the task launch */
    uint64_t tasks;        /* search tasks (whole windows and root subtrees) */
    double task_kernel_ms; /* device time of the task launch */
    double task_ms_max;    /* longest single task (device clock) */
    double task_ms_sum;    /* all tasks' device time; / warps = mean busy time of a warp */
} sgfim_windows_result;
int sgfim_ring_mine_windows(sgfim_ring *r, sgfim_handle *h, const uint64_t *starts, const uint64_t *lens,
                            const uint32_t *min_counts, uint64_t n_windows, sgfim_windows_result **out);
void sgfim_windows_result_free(sgfim_windows_result *res);

/* ---------------------------------------------------------------- transactionisation */

/* Sensor stream -> transactions on the GPU (code/pipeline/skab_spike.py:
 * fit_bins :38-52, bin_index :55-58, window_transactions :62-80).  `values` is
 * the row-major [n_rows, n_sensors] stream (NaN-free: EINVAL otherwise),
 * `anomaly` (nullable) its per-row 0/1 flags.  Per sensor the bin edges are
 * numpy's linear-method quantiles at linspace(0, 1, n_bins+1), made unique (a
 * constant column gets [v-0.5, v+0.5]); written to edges_out[s*(n_bins+1) ..]
 * with their count in n_edges_out[s].  Windows start at 0, stride, ... while
 * start + window <= n_rows (n_windows = (n_rows - window) / stride + 1, or
 * 0); window w's transaction is one item per sensor, s * n_bins + bin of the
 * window median, in items_out[w * n_sensors + s]; labels_out[w] = max of the
 * window's flags (0 without flags).  window <= 256.  With SGFIM_TX_LOAD the
 * transactions also become the handle's dataset (as sgfim_load_csr). */
#define SGFIM_TX_LOAD 0x1u
int sgfim_transactionize(sgfim_handle *h, const double *values, uint64_t n_rows, uint32_t n_sensors,
                         const int32_t *anomaly, uint32_t window, uint32_t stride, uint32_t n_bins, uint32_t flags,
                         double *edges_out, uint32_t *n_edges_out, uint32_t *items_out, int32_t *labels_out,
                         uint64_t *n_windows_out);

/* The online (streaming) form of the same transactions
 * (code/pipeline/online_discretize.py: P2Quantile :22-71, OnlineBinner
 * :74-103, bin_index :106-108, run_file :111-128).  Every sensor keeps
 * n_bins-1 five-marker P² estimators at i/n_bins; every row of every window,
 * in window order, is fed to them (rows of overlapping windows are fed again),
 * and after each window its median is binned with the edges of that moment:
 * edges_out[(w * n_sensors + s) * (n_bins+1) ..] (nullable: not copied back),
 * items_out[w * n_sensors + s] = s * n_bins + bin, labels_out[w] as in
 * sgfim_transactionize.  Windows as in sgfim_transactionize; a stream shorter
 * than one window gives 0 windows and SGFIM_OK.  2 <= n_bins <= 64, window <=
 * 256, NaN-free values (EINVAL otherwise).  SGFIM_TX_LOAD as above.  Each
 * (sensor, estimator) is one sequential chain; SGFIM_TX_LANES(l) packs l
 * chains (1..32) into a warp, 0 (the default) picks one chain per warp until
 * the warps outnumber the SMs' schedulers.  The reference's marker rule never
 * moves the middle marker for q != 1/2 (and for q = 1/2 only until a sample
 * falls between markers 1 and 3), so a chain stops stepping once its estimate
 * can no longer change; SGFIM_TX_P2_FULL runs every step instead (same
 * results). */
#define SGFIM_TX_LANES(l) (((uint32_t)(l) & 63u) << 8)
#define SGFIM_TX_P2_FULL 0x2u
int sgfim_transactionize_online(sgfim_handle *h, const double *values, uint64_t n_rows, uint32_t n_sensors,
                                const int32_t *anomaly, uint32_t window, uint32_t stride, uint32_t n_bins,
                                uint32_t flags, double *edges_out, uint32_t *items_out, int32_t *labels_out,
                                uint64_t *n_windows_out);

/* ---------------------------------------------------------------- scoring */

/* Load the frontier-scoring MLP used by SGFIM_ORDER_LEARNED: 3 layers,
 * in_dim -> hidden -> hidden -> 1, bf16 weights (row-major [out][in]) and
 * fp32 biases, ReLU between layers, sigmoid output. */
int sgfim_load_scorer(sgfim_handle *h, uint32_t in_dim, uint32_t hidden, const uint16_t *w1_bf16,
                      const float *b1, const uint16_t *w2_bf16, const float *b2, const uint16_t *w3_bf16,
                      const float *b3);

/* Training kernels of the scoring MLP (device pointers, asynchronous on
 * `stream`).  No reference counterpart: the reference has no learned part.
 * Forward: X [n][in_dim] fp32 -> P [n] probabilities; Z1/Z2 [n][hidden]
 * receive the pre-activations when non-null.  in_dim 1..64, hidden a
 * multiple of 32 up to 256. */
int sgfim_mlp_forward(sgfim_handle *h, const float *X, uint32_t n, uint32_t in_dim, uint32_t hidden,
                      const uint16_t *W1, const float *b1, const uint16_t *W2, const float *b2, const uint16_t *w3,
                      const float *b3, float *Z1, float *Z2, float *P, void *stream);
/* Backward of sum_r scale * WT[r] * BCE(P[r], Y[r]) (WT may be NULL = 1):
 * gradients are ADDED into dW1 [hidden][in_dim], db1, dW2 [hidden][hidden],
 * db2, dw3 [hidden], db3 [1]; loss [1] receives the summed loss. */
int sgfim_mlp_backward(sgfim_handle *h, const float *X, uint32_t n, uint32_t in_dim, uint32_t hidden,
                       const uint16_t *W2, const uint16_t *w3, const float *Z1, const float *Z2, const float *P,
                       const float *Y, const float *WT, float scale, float *dW1, float *db1, float *dW2, float *db2,
                       float *dw3, float *db3, float *loss, void *stream);
/* One Adam step on fp32 parameters; param_bf16 (nullable) receives the bf16 copy. */
int sgfim_adam_step(sgfim_handle *h, float *param, const float *grad, float *m, float *v, uint16_t *param_bf16,
                    uint32_t n, float lr, float beta1, float beta2, float eps, uint32_t step, float weight_decay,
                    void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SGFIM_H */
