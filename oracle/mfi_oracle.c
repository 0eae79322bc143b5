/*
 * mfi_oracle.c -- CPU restatement of the reference's MFI mining path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke test
 * and the CPU-baseline leg of bench.py link it to verify (or time) the CUDA
 * engine.  The engine itself never calls it; there is no CPU fallback.
 *
 * Every function restates one piece of the reference (paths relative to the
 * reference project root):
 *
 *   orc_build_bitmaps   vertical bitmap build      kernel_bitmap.cu:374-379
 *                       (code/engine_tensorfim/code/engine/src/)
 *   orc_support_batch   prefix-AND + popcount       kernel_bitmap.cu:390-408
 *   orc_cooccurrence    C[i][j]=popc(bv_i & bv_j)    microbench/bmma_bench.cu:180-191
 *   orc_mine_dfs        mine_mfi: ascending-id DFS   code/pipeline/skab_spike.py:84-135
 *                       over tidsets, leaves, then a
 *                       proper-subset filter
 *   orc_mine_engine     the engines' task-stack DFS  kernel_bitmap.cu:841-894,
 *                       ("little-endian" extension,  AnytimeMining/kernel.cu:862-899
 *                       global maximality count)
 *   orc_mine_fast       exact MFI miner with parent-equivalence pruning,
 *                       HUT/FHUT look-ahead and tidset projection, used where
 *                       mine_mfi's 200k-node cap makes the reference miner
 *                       unusable; it is checked against orc_mine_dfs.
 *   orc_mine_fast_order the same search with the extensions of every node in
 *                       ascending support (order 0, orc_mine_fast) or in the
 *                       reference's global descending-support order
 *                       (order 1: kernel_bitmap.cu:276-283,
 *                       code/pipeline/exp_e6_cpuvec.py:65-69), or in one
 *                       global order of a caller's per-item key (order 2,
 *                       no reference counterpart: a bound on what any
 *                       static order achieves); the set is the same, the
 *                       tree is not.
 *
 * Layout: bitmaps are uint64 [d][W] row-major; bit (t & 63) of word (t >> 6)
 * of row e is set when transaction t holds dense item e.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define POPC64(x) ((uint32_t)__builtin_popcountll((unsigned long long)(x)))
#define CTZ64(x) ((uint32_t)__builtin_ctzll((unsigned long long)(x)))

typedef struct {
    uint64_t n;        /* number of itemsets */
    uint64_t *ptr;     /* n+1 offsets into items */
    uint32_t *items;   /* dense ids, ascending inside each set */
    uint32_t *support; /* n supports */
    uint64_t nodes;    /* search nodes visited */
} orc_mfis;

/* ------------------------------------------------------------------ */
/* growable result buffer                                               */
typedef struct {
    uint64_t n, cap_sets, n_items, cap_items;
    uint64_t *ptr;
    uint32_t *items, *support;
} rbuf;

static int rb_init(rbuf *r) {
    memset(r, 0, sizeof(*r));
    r->cap_sets = 1024; r->cap_items = 8192;
    r->ptr = (uint64_t *)malloc((r->cap_sets + 1) * sizeof(uint64_t));
    r->items = (uint32_t *)malloc(r->cap_items * sizeof(uint32_t));
    r->support = (uint32_t *)malloc(r->cap_sets * sizeof(uint32_t));
    if (!r->ptr || !r->items || !r->support) return -1;
    r->ptr[0] = 0;
    return 0;
}
static void rb_free(rbuf *r) { free(r->ptr); free(r->items); free(r->support); memset(r, 0, sizeof(*r)); }

static int rb_push(rbuf *r, const uint32_t *set, uint32_t k, uint32_t sup) {
    if (r->n + 1 > r->cap_sets) {
        uint64_t nc = r->cap_sets * 2;
        uint64_t *p = (uint64_t *)realloc(r->ptr, (nc + 1) * sizeof(uint64_t));
        uint32_t *s = (uint32_t *)realloc(r->support, nc * sizeof(uint32_t));
        if (!p || !s) return -1;
        r->ptr = p; r->support = s; r->cap_sets = nc;
    }
    if (r->n_items + k > r->cap_items) {
        uint64_t nc = r->cap_items * 2 + k;
        uint32_t *it = (uint32_t *)realloc(r->items, nc * sizeof(uint32_t));
        if (!it) return -1;
        r->items = it; r->cap_items = nc;
    }
    memcpy(r->items + r->n_items, set, k * sizeof(uint32_t));
    r->n_items += k;
    r->support[r->n] = sup;
    r->n++;
    r->ptr[r->n] = r->n_items;
    return 0;
}

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

static void rb_to_out(rbuf *r, orc_mfis *out) {
    /* sort items inside each set ascending */
    for (uint64_t i = 0; i < r->n; i++)
        qsort(r->items + r->ptr[i], r->ptr[i + 1] - r->ptr[i], sizeof(uint32_t), cmp_u32);
    out->n = r->n; out->ptr = r->ptr; out->items = r->items; out->support = r->support;
}

void orc_free(orc_mfis *m) {
    if (!m) return;
    free(m->ptr); free(m->items); free(m->support);
    memset(m, 0, sizeof(*m));
}

/* ------------------------------------------------------------------ */
/* kernel_bitmap.cu:374-379: bm[x][t>>6] |= 1 << (t&63); also singleton counts */
void orc_build_bitmaps(const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn,
                       uint32_t d, uint64_t W, uint64_t *bm, uint32_t *counts) {
    memset(bm, 0, (size_t)d * W * sizeof(uint64_t));
    for (uint64_t t = 0; t < n_txn; t++)
        for (uint64_t j = row_ptr[t]; j < row_ptr[t + 1]; j++) {
            uint32_t x = items[j];
            if (x < d) bm[(size_t)x * W + (t >> 6)] |= 1ULL << (t & 63);
        }
    if (counts)
        for (uint32_t e = 0; e < d; e++) {
            uint32_t s = 0;
            const uint64_t *r = bm + (size_t)e * W;
            for (uint64_t w = 0; w < W; w++) s += POPC64(r[w]);
            counts[e] = s;
        }
}

/* ------------------------------------------------------------------ */
/* kernel_bitmap.cu:390-408 restated per candidate: sup(X) = sum_w popc(AND_{x in X} bv[x][w]) */
typedef struct {
    const uint64_t *bm; uint64_t W;
    const uint64_t *cand_ptr; const uint32_t *cand_items;
    uint64_t lo, hi; uint32_t *out; uint32_t d;
} sb_job;

static void *sb_worker(void *arg) {
    sb_job *j = (sb_job *)arg;
    for (uint64_t c = j->lo; c < j->hi; c++) {
        uint64_t a = j->cand_ptr[c], b = j->cand_ptr[c + 1];
        uint64_t s = 0;
        int absent = 0;
        for (uint64_t i = a; i < b; i++) absent |= j->cand_items[i] >= j->d;
        if (b == a) { s = j->W * 64; /* empty set: every (padded) transaction */ }
        else if (absent) { s = 0; /* an id without a row never occurs (kernel_bitmap.cu:354) */ }
        else {
            for (uint64_t w = 0; w < j->W; w++) {
                uint64_t m = ~0ULL;
                for (uint64_t i = a; i < b; i++) m &= j->bm[(size_t)j->cand_items[i] * j->W + w];
                s += POPC64(m);
            }
        }
        j->out[c] = (uint32_t)s;
    }
    return NULL;
}

void orc_support_batch(const uint64_t *bm, uint32_t d, uint64_t W, const uint64_t *cand_ptr,
                       const uint32_t *cand_items, uint64_t n_cand, uint32_t *out, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if ((uint64_t)n_threads > n_cand) n_threads = (int)(n_cand ? n_cand : 1);
    pthread_t th[256];
    sb_job jobs[256];
    if (n_threads > 256) n_threads = 256;
    for (int t = 0; t < n_threads; t++) {
        jobs[t].bm = bm; jobs[t].W = W; jobs[t].cand_ptr = cand_ptr; jobs[t].cand_items = cand_items;
        jobs[t].d = d;
        jobs[t].lo = n_cand * (uint64_t)t / (uint64_t)n_threads;
        jobs[t].hi = n_cand * (uint64_t)(t + 1) / (uint64_t)n_threads;
        jobs[t].out = out;
    }
    if (n_threads == 1) { sb_worker(&jobs[0]); return; }
    for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, sb_worker, &jobs[t]);
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* bmma_bench.cu:180-191 (cpu_ref) with A = B = the item bitmaps */
typedef struct { const uint64_t *bm; uint32_t d; uint64_t W; uint32_t lo, hi; uint32_t *out; } co_job;

static void *co_worker(void *arg) {
    co_job *j = (co_job *)arg;
    for (uint32_t i = j->lo; i < j->hi; i++)
        for (uint32_t k = 0; k < j->d; k++) {
            const uint64_t *a = j->bm + (size_t)i * j->W, *b = j->bm + (size_t)k * j->W;
            uint64_t s = 0;
            for (uint64_t w = 0; w < j->W; w++) s += POPC64(a[w] & b[w]);
            j->out[(size_t)i * j->d + k] = (uint32_t)s;
        }
    return NULL;
}

void orc_cooccurrence(const uint64_t *bm, uint32_t d, uint64_t W, uint32_t *out, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    if ((uint32_t)n_threads > d) n_threads = d ? (int)d : 1;
    pthread_t th[256];
    co_job jobs[256];
    for (int t = 0; t < n_threads; t++) {
        jobs[t].bm = bm; jobs[t].d = d; jobs[t].W = W; jobs[t].out = out;
        jobs[t].lo = (uint32_t)((uint64_t)d * t / n_threads);
        jobs[t].hi = (uint32_t)((uint64_t)d * (t + 1) / n_threads);
    }
    if (n_threads == 1) { co_worker(&jobs[0]); return; }
    for (int t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, co_worker, &jobs[t]);
    for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* helpers over bit vectors                                             */
static uint32_t and_popc(uint64_t *dst, const uint64_t *a, const uint64_t *b, uint64_t W) {
    uint32_t s = 0;
    for (uint64_t w = 0; w < W; w++) { uint64_t v = a[w] & b[w]; dst[w] = v; s += POPC64(v); }
    return s;
}
static uint32_t and_popc_count(const uint64_t *a, const uint64_t *b, uint64_t W) {
    uint32_t s = 0;
    for (uint64_t w = 0; w < W; w++) s += POPC64(a[w] & b[w]);
    return s;
}

/* ------------------------------------------------------------------ */
/* skab_spike.py:84-135 -- mine_mfi restated over bitmaps.                   */
/*   items: frequent items, ascending id (skab_spike.py:107)               */
/*   dfs: ext = candidates whose tidset intersection reaches thresh;       */
/*        no ext -> emit prefix (if non-empty); else recurse on each ext   */
/*        with the later ext items as candidates (skab_spike.py:111-126)   */
/*   node cap: RuntimeError above `cap` nodes (skab_spike.py:109-116)      */
/*   final filter: by length descending, drop proper subsets of kept sets  */
/*        (skab_spike.py:129-135)                                          */
typedef struct {
    const uint64_t *bm; uint64_t W; uint32_t thr;
    uint64_t nodes, cap; int overflow;
    rbuf leaves;
    uint32_t *prefix;
    uint64_t **level_bm;  /* scratch bitmap per depth */
    uint32_t **level_ext; /* ext item list per depth */
} dfs_ctx;

static void dfs_rec(dfs_ctx *c, uint32_t depth, const uint32_t *cand, uint32_t n_cand,
                    const uint64_t *cur, uint32_t cur_sup) {
    if (c->overflow) return;
    c->nodes++;
    if (c->cap && c->nodes > c->cap) { c->overflow = 1; return; }
    /* ext = [(x, cur & tidset[x]) for x in cand if |.| >= thresh] */
    uint32_t *ext = c->level_ext[depth];
    uint32_t n_ext = 0;
    for (uint32_t i = 0; i < n_cand; i++)
        if (and_popc_count(cur, c->bm + (size_t)cand[i] * c->W, c->W) >= c->thr) ext[n_ext++] = cand[i];
    if (n_ext == 0) {
        if (depth > 0) rb_push(&c->leaves, c->prefix, depth, cur_sup);
        return;
    }
    uint64_t *nb = c->level_bm[depth];
    for (uint32_t i = 0; i < n_ext; i++) {
        uint32_t s = and_popc(nb, cur, c->bm + (size_t)ext[i] * c->W, c->W);
        c->prefix[depth] = ext[i];
        dfs_rec(c, depth + 1, ext + i + 1, n_ext - i - 1, nb, s);
        if (c->overflow) return;
    }
}

/* is set a (sorted, ka) a proper subset of set b (sorted, kb)? */
static int proper_subset(const uint32_t *a, uint64_t ka, const uint32_t *b, uint64_t kb) {
    if (ka >= kb) return 0;
    uint64_t i = 0, j = 0;
    while (i < ka && j < kb) {
        if (a[i] == b[j]) { i++; j++; }
        else if (a[i] > b[j]) j++;
        else return 0;
    }
    return i == ka;
}

/* Returns 0 on success, 1 when the node cap was exceeded, -1 on allocation failure. */
int orc_mine_dfs(const uint64_t *bm, uint32_t d, uint64_t W, uint64_t n_txn, uint32_t thr,
                 uint64_t node_cap, orc_mfis *out) {
    memset(out, 0, sizeof(*out));
    if (thr < 1) thr = 1;
    dfs_ctx c;
    memset(&c, 0, sizeof(c));
    c.bm = bm; c.W = W; c.thr = thr; c.cap = node_cap;
    if (rb_init(&c.leaves)) return -1;
    c.prefix = (uint32_t *)calloc(d + 1, sizeof(uint32_t));
    c.level_bm = (uint64_t **)calloc(d + 1, sizeof(uint64_t *));
    c.level_ext = (uint32_t **)calloc(d + 1, sizeof(uint32_t *));
    uint32_t *items = (uint32_t *)malloc((d + 1) * sizeof(uint32_t));
    uint64_t *all = (uint64_t *)calloc(W ? W : 1, sizeof(uint64_t));
    int rc = 0;
    if (!c.prefix || !c.level_bm || !c.level_ext || !items || !all) { rc = -1; goto done; }
    for (uint32_t i = 0; i <= d; i++) {
        c.level_bm[i] = (uint64_t *)malloc((W ? W : 1) * sizeof(uint64_t));
        c.level_ext[i] = (uint32_t *)malloc((d + 1) * sizeof(uint32_t));
        if (!c.level_bm[i] || !c.level_ext[i]) { rc = -1; goto done; }
    }
    /* set(range(n)) as a bitmap */
    for (uint64_t t = 0; t < n_txn; t++) all[t >> 6] |= 1ULL << (t & 63);
    uint32_t n_items = 0;
    for (uint32_t e = 0; e < d; e++)
        if (and_popc_count(all, bm + (size_t)e * W, W) >= thr) items[n_items++] = e;
    dfs_rec(&c, 0, items, n_items, all, (uint32_t)n_txn);
    out->nodes = c.nodes;
    if (c.overflow) { rc = 1; goto done; }
    {
        /* inclusion filter: stable order by length descending */
        uint64_t n = c.leaves.n;
        uint64_t *order = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
        uint8_t *keep = (uint8_t *)calloc(n ? n : 1, 1);
        if (!order || !keep) { free(order); free(keep); rc = -1; goto done; }
        uint64_t m = 0;
        for (uint32_t len = d; len >= 1; len--)
            for (uint64_t i = 0; i < n; i++)
                if (c.leaves.ptr[i + 1] - c.leaves.ptr[i] == len) order[m++] = i;
        rbuf kept;
        if (rb_init(&kept)) { free(order); free(keep); rc = -1; goto done; }
        for (uint64_t a = 0; a < m; a++) {
            uint64_t i = order[a];
            const uint32_t *s = c.leaves.items + c.leaves.ptr[i];
            uint64_t ks = c.leaves.ptr[i + 1] - c.leaves.ptr[i];
            int sub = 0;
            for (uint64_t b = 0; b < kept.n && !sub; b++)
                sub = proper_subset(s, ks, kept.items + kept.ptr[b], kept.ptr[b + 1] - kept.ptr[b]);
            if (!sub) rb_push(&kept, s, (uint32_t)ks, c.leaves.support[i]);
        }
        free(order); free(keep);
        rb_to_out(&kept, out);
        out->nodes = c.nodes;
    }
done:
    if (c.level_bm) for (uint32_t i = 0; i <= d; i++) free(c.level_bm[i]);
    if (c.level_ext) for (uint32_t i = 0; i <= d; i++) free(c.level_ext[i]);
    free(c.level_bm); free(c.level_ext); free(c.prefix); free(items); free(all);
    rb_free(&c.leaves);
    return rc;
}

/* ------------------------------------------------------------------ */
/* The engines' search (kernel_bitmap.cu:841-894; AnytimeMining/kernel.cu:   */
/* 850-899): a stack of FI{itemsSet, progress}; popping X computes            */
/* sup(X u {e}) for every surviving item e; X is an MFI when the number of    */
/* e with sup >= thr equals |X| (kernel_bitmap.cu:870); otherwise push        */
/* X u {i} for every i < progress with sup >= thr and i not in X (:875-888).  */
/* Roots are single items with progress = their own id (:841-850).            */
/* Dense ids order like original ids, so "i < progress" is the same test.     */
int orc_mine_engine(const uint64_t *bm, uint32_t d, uint64_t W, uint32_t thr,
                    const uint32_t *roots, uint32_t n_roots, uint64_t node_cap, orc_mfis *out) {
    memset(out, 0, sizeof(*out));
    rbuf res;
    if (rb_init(&res)) return -1;
    /* explicit stack of (set, k); sets stored in a flat growable array */
    uint64_t cap = 1024, top = 0;
    uint32_t *sets = (uint32_t *)malloc(cap * (d + 1) * sizeof(uint32_t));
    uint32_t *cnt = (uint32_t *)malloc((d ? d : 1) * sizeof(uint32_t));
    uint64_t *mask = (uint64_t *)malloc((W ? W : 1) * sizeof(uint64_t));
    uint32_t *tmp = (uint32_t *)malloc((d + 1) * sizeof(uint32_t));
    uint64_t nodes = 0;
    int rc = 0;
    if (!sets || !cnt || !mask || !tmp) { rc = -1; goto done; }
    for (uint32_t r = 0; r < n_roots; r++) {
        if (top == cap) {
            cap *= 2;
            uint32_t *ns = (uint32_t *)realloc(sets, cap * (d + 1) * sizeof(uint32_t));
            if (!ns) { rc = -1; goto done; }
            sets = ns;
        }
        uint32_t *s = sets + top * (d + 1);
        s[0] = 1; s[1] = roots[r];
        top++;
    }
    while (top > 0) {
        top--;
        uint32_t *s = sets + top * (d + 1);
        uint32_t k = s[0];
        memcpy(tmp, s + 1, k * sizeof(uint32_t));
        nodes++;
        if (node_cap && nodes > node_cap) { rc = 1; goto done; }
        for (uint64_t w = 0; w < W; w++) mask[w] = ~0ULL;
        for (uint32_t i = 0; i < k; i++) {
            const uint64_t *b = bm + (size_t)tmp[i] * W;
            for (uint64_t w = 0; w < W; w++) mask[w] &= b[w];
        }
        uint32_t nfreq = 0, sup_x = 0;
        for (uint64_t w = 0; w < W; w++) sup_x += POPC64(mask[w]);
        for (uint32_t e = 0; e < d; e++) {
            cnt[e] = and_popc_count(mask, bm + (size_t)e * W, W);
            if (cnt[e] >= thr) nfreq++;
        }
        if (nfreq == k) { rb_push(&res, tmp, k, sup_x); continue; }
        uint32_t progress = tmp[k - 1];
        for (uint32_t i = 0; i < progress; i++) {
            if (cnt[i] < thr) continue;
            int inside = 0;
            for (uint32_t j = 0; j < k; j++) if (tmp[j] == i) { inside = 1; break; }
            if (inside) continue;
            if (top == cap) {
                cap *= 2;
                uint32_t *ns = (uint32_t *)realloc(sets, cap * (d + 1) * sizeof(uint32_t));
                if (!ns) { rc = -1; goto done; }
                sets = ns;
            }
            uint32_t *c = sets + top * (d + 1);
            c[0] = k + 1;
            memcpy(c + 1, tmp, k * sizeof(uint32_t));
            c[k + 1] = i;
            top++;
        }
    }
    rb_to_out(&res, out);
    memset(&res, 0, sizeof(res));
done:
    out->nodes = nodes;
    rb_free(&res);
    free(sets); free(cnt); free(mask); free(tmp);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Pruned exact MFI miner (set-enumeration DFS with PEP, HUT and FHUT).    */
/*                                                                        */
/* Node (H, T): for e in T count s_e = sup(H u {e}); F = {e : s_e >= thr}; */
/* PEP moves e with s_e == sup(H) into H; the rest of F is ordered by       */
/* ascending support (ties: ascending id).  A node without extension is a   */
/* candidate MFI unless a pool member contains it.  HUT: if H u F is        */
/* contained in a pool member the subtree holds no new MFI; FHUT: if H u F  */
/* itself is frequent it is the only candidate of the subtree.  Any MFI     */
/* superset of a candidate lies in an earlier subtree, so the pool test     */
/* decides maximality.  Tidsets are bitmaps; when sup(H) drops below a      */
/* quarter of the current bitmap length the tail bitmaps are projected onto */
/* H's transactions.                                                        */
typedef struct {
    uint32_t d, words;     /* item count, u64 words per item bitset */
    uint32_t thr;
    int order;             /* 0: ascending support in the node's context; 1: one global order,
                              descending item support, ties ascending id (kernel_bitmap.cu:276-283,
                              exp_e6_cpuvec.py:65-69); 2: one global order, ascending caller key,
                              ties ascending id */
    uint32_t *gsup;        /* item supports (order 1) */
    const double *key;     /* per-item key (order 2) */
    rbuf pool;             /* candidates (sorted items) */
    uint64_t *pool_bits;   /* words per candidate */
    uint64_t pool_cap;
    uint64_t nodes, cap; int overflow;
    uint32_t **lmfi; uint64_t *lmfi_n, *lmfi_cap; /* per-depth local pool lists */
} fast_ctx;

static int pool_add(fast_ctx *c, const uint32_t *set, uint32_t k, uint32_t sup, uint32_t depth) {
    uint32_t *tmp = (uint32_t *)malloc((k ? k : 1) * sizeof(uint32_t));
    if (!tmp) return -1;
    memcpy(tmp, set, k * sizeof(uint32_t));
    qsort(tmp, k, sizeof(uint32_t), cmp_u32);
    if (rb_push(&c->pool, tmp, k, sup)) { free(tmp); return -1; }
    free(tmp);
    uint64_t idx = c->pool.n - 1;
    if (c->pool.n > c->pool_cap) {
        uint64_t nc = c->pool_cap ? c->pool_cap * 2 : 1024;
        uint64_t *nb = (uint64_t *)realloc(c->pool_bits, nc * c->words * sizeof(uint64_t));
        if (!nb) return -1;
        c->pool_bits = nb; c->pool_cap = nc;
    }
    uint64_t *b = c->pool_bits + idx * c->words;
    memset(b, 0, c->words * sizeof(uint64_t));
    for (uint32_t i = 0; i < k; i++) b[set[i] >> 6] |= 1ULL << (set[i] & 63);
    /* every ancestor head is contained in the new candidate */
    for (uint32_t l = 0; l <= depth; l++) {
        if (c->lmfi_n[l] == c->lmfi_cap[l]) {
            uint64_t nc = c->lmfi_cap[l] ? c->lmfi_cap[l] * 2 : 64;
            uint32_t *nl = (uint32_t *)realloc(c->lmfi[l], nc * sizeof(uint32_t));
            if (!nl) return -1;
            c->lmfi[l] = nl; c->lmfi_cap[l] = nc;
        }
        c->lmfi[l][c->lmfi_n[l]++] = (uint32_t)idx;
    }
    return 0;
}

/* is bitset q (words) contained in any pool member listed at depth l? */
static int covered(const fast_ctx *c, uint32_t l, const uint64_t *q) {
    for (uint64_t a = 0; a < c->lmfi_n[l]; a++) {
        const uint64_t *p = c->pool_bits + (uint64_t)c->lmfi[l][a] * c->words;
        int ok = 1;
        for (uint32_t w = 0; w < c->words; w++) if (q[w] & ~p[w]) { ok = 0; break; }
        if (ok) return 1;
    }
    return 0;
}

/* rebuild the local list of depth l+1 from depth l: members containing head */
static int lmfi_push_level(fast_ctx *c, uint32_t l, const uint64_t *head) {
    c->lmfi_n[l + 1] = 0;
    for (uint64_t a = 0; a < c->lmfi_n[l]; a++) {
        uint32_t idx = c->lmfi[l][a];
        const uint64_t *p = c->pool_bits + (uint64_t)idx * c->words;
        int ok = 1;
        for (uint32_t w = 0; w < c->words; w++) if (head[w] & ~p[w]) { ok = 0; break; }
        if (!ok) continue;
        if (c->lmfi_n[l + 1] == c->lmfi_cap[l + 1]) {
            uint64_t nc = c->lmfi_cap[l + 1] ? c->lmfi_cap[l + 1] * 2 : 64;
            uint32_t *nl = (uint32_t *)realloc(c->lmfi[l + 1], nc * sizeof(uint32_t));
            if (!nl) return -1;
            c->lmfi[l + 1] = nl; c->lmfi_cap[l + 1] = nc;
        }
        c->lmfi[l + 1][c->lmfi_n[l + 1]++] = idx;
    }
    return 0;
}

typedef struct { uint32_t item, sup; } isup;
static int cmp_isup(const void *a, const void *b) {
    const isup *x = (const isup *)a, *y = (const isup *)b;
    if (x->sup != y->sup) return (x->sup > y->sup) - (x->sup < y->sup);
    return (x->item > y->item) - (x->item < y->item);
}

/* x before y in the search order of the extensions */
static int ext_before(const fast_ctx *c, const isup *x, const isup *y) {
    if (c->order == 2) {
        const double p = c->key[x->item], q = c->key[y->item];
        if (p != q) return p < q;
        return x->item < y->item;
    }
    if (c->order == 1) {
        const uint32_t p = c->gsup[x->item], q = c->gsup[y->item];
        if (p != q) return p > q;
        return x->item < y->item;
    }
    if (x->sup != y->sup) return x->sup < y->sup;
    return x->item < y->item;
}

/* stable insertion sort of the extensions (F is at most d long) */
static void sort_ext(const fast_ctx *c, isup *g, uint32_t n) {
    for (uint32_t i = 1; i < n; i++) {
        isup v = g[i];
        uint32_t j = i;
        while (j > 0 && ext_before(c, &v, &g[j - 1])) { g[j] = g[j - 1]; j--; }
        g[j] = v;
    }
}

/* tail bitmaps: tb[i] is the (possibly projected) bitmap of tail item i, nw words;
 * head bitmap hb is over the same transaction space. */
static int fast_rec(fast_ctx *c, uint32_t depth, uint32_t *head, uint32_t hk, uint64_t *hbits,
                    const uint64_t *hb, uint32_t hsup, const uint32_t *tail, const uint64_t *const *tb,
                    uint32_t nt, uint64_t nw) {
    if (c->overflow) return 0;
    c->nodes++;
    if (c->cap && c->nodes > c->cap) { c->overflow = 1; return 0; }
    isup *f = (isup *)malloc((nt ? nt : 1) * sizeof(isup));
    uint32_t *fidx = (uint32_t *)malloc((nt ? nt : 1) * sizeof(uint32_t));
    if (!f || !fidx) { free(f); free(fidx); return -1; }
    uint32_t nf = 0, h2 = hk;
    uint32_t *pep_items = head + hk;  /* PEP items are appended to head */
    for (uint32_t i = 0; i < nt; i++) {
        uint32_t s = and_popc_count(hb, tb[i], nw);
        if (s < c->thr) continue;
        if (s == hsup) { head[h2++] = tail[i]; hbits[tail[i] >> 6] |= 1ULL << (tail[i] & 63); continue; }
        f[nf].item = i; f[nf].sup = s; nf++;  /* item holds the tail index for now */
    }
    (void)pep_items;
    int rc = 0;
    if (nf == 0) {
        if (h2 > 0 && !covered(c, depth, hbits)) rc = pool_add(c, head, h2, hsup, depth);
        goto out;
    }
    /* order F: ascending support, ties by ascending item id (order 0), or the
     * global descending-support order (order 1) */
    for (uint32_t i = 0; i < nf; i++) { fidx[i] = f[i].item; f[i].item = tail[fidx[i]]; }
    {
        /* keep the tail-index association through the sort */
        isup *g = (isup *)malloc(nf * sizeof(isup));
        uint32_t *map = (uint32_t *)malloc((c->d + 1) * sizeof(uint32_t));
        if (!g || !map) { free(g); free(map); rc = -1; goto out; }
        for (uint32_t i = 0; i < nf; i++) { g[i] = f[i]; map[f[i].item] = fidx[i]; }
        if (c->order == 0) qsort(g, nf, sizeof(isup), cmp_isup);
        else sort_ext(c, g, nf);
        for (uint32_t i = 0; i < nf; i++) { f[i] = g[i]; fidx[i] = map[g[i].item]; }
        free(g); free(map);
    }
    {
        /* HUT: head u F contained in a known candidate */
        uint64_t *u = (uint64_t *)malloc(c->words * sizeof(uint64_t));
        if (!u) { rc = -1; goto out; }
        memcpy(u, hbits, c->words * sizeof(uint64_t));
        for (uint32_t i = 0; i < nf; i++) u[f[i].item >> 6] |= 1ULL << (f[i].item & 63);
        if (covered(c, depth, u)) { free(u); goto out; }
        /* FHUT: is head u F frequent? */
        uint64_t *m = (uint64_t *)malloc((nw ? nw : 1) * sizeof(uint64_t));
        if (!m) { free(u); rc = -1; goto out; }
        memcpy(m, hb, nw * sizeof(uint64_t));
        uint32_t s = 0;
        for (uint64_t w = 0; w < nw; w++) {
            uint64_t v = m[w];
            for (uint32_t i = 0; i < nf && v; i++) v &= tb[fidx[i]][w];
            s += POPC64(v);
        }
        free(m);
        if (s >= c->thr) {
            for (uint32_t i = 0; i < nf; i++) head[h2 + i] = f[i].item;
            rc = pool_add(c, head, h2 + nf, s, depth);
            free(u);
            goto out;
        }
        free(u);
    }
    {
        /* project when the head's support is small relative to the bitmap length */
        int project = (uint64_t)hsup * 4 < nw * 64 && nf > 1;
        uint64_t pnw = project ? ((uint64_t)hsup + 63) / 64 : nw;
        uint64_t *pool_tb = NULL, *phb = NULL;
        const uint64_t **ctb = (const uint64_t **)malloc(nf * sizeof(uint64_t *));
        if (!ctb) { rc = -1; goto out; }
        if (project) {
            pool_tb = (uint64_t *)calloc((size_t)nf * pnw, sizeof(uint64_t));
            phb = (uint64_t *)calloc(pnw, sizeof(uint64_t));
            if (!pool_tb || !phb) { free(pool_tb); free(phb); free(ctb); rc = -1; goto out; }
            for (uint32_t i = 0; i < nf; i++) {
                const uint64_t *src = tb[fidx[i]];
                uint64_t *dst = pool_tb + (size_t)i * pnw;
                uint64_t pos = 0;
                for (uint64_t w = 0; w < nw; w++) {
                    uint64_t mm = hb[w];
                    while (mm) {
                        uint32_t b = CTZ64(mm);
                        mm &= mm - 1;
                        if ((src[w] >> b) & 1) dst[pos >> 6] |= 1ULL << (pos & 63);
                        pos++;
                    }
                }
                ctb[i] = dst;
            }
            for (uint64_t t = 0; t < hsup; t++) phb[t >> 6] |= 1ULL << (t & 63);
        } else {
            for (uint32_t i = 0; i < nf; i++) ctb[i] = tb[fidx[i]];
        }
        uint64_t *child_hb = (uint64_t *)malloc((pnw ? pnw : 1) * sizeof(uint64_t));
        uint32_t *ctail = (uint32_t *)malloc(nf * sizeof(uint32_t));
        uint64_t *q = (uint64_t *)malloc(c->words * sizeof(uint64_t));
        uint64_t *child_bits = (uint64_t *)malloc(c->words * sizeof(uint64_t));
        if (!child_hb || !ctail || !q || !child_bits) rc = -1;
        for (uint32_t i = 0; i < nf && rc == 0 && !c->overflow; i++) {
            uint32_t e = f[i].item;
            /* HUT for the child: head u {e} u F[i+1:] */
            memcpy(q, hbits, c->words * sizeof(uint64_t));
            for (uint32_t j = i; j < nf; j++) q[f[j].item >> 6] |= 1ULL << (f[j].item & 63);
            if (covered(c, depth, q)) continue;
            const uint64_t *base = project ? phb : hb;
            for (uint64_t w = 0; w < pnw; w++) child_hb[w] = base[w] & ctb[i][w];
            memcpy(child_bits, hbits, c->words * sizeof(uint64_t));
            child_bits[e >> 6] |= 1ULL << (e & 63);
            if (lmfi_push_level(c, depth, child_bits)) { rc = -1; break; }
            for (uint32_t j = i + 1; j < nf; j++) ctail[j - i - 1] = f[j].item;
            head[h2] = e;
            rc = fast_rec(c, depth + 1, head, h2 + 1, child_bits, child_hb, f[i].sup, ctail,
                          (const uint64_t *const *)(ctb + i + 1), nf - i - 1, pnw);
        }
        free(child_hb); free(ctail); free(q); free(child_bits);
        free(pool_tb); free(phb); free(ctb);
    }
out:
    /* undo PEP bits on the caller's head bitset */
    for (uint32_t i = hk; i < h2; i++) hbits[head[i] >> 6] &= ~(1ULL << (head[i] & 63));
    free(f); free(fidx);
    return rc;
}

/* Exact MFI set at absolute threshold thr (every MFI once, with its support).
 * Returns 0, 1 on node-cap overflow, -1 on allocation failure. */
int orc_mine_fast_order(const uint64_t *bm, uint32_t d, uint64_t W, uint64_t n_txn, uint32_t thr,
                        uint64_t node_cap, int order, const double *key, orc_mfis *out) {
    memset(out, 0, sizeof(*out));
    if (thr < 1) thr = 1;
    if (order < 0 || order > 2 || (order == 2 && !key)) return -1;
    fast_ctx c;
    memset(&c, 0, sizeof(c));
    c.d = d; c.words = (d + 63) / 64; if (!c.words) c.words = 1;
    c.thr = thr; c.cap = node_cap; c.order = order; c.key = key;
    int rc = 0;
    if (order == 1) {
        c.gsup = (uint32_t *)calloc(d ? d : 1, sizeof(uint32_t));
        if (!c.gsup) return -1;
        for (uint32_t e = 0; e < d; e++) {
            uint32_t s = 0;
            for (uint64_t w = 0; w < W; w++) s += POPC64(bm[(size_t)e * W + w]);
            c.gsup[e] = s;
        }
    }
    if (rb_init(&c.pool)) return -1;
    c.lmfi = (uint32_t **)calloc(d + 2, sizeof(uint32_t *));
    c.lmfi_n = (uint64_t *)calloc(d + 2, sizeof(uint64_t));
    c.lmfi_cap = (uint64_t *)calloc(d + 2, sizeof(uint64_t));
    uint32_t *head = (uint32_t *)calloc(d + 1, sizeof(uint32_t));
    uint64_t *hbits = (uint64_t *)calloc(c.words, sizeof(uint64_t));
    uint64_t *all = (uint64_t *)calloc(W ? W : 1, sizeof(uint64_t));
    uint32_t *tail = (uint32_t *)malloc((d ? d : 1) * sizeof(uint32_t));
    const uint64_t **tb = (const uint64_t **)malloc((d ? d : 1) * sizeof(uint64_t *));
    if (!c.lmfi || !c.lmfi_n || !c.lmfi_cap || !head || !hbits || !all || !tail || !tb) { rc = -1; goto done; }
    for (uint64_t t = 0; t < n_txn; t++) all[t >> 6] |= 1ULL << (t & 63);
    for (uint32_t e = 0; e < d; e++) { tail[e] = e; tb[e] = bm + (size_t)e * W; }
    rc = fast_rec(&c, 0, head, 0, hbits, all, (uint32_t)n_txn, tail, (const uint64_t *const *)tb, d, W);
    out->nodes = c.nodes;
    if (rc == 0 && c.overflow) rc = 1;
    if (rc == 0) { rb_to_out(&c.pool, out); memset(&c.pool, 0, sizeof(c.pool)); out->nodes = c.nodes; }
done:
    rb_free(&c.pool);
    free(c.pool_bits);
    if (c.lmfi) for (uint32_t i = 0; i < d + 2; i++) free(c.lmfi[i]);
    free(c.lmfi); free(c.lmfi_n); free(c.lmfi_cap);
    free(head); free(hbits); free(all); free(tail); free(tb);
    free(c.gsup);
    return rc;
}

int orc_mine_fast(const uint64_t *bm, uint32_t d, uint64_t W, uint64_t n_txn, uint32_t thr,
                  uint64_t node_cap, orc_mfis *out) {
    return orc_mine_fast_order(bm, d, W, n_txn, thr, node_cap, 0, NULL, out);
}
