// kernels_wmine.cu -- batched per-window MFI mining on the ring.
//
// The reference mines one window per engine process (code/pipeline/
// skab_spike.py:61-80 builds the windows; the engines' DFS is
// kernel_bitmap.cu:841-894); its result for a window is the MFI set of that
// window's transactions at the window's floor, which these kernels reproduce.
//
// Representation.  Items are the ring's dense ids 0..d-1 (d <= 64*MW); an
// itemset is an MW-word mask.  A task's base database holds one MW-word entry
// per window transaction that contains the task's required items and still
// holds a tail item, restricted to the tail (build_base: the transactions are
// found through the ring's vertical rows, their item masks read from the
// ring's horizontal masks).  wvtask_kernel (the default) turns the base into
// vertical rows, one bit per entry per item, and keeps one tidset per search
// level: counts are AND-popcounts of the level's tidset with the item rows.
// wtask_kernel (SGFIM_F_WINDOWS_HORIZONTAL) instead stacks each level's
// projected database as entries.
//
// Search.  Depth-first over the set-enumeration tree, one node at a time per
// warp, children in ascending (support, id) order -- the order under which a
// candidate found later is never a proper superset of one found earlier in
// the same subtree: child j's subtree lacks item f_i of every earlier sibling
// i < j, which all candidates of sibling i contain.  Every node applies
//   counts  c_e = |t(H u {e})|, e in T       (ballot popcounts over entries)
//   PEP     c_e == sup(H) (and >= thr)       -> e joins H
//   leaf    F = {e : thr <= c_e < sup(H)} empty: H is a candidate
//   HUT     H u F inside a known MFI          -> nothing new below
//   FHUT    |t(H u F)| >= thr                  -> H u F is the only candidate
// and candidates are checked against the MFIs found so far that contain the
// node's head (the "local MFI" list: the parent's list filtered to members
// containing the child's head, plus everything found inside the parent's
// subtree, which contains the parent's head by construction).
//
// Work split.  A window shorter than 64 transactions is one task: its warp
// searches the whole tree and its pool is the exact MFI set.  Longer windows
// are split at the root: wroot_kernel counts the root and sorts its frequent
// tail f_0..f_{k-1}; task (w, j) searches child j's subtree alone.  The
// costliest children are split once more (wsub_kernel expands child j the same
// way; task (w, j, g) searches its child g).  Tasks share no pool, so a
// candidate of one subtree may sit inside a candidate of an earlier subtree
// in depth-first order (never of a later one, by the argument above);
// wfilter_kernel removes exactly those with a vertical bitmap of the window's
// candidates, and wgather_kernel writes the kept candidates in window order.
//
// Work is distributed by atomic counters (costliest tasks first); every
// loop is bounded by list lengths, and any capacity overflow (entry stack,
// local-MFI stack, pool, depth, filter scratch) marks the window for the
// host-driven wave miner instead of producing a partial result.
#include <cstddef>

#include "common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <int MW> struct Mask {
    uint64_t w[MW];
};

template <int MW> __device__ __forceinline__ uint64_t m_word(const Mask<MW> &m, uint32_t i) {
    // arithmetic selection: no indexable copy of m
    uint64_t r = 0;
#pragma unroll
    for (int k = 0; k < MW; ++k) r |= m.w[k] & (0ull - (uint64_t)((uint32_t)k == i));
    return r;
}
template <int MW> __device__ __forceinline__ bool m_has(const Mask<MW> &m, uint32_t e) {
    return (m_word(m, e >> 6) >> (e & 63)) & 1ull;
}
template <int MW> __device__ __forceinline__ void m_set(Mask<MW> &m, uint32_t e) {
    const uint64_t bit = 1ull << (e & 63);
#pragma unroll
    for (int k = 0; k < MW; ++k) m.w[k] |= bit & (0ull - (uint64_t)((uint32_t)k == (e >> 6)));
}
template <int MW> __device__ __forceinline__ bool m_nz(const Mask<MW> &m) {
    uint64_t x = 0;
#pragma unroll
    for (int i = 0; i < MW; ++i) x |= m.w[i];
    return x != 0;
}
// a subset of b
template <int MW> __device__ __forceinline__ bool m_sub(const Mask<MW> &a, const Mask<MW> &b) {
    uint64_t x = 0;
#pragma unroll
    for (int i = 0; i < MW; ++i) x |= a.w[i] & ~b.w[i];
    return x == 0;
}
template <int MW> __device__ __forceinline__ Mask<MW> m_and(const Mask<MW> &a, const Mask<MW> &b) {
    Mask<MW> r;
#pragma unroll
    for (int i = 0; i < MW; ++i) r.w[i] = a.w[i] & b.w[i];
    return r;
}
template <int MW> __device__ __forceinline__ Mask<MW> m_zero() {
    Mask<MW> r;
#pragma unroll
    for (int i = 0; i < MW; ++i) r.w[i] = 0;
    return r;
}
// 16-byte vector accesses: every mask array is 16-byte aligned (MW even)
template <int MW> __device__ __forceinline__ Mask<MW> m_load(const uint64_t *p) {
    static_assert(MW % 2 == 0, "mask width must be even");
    Mask<MW> r;
#pragma unroll
    for (int i = 0; i < MW; i += 2) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(p + i);
        r.w[i] = v.x;
        r.w[i + 1] = v.y;
    }
    return r;
}
template <int MW> __device__ __forceinline__ void m_store(uint64_t *p, const Mask<MW> &m) {
#pragma unroll
    for (int i = 0; i < MW; i += 2) *reinterpret_cast<ulonglong2 *>(p + i) = make_ulonglong2(m.w[i], m.w[i + 1]);
}
template <int MW> __device__ __forceinline__ Mask<MW> warp_or(const Mask<MW> &m) {
    Mask<MW> r;
#pragma unroll
    for (int i = 0; i < MW; ++i) {
        const uint32_t lo = __reduce_or_sync(kFull, (uint32_t)m.w[i]);
        const uint32_t hi = __reduce_or_sync(kFull, (uint32_t)(m.w[i] >> 32));
        r.w[i] = ((uint64_t)hi << 32) | lo;
    }
    return r;
}

// Per-level record of the search stack (global memory, one stack per warp).
template <int MW> struct alignas(16) WLevel {
    uint64_t hp[MW];        // head after PEP
    uint64_t list_off;      // first entry of this node's projected database
    uint32_t list_n;
    uint32_t lm_off, lm_n;  // local-MFI list (pool indices)
    uint32_t entry;         // pool size when the node was entered
    uint32_t k, j;          // frequent tail size, next child
    uint8_t f[128];         // frequent tail, ascending (support, id)
    uint32_t c[128];        // supports of f
};

// Root of a split window (wroot_kernel), or a root child that is split again
// (wsub_kernel); read by wtask_kernel.
template <int MW> struct alignas(16) WRoot {
    uint64_t hp[MW];        // root head after PEP (items in every transaction)
    uint64_t cand[MW];      // the window's only MFI when the root is terminal
    uint32_t cand_sup;
    uint32_t has_cand;      // 1: the MFI set is {cand}; 0: the tasks (k of them) hold it
    uint32_t k;
    uint32_t overflow;      // subtree records: the node's database did not fit (mine the window elsewhere)
    uint8_t f[128];
    uint32_t c[128];
};

// the host reads these fields of the root records (ring.cu)
static_assert(offsetof(WRoot<2>, cand) == 16 && offsetof(WRoot<2>, cand_sup) == 32 &&
                  offsetof(WRoot<2>, has_cand) == 36 && offsetof(WRoot<2>, k) == 40 &&
                  offsetof(WRoot<2>, overflow) == 44 && offsetof(WRoot<2>, f) == 48 && offsetof(WRoot<2>, c) == 176,
              "root record layout read by sgfim_ring_mine_windows");

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The search stack holds itemsets of up to kWDepth - 1 items.
constexpr int kWDepth = 48;
// chunks of 32 entries loaded before any is processed (memory-level parallelism)
constexpr int kU = 4;

// One projected-database entry: ring slot (start + i) of the window, or entry
// i of the warp's stack.
template <int MW> __device__ __forceinline__ const uint64_t *entry_ptr(bool ring, const WMineParams &p, uint64_t start,
                                                                      const uint64_t *lists, uint64_t off, uint32_t i) {
    return ring ? p.hm + ((start + i) & p.cap_mask) * MW : lists + (off + i) * MW;
}

// c_e over the database (lane 0 accumulates into the warp's counters cnt[128]).
template <int MW>
__device__ __forceinline__ void count_items(bool ring, const WMineParams &p, uint64_t start, const uint64_t *lists,
                                            uint64_t off, uint32_t n, const Mask<MW> &T, uint32_t *cnt,
                                            uint32_t lane) {
    for (uint32_t q = lane; q < 128; q += 32) cnt[q] = 0;
    __syncwarp();
    for (uint32_t b = 0; b < n; b += 32 * kU) {
        Mask<MW> m[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = b + u * 32 + lane;
            m[u] = i < n ? m_and(m_load<MW>(entry_ptr<MW>(ring, p, start, lists, off, i)), T) : m_zero<MW>();
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const Mask<MW> om = warp_or(m[u]);
#pragma unroll
            for (int ww = 0; ww < MW; ++ww) {
                const uint64_t mine = m[u].w[ww];
                uint64_t x = om.w[ww];
                while (x) {
                    const uint32_t bit = __ffsll((long long)x) - 1;
                    x &= x - 1;
                    const uint32_t c = __popc(__ballot_sync(kFull, (mine >> bit) & 1ull));
                    if (lane == 0) cnt[ww * 64 + bit] += c;
                }
            }
        }
    }
    __syncwarp();
}

// PEP items P and frequent tail F of a node from its counts.
template <int MW>
__device__ __forceinline__ void classify(const Mask<MW> &T, const uint32_t *cnt, uint32_t d, uint32_t thr, uint32_t sup,
                                         uint32_t lane, Mask<MW> &P, Mask<MW> &F) {
    P = m_zero<MW>();
    F = m_zero<MW>();
#pragma unroll
    for (int q = 0; q < 2 * MW; ++q) {
        const uint32_t e = q * 32 + lane;
        const bool inT = e < d && ((T.w[q >> 1] >> ((q & 1) * 32 + lane)) & 1ull);
        const uint32_t c = inT ? cnt[e] : 0;
        const uint32_t bp = __ballot_sync(kFull, inT && c >= thr && c == sup);
        const uint32_t bf = __ballot_sync(kFull, inT && c >= thr && c < sup);
        P.w[q >> 1] |= (uint64_t)bp << ((q & 1) * 32);
        F.w[q >> 1] |= (uint64_t)bf << ((q & 1) * 32);
    }
}

// |{entries containing F}|
template <int MW>
__device__ __forceinline__ uint32_t count_superset(bool ring, const WMineParams &p, uint64_t start,
                                                   const uint64_t *lists, uint64_t off, uint32_t n,
                                                   const Mask<MW> &F, uint32_t lane) {
    uint32_t cf = 0;
    for (uint32_t b = 0; b < n; b += 32 * kU) {
        bool h[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = b + u * 32 + lane;
            h[u] = i < n && m_sub(F, m_load<MW>(entry_ptr<MW>(ring, p, start, lists, off, i)));
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) cf += __popc(__ballot_sync(kFull, h[u]));
    }
    return cf;
}

// F sorted by (count, id) ascending into f[], c[] (the lanes own the 4*MW/2
// items lane, lane+32, ...; one pass over F compares against all of them).
template <int MW>
__device__ __forceinline__ void sort_tail(const Mask<MW> &F, const uint32_t *cnt, uint32_t lane, uint8_t *f,
                                          uint32_t *c) {
    uint32_t ce[2 * MW], rank[2 * MW];
#pragma unroll
    for (int q = 0; q < 2 * MW; ++q) {
        const uint32_t e = q * 32 + lane;
        ce[q] = ((F.w[q >> 1] >> ((q & 1) * 32 + lane)) & 1ull) ? cnt[e] : 0xffffffffu;
        rank[q] = 0;
    }
#pragma unroll
    for (int ww = 0; ww < MW; ++ww) {
        uint64_t x = F.w[ww];
        while (x) {
            const uint32_t e2 = ww * 64 + (__ffsll((long long)x) - 1);
            x &= x - 1;
            const uint32_t c2 = cnt[e2];
#pragma unroll
            for (int q = 0; q < 2 * MW; ++q) {
                const uint32_t e = q * 32 + lane;
                rank[q] += (c2 < ce[q]) || (c2 == ce[q] && e2 < e);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 2 * MW; ++q) {
        if (ce[q] != 0xffffffffu) {
            f[rank[q]] = (uint8_t)(q * 32 + lane);
            c[rank[q]] = ce[q];
        }
    }
}

// Child database: entries holding every item of req, restricted to Tc,
// non-empty, written at dst .. dst+cn of the warp's stack.  Returns cn, or
// 0xffffffff on overflow.
template <int MW>
__device__ __forceinline__ uint32_t build_child(bool ring, const WMineParams &p, uint64_t start, uint64_t *lists,
                                                uint64_t src_off, uint32_t src_n, const Mask<MW> &req,
                                                const Mask<MW> &Tc, uint64_t dst, uint32_t lane) {
    uint32_t cn = 0;
    for (uint32_t b = 0; b < src_n; b += 32 * kU) {
        Mask<MW> m[kU];
        bool keep[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = b + u * 32 + lane;
            m[u] = m_zero<MW>();
            keep[u] = false;
            if (i < src_n) {
                const Mask<MW> r = m_load<MW>(entry_ptr<MW>(ring, p, start, lists, src_off, i));
                m[u] = m_and(r, Tc);
                keep[u] = m_sub(req, r) && m_nz(m[u]);
            }
        }
        // the child's entries go after the source's: writes never touch entries still to be read
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t bal = __ballot_sync(kFull, keep[u]);
            const uint64_t pos = dst + cn + __popc(bal & ((1u << lane) - 1));
            if (keep[u] && pos < p.list_cap) m_store(lists + pos * MW, m[u]);
            cn += __popc(bal);
        }
    }
    return dst + cn > p.list_cap ? 0xffffffffu : cn;
}


// Base database of a task, found through the ring's vertical rows: the
// window's transactions holding every item of req (at most two items; none =
// every transaction), each as its item mask restricted to T, dropped when
// empty, in transaction order, written at lists[0 ..).  Returns the count, or
// 0xffffffff when it does not fit.
template <int MW>
__device__ __forceinline__ uint32_t build_base(const WMineParams &p, uint64_t start, uint32_t n, const Mask<MW> &req,
                                               const Mask<MW> &T, uint64_t *lists, uint32_t lane) {
    uint32_t r0 = 0xffffffffu, r1 = 0xffffffffu;
#pragma unroll
    for (int ww = 0; ww < MW; ++ww) {
        uint64_t x = req.w[ww];
        while (x) {
            const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
            x &= x - 1;
            if (r0 == 0xffffffffu) r0 = e;
            else r1 = e;
        }
    }
    const uint64_t cwm = p.ring_words - 1;
    const uint64_t w0 = start >> 6;
    const uint64_t nwd = n ? ((start + n - 1) >> 6) - w0 + 1 : 0;
    const uint64_t m_first = ~0ull << (start & 63);
    const uint64_t m_last = n ? (~0ull >> (63 - ((start + n - 1) & 63))) : 0;
    uint32_t cn = 0;
    for (uint64_t b = 0; b < nwd; b += 32) {
        const uint64_t i = b + lane;
        uint64_t bits = 0;
        if (i < nwd) {
            bits = ~0ull;
            if (i == 0) bits &= m_first;
            if (i + 1 == nwd) bits &= m_last;
            const uint64_t wq = (w0 + i) & cwm;
            if (r0 != 0xffffffffu) bits &= p.ring_rows[(uint64_t)r0 * p.ring_words + wq];
            if (r1 != 0xffffffffu) bits &= p.ring_rows[(uint64_t)r1 * p.ring_words + wq];
        }
        // pass 1: how many of this lane's transactions keep a tail item
        uint32_t mine = 0;
        for (uint64_t x = bits; x; x &= x - 1) {
            const uint64_t pos = ((w0 + i) << 6) + (__ffsll((long long)x) - 1);
            mine += m_nz(m_and(m_load<MW>(p.hm + (pos & p.cap_mask) * MW), T));
        }
        // exclusive prefix over the lanes keeps transaction order
        uint32_t incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        uint64_t at = cn + incl - mine;
        // pass 2: write them
        for (uint64_t x = bits; x; x &= x - 1) {
            const uint64_t pos = ((w0 + i) << 6) + (__ffsll((long long)x) - 1);
            const Mask<MW> m = m_and(m_load<MW>(p.hm + (pos & p.cap_mask) * MW), T);
            if (m_nz(m)) {
                if (at < p.list_cap) m_store(lists + at * MW, m);
                ++at;
            }
        }
        cn += __shfl_sync(kFull, incl, 31);
    }
    __syncwarp();
    return cn > p.list_cap ? 0xffffffffu : cn;
}

// Position of item e among the items of T0: its row slot in the vertical layout.
template <int MW> __device__ __forceinline__ uint32_t m_rank(const Mask<MW> &T0, uint32_t e) {
    uint32_t r = 0;
    const uint32_t wi = e >> 6;
#pragma unroll
    for (int k = 0; k < MW; ++k) {
        const uint64_t below = (uint32_t)k < wi ? ~0ull : ((uint32_t)k == wi ? ((1ull << (e & 63)) - 1) : 0ull);
        r += __popcll(T0.w[k] & below);
    }
    return r;
}

// Vertical rows of a database of n0 entries: bit i of word c of row slot s is
// set when entry 32c+i holds the s-th item of T0 (entries are restricted to T0).
template <int MW>
__device__ __forceinline__ void build_rows(const uint64_t *lists, uint32_t n0, const Mask<MW> &T0, uint32_t *rows,
                                           uint32_t vw, uint32_t lane) {
    const uint32_t W = (n0 + 31) / 32;
    for (uint32_t c = 0; c < W; ++c) {
        const uint32_t i = c * 32 + lane;
        const Mask<MW> m = i < n0 ? m_load<MW>(lists + (uint64_t)i * MW) : m_zero<MW>();
        uint32_t mine = 0, slot = 0;
#pragma unroll
        for (int ww = 0; ww < MW; ++ww) {
            const uint64_t mw_ = m.w[ww];
            uint64_t x = T0.w[ww];
            while (x) {
                const uint32_t bit = __ffsll((long long)x) - 1;
                x &= x - 1;
                const uint32_t word = __ballot_sync(kFull, (mw_ >> bit) & 1ull);
                if (lane == (slot & 31)) mine = word;
                ++slot;
                if ((slot & 31) == 0) rows[(uint64_t)(slot - 32 + lane) * vw + c] = mine;
            }
        }
        if ((slot & 31) && lane < (slot & 31)) rows[(uint64_t)((slot & ~31u) + lane) * vw + c] = mine;
    }
    __syncwarp();
}

// c_e = popc(tid AND row(e)) for e in T (lane 0 writes cnt[e]).
template <int MW>
__device__ __forceinline__ void vcount(const uint32_t *tid, const uint32_t *rows, uint32_t vw, uint32_t W,
                                       const Mask<MW> &T, const Mask<MW> &T0, uint32_t *cnt, uint32_t lane) {
    constexpr uint32_t kReg = 4;   // tidsets of up to 128 words stay in registers across the items
    uint32_t tr[kReg];
    const bool small = W <= 32 * kReg;
#pragma unroll
    for (uint32_t k = 0; k < kReg; ++k) tr[k] = (small && lane + 32 * k < W) ? tid[lane + 32 * k] : 0u;
#pragma unroll
    for (int ww = 0; ww < MW; ++ww) {
        uint64_t x = T.w[ww];
        while (x) {
            const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
            x &= x - 1;
            const uint32_t *row = rows + (uint64_t)m_rank(T0, e) * vw;
            uint32_t acc = 0;
            if (small) {
#pragma unroll
                for (uint32_t k = 0; k < kReg; ++k)
                    if (lane + 32 * k < W) acc += __popc(tr[k] & row[lane + 32 * k]);
            } else {
                for (uint32_t w = lane; w < W; w += 32) acc += __popc(tid[w] & row[w]);
            }
            acc = __reduce_add_sync(kFull, acc);
            if (lane == 0) cnt[e] = acc;
        }
    }
    __syncwarp();
}

// |{entries of tid holding every item of F}|
template <int MW>
__device__ __forceinline__ uint32_t vcount_superset(const uint32_t *tid, const uint32_t *rows, uint32_t vw, uint32_t W,
                                                    const Mask<MW> &F, const Mask<MW> &T0, uint32_t lane) {
    uint32_t acc = 0;
    for (uint32_t w = lane; w < W; w += 32) {
        uint32_t v = tid[w];
#pragma unroll
        for (int ww = 0; ww < MW; ++ww) {
            uint64_t x = F.w[ww];
            while (x && v) {
                const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
                x &= x - 1;
                v &= rows[(uint64_t)m_rank(T0, e) * vw + w];
            }
        }
        acc += __popc(v);
    }
    return __reduce_add_sync(kFull, acc);
}

}  // namespace

// ------------------------------------------------------------------ roots
// Root counts from the ring's vertical rows: item e's support in the window
// is the popcount of its row over the window's bit range (the ring keeps
// one row per item, 64 transactions per word).
template <int MW> __global__ void __launch_bounds__(128) wroot_kernel(WMineParams p) {
    __shared__ uint32_t s_cnt[4][128];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    uint32_t *cnt = s_cnt[wib];
    WRoot<MW> *roots = reinterpret_cast<WRoot<MW> *>(p.roots);
    const uint64_t cwm = p.ring_words - 1;   // ring words: a power of two
    for (;;) {
        uint32_t wi = 0;
        if (lane == 0) wi = atomicAdd(p.next + 1, 1u);
        wi = __shfl_sync(kFull, wi, 0);
        if (wi >= p.n_split) break;
        const uint32_t w = p.split_win[wi];
        const uint64_t start = p.starts[w];
        const uint32_t n = p.lens[w];
        const uint32_t thr = p.thrs[w] ? p.thrs[w] : 1;
        // window bits: unwrapped words w0 .. w1, masked at both ends
        const uint64_t w0 = start >> 6, w1 = n ? (start + n - 1) >> 6 : w0;
        const uint64_t nwd = n ? w1 - w0 + 1 : 0;
        const uint64_t m_first = ~0ull << (start & 63);
        const uint64_t m_last = n ? (~0ull >> (63 - ((start + n - 1) & 63))) : 0;
        auto word_mask = [&](uint64_t i) {
            uint64_t m = ~0ull;
            if (i == 0) m &= m_first;
            if (i + 1 == nwd) m &= m_last;
            return m;
        };
        Mask<MW> T = m_zero<MW>();
        for (uint32_t e = 0; e < p.d; ++e) m_set(T, e);
        for (uint32_t e = 0; e < p.d; ++e) {
            const uint64_t *row = p.ring_rows + (uint64_t)e * p.ring_words;
            uint32_t acc = 0;
            for (uint64_t i = lane; i < nwd; i += 32) acc += __popcll(row[(w0 + i) & cwm] & word_mask(i));
            acc = __reduce_add_sync(kFull, acc);
            if (lane == 0) cnt[e] = acc;
        }
        __syncwarp();
        Mask<MW> P, F;
        classify<MW>(T, cnt, p.d, thr, n, lane, P, F);
        uint32_t k = 0;
#pragma unroll
        for (int i = 0; i < MW; ++i) k += __popcll(F.w[i]);
        WRoot<MW> &R = roots[w];
        uint32_t has = 0, csup = 0;
        Mask<MW> cand = P;   // root head after PEP (H = {} at the root)
        if (k == 0) {
            has = m_nz(P) ? 1u : 0u;
            csup = n;
        } else {
            // FHUT: transactions holding every item of F
            uint32_t acc = 0;
            for (uint64_t i = lane; i < nwd; i += 32) {
                uint64_t v = word_mask(i);
#pragma unroll
                for (int ww = 0; ww < MW; ++ww) {
                    uint64_t x = F.w[ww];
                    while (x && v) {
                        const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
                        x &= x - 1;
                        v &= p.ring_rows[(uint64_t)e * p.ring_words + ((w0 + i) & cwm)];
                    }
                }
                acc += __popcll(v);
            }
            const uint32_t cf = __reduce_add_sync(kFull, acc);
            if (cf >= thr) {
                has = 1;
                csup = cf;
#pragma unroll
                for (int i = 0; i < MW; ++i) cand.w[i] |= F.w[i];
            }
        }
        if (!has && k) sort_tail<MW>(F, cnt, lane, R.f, R.c);
        if (lane < MW) {
            R.hp[lane] = m_word(P, lane);
            R.cand[lane] = m_word(cand, lane);
        }
        if (lane == 0) {
            R.cand_sup = csup;
            R.has_cand = has;
            R.k = has ? 0 : k;
            R.overflow = 0;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ split root children
// Child j of a split window's root, expanded like a root: its database is
// built from the ring (transactions holding f_j, restricted to f_{j+1..}),
// then counts, PEP, FHUT and the sorted frequent tail go to its record.
template <int MW> __global__ void __launch_bounds__(128) wsub_kernel(WMineParams p) {
    __shared__ uint32_t s_cnt[4][128];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint32_t *cnt = s_cnt[wib];
    uint64_t *lists = p.lists + warp * (uint64_t)p.list_cap * MW;
    const WRoot<MW> *roots = reinterpret_cast<const WRoot<MW> *>(p.roots);
    WRoot<MW> *subs = reinterpret_cast<WRoot<MW> *>(p.subs);
    for (;;) {
        uint32_t si = 0;
        if (lane == 0) si = atomicAdd(p.next + 2, 1u);
        si = __shfl_sync(kFull, si, 0);
        if (si >= p.n_sub) break;
        const uint32_t w = p.sub_win[si], j = p.sub_child[si];
        const uint64_t start = p.starts[w];
        const uint32_t n = p.lens[w];
        const uint32_t thr = p.thrs[w] ? p.thrs[w] : 1;
        const WRoot<MW> &R = roots[w];
        const uint32_t k = R.k;
        Mask<MW> T = m_zero<MW>(), req = m_zero<MW>();
        for (uint32_t q = j + 1 + lane; q < k; q += 32) m_set(T, R.f[q]);
        T = warp_or(T);
        const uint32_t e = R.f[j];
        m_set(req, e);
        Mask<MW> H = m_load<MW>(R.hp);
        m_set(H, e);
        const uint32_t sup = R.c[j];
        WRoot<MW> &S = subs[si];
        uint32_t n1 = 0, overflow = 0;
        if (m_nz(T)) {
            // the child's database through the ring's row of item e: only the window's
            // transactions holding e have their item masks read
            n1 = build_base<MW>(p, start, n, req, T, lists, lane);
            if (n1 == 0xffffffffu) {
                overflow = 1;
                n1 = 0;
            }
        }
        count_items<MW>(false, p, start, lists, 0, n1, T, cnt, lane);
        Mask<MW> P, F;
        classify<MW>(T, cnt, p.d, thr, sup, lane, P, F);
        uint32_t k1 = 0;
        Mask<MW> Hp, cand;
#pragma unroll
        for (int i = 0; i < MW; ++i) {
            Hp.w[i] = H.w[i] | P.w[i];
            cand.w[i] = Hp.w[i];
            k1 += __popcll(F.w[i]);
        }
        uint32_t has = 0, csup = 0;
        if (k1 == 0) {
            has = 1;   // Hp holds f_j
            csup = sup;
        } else {
            const uint32_t cf = count_superset<MW>(false, p, start, lists, 0, n1, F, lane);
            if (cf >= thr) {
                has = 1;
                csup = cf;
#pragma unroll
                for (int i = 0; i < MW; ++i) cand.w[i] |= F.w[i];
            }
        }
        if (!has) sort_tail<MW>(F, cnt, lane, S.f, S.c);
        if (lane < MW) {
            S.hp[lane] = m_word(Hp, lane);
            S.cand[lane] = m_word(cand, lane);
        }
        if (lane == 0) {
            S.cand_sup = csup;
            S.has_cand = has;
            S.k = has ? 0 : k1;
            S.overflow = overflow;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ tasks
template <int MW> __global__ void __launch_bounds__(128) wtask_kernel(WMineParams p) {
    __shared__ uint32_t s_cnt[4][128];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint32_t *cnt = s_cnt[wib];
    uint64_t *lists = p.lists + warp * (uint64_t)p.list_cap * MW;
    uint32_t *lmfi = p.lmfi + warp * (uint64_t)p.lmfi_cap;
    uint64_t *pool = p.pool_m + warp * (uint64_t)p.pool_cap * MW;
    uint32_t *pool_s = p.pool_s + warp * (uint64_t)p.pool_cap;
    WLevel<MW> *LV = reinterpret_cast<WLevel<MW> *>(p.levels) + warp * kWDepth;
    const WRoot<MW> *roots = reinterpret_cast<const WRoot<MW> *>(p.roots);
    const uint32_t d = p.d;

    for (;;) {
        uint32_t ti = 0;
        if (lane == 0) ti = atomicAdd(p.next, 1u);
        ti = __shfl_sync(kFull, ti, 0);
        if (ti >= p.n_tasks) break;
        const uint64_t t_begin = globaltimer_ns();
        const uint32_t t = p.task_order[ti];
        const uint32_t w = p.task_win[t];
        const uint32_t child = p.task_child[t];
        const uint32_t sub = p.task_sub ? p.task_sub[t] : kWholeWindow;
        const uint32_t gchild = p.task_gchild ? p.task_gchild[t] : kWholeWindow;
        const uint64_t start = p.starts[w];
        const uint32_t n = p.lens[w];
        const uint32_t thr = p.thrs[w] ? p.thrs[w] : 1;
        int status = 0;
        uint32_t np = 0;
        uint64_t nodes = 0;

        // the task's first node: the whole window, or child `child` of its root
        bool ring0 = child == kWholeWindow;
        Mask<MW> H = m_zero<MW>(), T = m_zero<MW>();
        uint32_t sup = n, list_n = n;
        bool done = false;   // a split child that is itself terminal: its one candidate
        if (ring0) {
            for (uint32_t e = 0; e < d; ++e) m_set(T, e);
        } else if (sub == kWholeWindow) {
            const WRoot<MW> &R = roots[w];
            const uint32_t k = R.k;
            for (uint32_t q = child + 1 + lane; q < k; q += 32) m_set(T, R.f[q]);
            T = warp_or(T);
            H = m_load<MW>(R.hp);
            Mask<MW> req = m_zero<MW>();
            m_set(req, R.f[child]);
            m_set(H, R.f[child]);
            sup = R.c[child];
            list_n = 0;
            if (m_nz(T)) {
                list_n = build_child<MW>(true, p, start, lists, 0, n, req, T, 0, lane);
                if (list_n == 0xffffffffu) status = 1;
            }
        } else {
            const WRoot<MW> &S = reinterpret_cast<const WRoot<MW> *>(p.subs)[sub];
            if (S.overflow) {
                status = 1;
            } else if (gchild == kWholeWindow) {
                if (lane < MW) pool[lane] = S.cand[lane];
                if (lane == 0) pool_s[0] = S.cand_sup;
                np = 1;
                nodes = 1;
                done = true;
            } else {
                const uint32_t k1 = S.k;
                for (uint32_t q = gchild + 1 + lane; q < k1; q += 32) m_set(T, S.f[q]);
                T = warp_or(T);
                H = m_load<MW>(S.hp);
                Mask<MW> req = m_zero<MW>();
                m_set(req, roots[w].f[child]);
                m_set(req, S.f[gchild]);
                m_set(H, S.f[gchild]);
                sup = S.c[gchild];
                list_n = 0;
                if (m_nz(T)) {
                    list_n = build_child<MW>(true, p, start, lists, 0, n, req, T, 0, lane);
                    if (list_n == 0xffffffffu) status = 1;
                }
            }
        }
        int l = 0;
        uint64_t list_off = 0;
        uint32_t lm_off = 0, lm_n = 0, entry = 0;
        bool expand = true;

        while (status == 0 && !done) {
            if (expand) {
                expand = false;
                ++nodes;
                const bool ring = ring0 && l == 0;
                count_items<MW>(ring, p, start, lists, list_off, list_n, T, cnt, lane);
                Mask<MW> P, F;
                classify<MW>(T, cnt, d, thr, sup, lane, P, F);
                Mask<MW> Hp, Q;
                uint32_t k = 0;
#pragma unroll
                for (int i = 0; i < MW; ++i) {
                    Hp.w[i] = H.w[i] | P.w[i];
                    Q.w[i] = Hp.w[i] | F.w[i];
                    k += __popcll(F.w[i]);
                }
                // ---- is H u P u F inside a known MFI?  (local list; nothing was found since entry)
                bool hit = false;
                for (uint32_t b = 0; b < lm_n && !hit; b += 32 * kU) {
                    uint32_t idx[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t i = b + u * 32 + lane;
                        idx[u] = i < lm_n ? lmfi[lm_off + i] : 0xffffffffu;
                    }
                    bool h = false;
#pragma unroll
                    for (int u = 0; u < kU; ++u)
                        if (idx[u] != 0xffffffffu) h |= m_sub(Q, m_load<MW>(pool + (uint64_t)idx[u] * MW));
                    hit = __any_sync(kFull, h);
                }
                if (k == 0 || hit) {
                    if (k == 0 && !hit && m_nz(Hp)) {
                        if (np >= p.pool_cap) { status = 1; break; }
                        if (lane < MW) pool[(uint64_t)np * MW + lane] = m_word(Hp, lane);
                        if (lane == 0) pool_s[np] = sup;
                        ++np;
                    }
                    if (l == 0) break;
                    --l;
                    __syncwarp();
                    continue;
                }
                // ---- FHUT: support of H u P u F
                const uint32_t cf = count_superset<MW>(ring, p, start, lists, list_off, list_n, F, lane);
                if (cf >= thr) {
                    if (np >= p.pool_cap) { status = 1; break; }
                    if (lane < MW) pool[(uint64_t)np * MW + lane] = m_word(Q, lane);
                    if (lane == 0) pool_s[np] = cf;
                    ++np;
                    if (l == 0) break;
                    --l;
                    __syncwarp();
                    continue;
                }
                // ---- record the node: frequent tail sorted by (support, id)
                WLevel<MW> &A = LV[l];
                sort_tail<MW>(F, cnt, lane, A.f, A.c);
                if (lane < MW) A.hp[lane] = m_word(Hp, lane);
                if (lane == 0) {
                    A.list_off = list_off;
                    A.list_n = list_n;
                    A.lm_off = lm_off;
                    A.lm_n = lm_n;
                    A.entry = entry;
                    A.k = k;
                    A.j = 0;
                }
                __syncwarp();
            }
            // ---- next child of level l, or up
            WLevel<MW> &A = LV[l];
            const uint32_t j = A.j, k = A.k;
            if (j >= k) {
                if (l == 0) break;
                --l;
                continue;
            }
            __syncwarp();
            if (lane == 0) A.j = j + 1;
            const uint32_t e = A.f[j];
            const uint32_t csup = A.c[j];
            Mask<MW> Tc = m_zero<MW>();
            for (uint32_t q = j + 1 + lane; q < k; q += 32) m_set(Tc, A.f[q]);
            Tc = warp_or(Tc);
            Mask<MW> Hc = m_load<MW>(A.hp);
            m_set(Hc, e);
            const bool pring = ring0 && l == 0;
            const uint64_t p_off = A.list_off;
            const uint32_t p_n = A.list_n;
            const uint64_t c_off = pring ? 0 : p_off + p_n;
            uint32_t cn = 0;
            if (m_nz(Tc)) {
                Mask<MW> req = m_zero<MW>();
                m_set(req, e);
                cn = build_child<MW>(pring, p, start, lists, p_off, p_n, req, Tc, c_off, lane);
                if (cn == 0xffffffffu) { status = 1; break; }
            }
            // child local-MFI list: members containing the child's head
            const uint32_t c_lm = A.lm_off + A.lm_n;
            const uint32_t p_lm_off = A.lm_off, p_lm_n = A.lm_n, p_entry = A.entry;
            const uint32_t n_src = p_lm_n + (np - p_entry);
            uint32_t ln = 0;
            for (uint32_t b = 0; b < n_src; b += 32 * kU) {
                uint32_t idx[kU];
                bool keep[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t i = b + u * 32 + lane;
                    idx[u] = 0;
                    keep[u] = false;
                    if (i < n_src) idx[u] = i < p_lm_n ? lmfi[p_lm_off + i] : p_entry + (i - p_lm_n);
                }
#pragma unroll
                for (int u = 0; u < kU; ++u)
                    if (b + u * 32 + lane < n_src) keep[u] = m_sub(Hc, m_load<MW>(pool + (uint64_t)idx[u] * MW));
                // the child's list goes after the parent's: writes never touch indices still to be read
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t bal = __ballot_sync(kFull, keep[u]);
                    const uint64_t pos = (uint64_t)c_lm + ln + __popc(bal & ((1u << lane) - 1));
                    if (keep[u] && pos < p.lmfi_cap) lmfi[pos] = idx[u];
                    ln += __popc(bal);
                }
            }
            if ((uint64_t)c_lm + ln > p.lmfi_cap) { status = 1; break; }
            if (l + 1 >= kWDepth) { status = 1; break; }
            __syncwarp();
            ++l;
            H = Hc;
            T = Tc;
            sup = csup;
            list_off = c_off;
            list_n = cn;
            lm_off = c_lm;
            lm_n = ln;
            entry = np;
            expand = true;
        }

        // ---- publish the task's candidates
        uint64_t off = 0;
        if (status == 0) {
            if (lane == 0) off = atomicAdd(p.out_pos, (unsigned long long)np);
            off = __shfl_sync(kFull, off, 0);
            if (off + np > p.out_cap) {
                status = 2;
            } else {
                __syncwarp();
                for (uint32_t i = lane; i < np * MW; i += 32) p.out_m[off * MW + i] = pool[i];
                for (uint32_t i = lane; i < np; i += 32) p.out_s[off + i] = pool_s[i];
            }
        }
        if (lane == 0) {
            p.task_off[t] = off;
            p.task_cnt[t] = status == 0 ? np : 0;
            p.task_status[t] = status;
            p.task_nodes[t] = nodes;
            if (p.task_ns) p.task_ns[t] = globaltimer_ns() - t_begin;
        }
        __syncwarp();
    }
}

// Resident CTAs per SM the register allocation is fitted to.  Measured on the
// 4,096 service windows: 6 (80 registers, 3,648 warps) 337 ms, 7 (72 registers,
// 4,176 warps, the workspace budget's limit) 338 ms with a longer makespan, 8
// (64 registers, spills) 358 ms -- more resident warps do not shorten the search.
#ifndef SGFIM_WVTASK_MIN_BLOCKS
#define SGFIM_WVTASK_MIN_BLOCKS 6
#endif

template <int MW> __global__ void __launch_bounds__(128, SGFIM_WVTASK_MIN_BLOCKS) wvtask_kernel(WMineParams p) {
    __shared__ uint32_t s_cnt[4][128];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t warp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint32_t *cnt = s_cnt[wib];
    uint64_t *lists = p.lists + warp * (uint64_t)p.list_cap * MW;
    uint32_t *lmfi = p.lmfi + warp * (uint64_t)p.lmfi_cap;
    uint64_t *pool = p.pool_m + warp * (uint64_t)p.pool_cap * MW;
    uint32_t *pool_s = p.pool_s + warp * (uint64_t)p.pool_cap;
    WLevel<MW> *LV = reinterpret_cast<WLevel<MW> *>(p.levels) + warp * kWDepth;
    const WRoot<MW> *roots = reinterpret_cast<const WRoot<MW> *>(p.roots);
    const uint32_t d = p.d;
    const uint32_t vw = p.v_words;
    uint32_t *vrows = p.vbuf + warp * (uint64_t)(128 + kWDepth) * vw;   // row slot s: vrows + s * vw
    uint32_t *vtid = vrows + (uint64_t)128 * vw;                        // level l: vtid + l * vw

    for (;;) {
        uint32_t ti = 0;
        if (lane == 0) ti = atomicAdd(p.next, 1u);
        ti = __shfl_sync(kFull, ti, 0);
        if (ti >= p.n_tasks) break;
        const uint64_t t_begin = globaltimer_ns();
        const uint32_t t = p.task_order[ti];
        const uint32_t w = p.task_win[t];
        const uint32_t child = p.task_child[t];
        const uint32_t sub = p.task_sub ? p.task_sub[t] : kWholeWindow;
        const uint32_t gchild = p.task_gchild ? p.task_gchild[t] : kWholeWindow;
        const uint64_t start = p.starts[w];
        const uint32_t n = p.lens[w];
        const uint32_t thr = p.thrs[w] ? p.thrs[w] : 1;
        int status = 0;
        uint32_t np = 0;
        uint64_t nodes = 0;

        // the task's first node: the whole window, or child `child` of its root
        bool ring0 = child == kWholeWindow;
        Mask<MW> H = m_zero<MW>(), T = m_zero<MW>();
        uint32_t sup = n, list_n = n;
        bool done = false;   // a split child that is itself terminal: its one candidate
        if (ring0) {
            for (uint32_t e = 0; e < d; ++e) m_set(T, e);
            list_n = build_base<MW>(p, start, n, m_zero<MW>(), T, lists, lane);
            if (list_n == 0xffffffffu) status = 1;
        } else if (sub == kWholeWindow) {
            const WRoot<MW> &R = roots[w];
            const uint32_t k = R.k;
            for (uint32_t q = child + 1 + lane; q < k; q += 32) m_set(T, R.f[q]);
            T = warp_or(T);
            H = m_load<MW>(R.hp);
            Mask<MW> req = m_zero<MW>();
            m_set(req, R.f[child]);
            m_set(H, R.f[child]);
            sup = R.c[child];
            list_n = 0;
            if (m_nz(T)) {
                list_n = build_base<MW>(p, start, n, req, T, lists, lane);
                if (list_n == 0xffffffffu) status = 1;
            }
        } else {
            const WRoot<MW> &S = reinterpret_cast<const WRoot<MW> *>(p.subs)[sub];
            if (S.overflow) {
                status = 1;
            } else if (gchild == kWholeWindow) {
                if (lane < MW) pool[lane] = S.cand[lane];
                if (lane == 0) pool_s[0] = S.cand_sup;
                np = 1;
                nodes = 1;
                done = true;
            } else {
                const uint32_t k1 = S.k;
                for (uint32_t q = gchild + 1 + lane; q < k1; q += 32) m_set(T, S.f[q]);
                T = warp_or(T);
                H = m_load<MW>(S.hp);
                Mask<MW> req = m_zero<MW>();
                m_set(req, roots[w].f[child]);
                m_set(req, S.f[gchild]);
                m_set(H, S.f[gchild]);
                sup = S.c[gchild];
                list_n = 0;
                if (m_nz(T)) {
                    list_n = build_base<MW>(p, start, n, req, T, lists, lane);
                    if (list_n == 0xffffffffu) status = 1;
                }
            }
        }
        // ---- the task's database as vertical rows over its entries (one row per item of T0)
        const Mask<MW> T0 = T;
        const uint32_t W = (list_n + 31) / 32;
        if (status == 0 && !done) {
            if (W > vw) {
                status = 1;
            } else {
                build_rows<MW>(lists, list_n, T0, vrows, vw, lane);
                for (uint32_t x = lane; x < W; x += 32)
                    vtid[x] = (x + 1 < W || (list_n & 31) == 0) ? 0xffffffffu : ((1u << (list_n & 31)) - 1);
                __syncwarp();
            }
        }
        int l = 0;
        uint32_t lm_off = 0, lm_n = 0, entry = 0;
        bool expand = true;

        while (status == 0 && !done) {
            if (expand) {
                expand = false;
                ++nodes;
                const uint32_t *tid = vtid + (uint64_t)l * vw;
                vcount<MW>(tid, vrows, vw, W, T, T0, cnt, lane);
                Mask<MW> P, F;
                classify<MW>(T, cnt, d, thr, sup, lane, P, F);
                Mask<MW> Hp, Q;
                uint32_t k = 0;
#pragma unroll
                for (int i = 0; i < MW; ++i) {
                    Hp.w[i] = H.w[i] | P.w[i];
                    Q.w[i] = Hp.w[i] | F.w[i];
                    k += __popcll(F.w[i]);
                }
                // ---- is H u P u F inside a known MFI?  (local list; nothing was found since entry)
                bool hit = false;
                for (uint32_t b = 0; b < lm_n && !hit; b += 32 * kU) {
                    uint32_t idx[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t i = b + u * 32 + lane;
                        idx[u] = i < lm_n ? lmfi[lm_off + i] : 0xffffffffu;
                    }
                    bool h = false;
#pragma unroll
                    for (int u = 0; u < kU; ++u)
                        if (idx[u] != 0xffffffffu) h |= m_sub(Q, m_load<MW>(pool + (uint64_t)idx[u] * MW));
                    hit = __any_sync(kFull, h);
                }
                if (k == 0 || hit) {
                    if (k == 0 && !hit && m_nz(Hp)) {
                        if (np >= p.pool_cap) { status = 1; break; }
                        if (lane < MW) pool[(uint64_t)np * MW + lane] = m_word(Hp, lane);
                        if (lane == 0) pool_s[np] = sup;
                        ++np;
                    }
                    if (l == 0) break;
                    --l;
                    __syncwarp();
                    continue;
                }
                // ---- FHUT: support of H u P u F
                const uint32_t cf = vcount_superset<MW>(tid, vrows, vw, W, F, T0, lane);
                if (cf >= thr) {
                    if (np >= p.pool_cap) { status = 1; break; }
                    if (lane < MW) pool[(uint64_t)np * MW + lane] = m_word(Q, lane);
                    if (lane == 0) pool_s[np] = cf;
                    ++np;
                    if (l == 0) break;
                    --l;
                    __syncwarp();
                    continue;
                }
                // ---- record the node: frequent tail sorted by (support, id)
                WLevel<MW> &A = LV[l];
                sort_tail<MW>(F, cnt, lane, A.f, A.c);
                if (lane < MW) A.hp[lane] = m_word(Hp, lane);
                if (lane == 0) {
                    A.lm_off = lm_off;
                    A.lm_n = lm_n;
                    A.entry = entry;
                    A.k = k;
                    A.j = 0;
                }
                __syncwarp();
            }
            // ---- next child of level l, or up
            WLevel<MW> &A = LV[l];
            const uint32_t j = A.j, k = A.k;
            if (j >= k) {
                if (l == 0) break;
                --l;
                continue;
            }
            __syncwarp();
            if (lane == 0) A.j = j + 1;
            const uint32_t e = A.f[j];
            const uint32_t csup = A.c[j];
            Mask<MW> Tc = m_zero<MW>();
            for (uint32_t q = j + 1 + lane; q < k; q += 32) m_set(Tc, A.f[q]);
            Tc = warp_or(Tc);
            Mask<MW> Hc = m_load<MW>(A.hp);
            m_set(Hc, e);
            {
                // child tidset = parent tidset AND row(e)
                const uint32_t *ptid = vtid + (uint64_t)l * vw;
                uint32_t *ctid = vtid + (uint64_t)(l + 1) * vw;
                const uint32_t *row = vrows + (uint64_t)m_rank(T0, e) * vw;
                if (l + 1 < kWDepth)
                    for (uint32_t x = lane; x < W; x += 32) ctid[x] = ptid[x] & row[x];
            }
            // child local-MFI list: members containing the child's head
            const uint32_t c_lm = A.lm_off + A.lm_n;
            const uint32_t p_lm_off = A.lm_off, p_lm_n = A.lm_n, p_entry = A.entry;
            const uint32_t n_src = p_lm_n + (np - p_entry);
            uint32_t ln = 0;
            for (uint32_t b = 0; b < n_src; b += 32 * kU) {
                uint32_t idx[kU];
                bool keep[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t i = b + u * 32 + lane;
                    idx[u] = 0;
                    keep[u] = false;
                    if (i < n_src) idx[u] = i < p_lm_n ? lmfi[p_lm_off + i] : p_entry + (i - p_lm_n);
                }
#pragma unroll
                for (int u = 0; u < kU; ++u)
                    if (b + u * 32 + lane < n_src) keep[u] = m_sub(Hc, m_load<MW>(pool + (uint64_t)idx[u] * MW));
                // the child's list goes after the parent's: writes never touch indices still to be read
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t bal = __ballot_sync(kFull, keep[u]);
                    const uint64_t pos = (uint64_t)c_lm + ln + __popc(bal & ((1u << lane) - 1));
                    if (keep[u] && pos < p.lmfi_cap) lmfi[pos] = idx[u];
                    ln += __popc(bal);
                }
            }
            if ((uint64_t)c_lm + ln > p.lmfi_cap) { status = 1; break; }
            if (l + 1 >= kWDepth) { status = 1; break; }
            __syncwarp();
            ++l;
            H = Hc;
            T = Tc;
            sup = csup;
            lm_off = c_lm;
            lm_n = ln;
            entry = np;
            expand = true;
        }

        // ---- publish the task's candidates
        uint64_t off = 0;
        if (status == 0) {
            if (lane == 0) off = atomicAdd(p.out_pos, (unsigned long long)np);
            off = __shfl_sync(kFull, off, 0);
            if (off + np > p.out_cap) {
                status = 2;
            } else {
                __syncwarp();
                for (uint32_t i = lane; i < np * MW; i += 32) p.out_m[off * MW + i] = pool[i];
                for (uint32_t i = lane; i < np; i += 32) p.out_s[off + i] = pool_s[i];
            }
        }
        if (lane == 0) {
            p.task_off[t] = off;
            p.task_cnt[t] = status == 0 ? np : 0;
            p.task_status[t] = status;
            p.task_nodes[t] = nodes;
            if (p.task_ns) p.task_ns[t] = globaltimer_ns() - t_begin;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ cross-task filter
// One CTA per split window: the window's candidates in task order (subtrees
// in depth-first order) get a vertical bitmap rows[e][q]; candidate q of a
// task is dropped when the AND of its items' rows has a bit below the task's
// first candidate.  keep[] is written per arena slot, kept[] per task.
template <int MW> __global__ void __launch_bounds__(1024) wfilter_kernel(WFilterParams p) {
    __shared__ uint32_t s_w;
    __shared__ uint32_t s_freq[64 * MW];              // candidates holding each item
    __shared__ uint32_t s_lo[64 * MW], s_hi[64 * MW];  // first / last word of each item's row with a bit
    uint64_t *rows = p.scratch + (uint64_t)blockIdx.x * p.scratch_words;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_w = atomicAdd(p.next, 1u);
        for (uint32_t i = threadIdx.x; i < 64 * MW; i += blockDim.x) {
            s_freq[i] = 0;
            s_lo[i] = 0xffffffffu;
            s_hi[i] = 0;
        }
        __syncthreads();
        const uint32_t wi = s_w;
        if (wi >= p.n_win) break;
        const uint32_t e0 = p.win_task0[wi], e1 = p.win_task0[wi + 1];   // entries of this window, task order
        const uint64_t M = p.win_total[wi];
        const uint64_t W = (M + 63) / 64;
        if (W * p.d > p.scratch_words) {
            if (threadIdx.x == 0) p.win_status[wi] = 1;
            continue;
        }
        for (uint64_t i = threadIdx.x; i < W * p.d; i += blockDim.x) rows[i] = 0;
        __syncthreads();
        // candidate q (window order) -> entry (binary search over first[]), arena slot
        auto locate = [&](uint64_t q) {
            uint32_t lo = e0, hi = e1 - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (p.task_first[mid] <= q) lo = mid;
                else hi = mid - 1;
            }
            return lo;
        };
        for (uint64_t q = threadIdx.x; q < M; q += blockDim.x) {
            const uint32_t en = locate(q);
            const uint64_t slot = p.task_off[p.task_of[en]] + (q - p.task_first[en]);
            const Mask<MW> m = m_load<MW>(p.out_m + slot * MW);
#pragma unroll
            for (int ww = 0; ww < MW; ++ww) {
                uint64_t x = m.w[ww];
                while (x) {
                    const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
                    x &= x - 1;
                    atomicOr(reinterpret_cast<unsigned long long *>(rows + (uint64_t)e * W + (q >> 6)),
                             1ull << (q & 63));
                    atomicAdd(&s_freq[e], 1u);
                    atomicMin(&s_lo[e], (uint32_t)(q >> 6));
                    atomicMax(&s_hi[e], (uint32_t)(q >> 6));
                }
            }
        }
        __syncthreads();
        for (uint64_t q = threadIdx.x; q < M; q += blockDim.x) {
            const uint32_t en = locate(q);
            const uint32_t t = p.task_of[en];
            const uint64_t slot = p.task_off[t] + (q - p.task_first[en]);
            bool keep = true;
            const uint64_t lim = p.task_first[en];   // candidates of earlier subtrees: [0, lim)
            if (lim) {
                const Mask<MW> m = m_load<MW>(p.out_m + slot * MW);
                // the candidate's rarest item drives the scan: its row has the fewest bits
                uint32_t ef = 0, best = 0xffffffffu;
#pragma unroll
                for (int ww = 0; ww < MW; ++ww) {
                    uint64_t x = m.w[ww];
                    while (x) {
                        const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
                        x &= x - 1;
                        if (s_freq[e] < best) {
                            best = s_freq[e];
                            ef = e;
                        }
                    }
                }
                const uint64_t wd_end = (lim + 63) / 64;
                const uint64_t hi = (uint64_t)s_hi[ef] + 1 < wd_end ? (uint64_t)s_hi[ef] + 1 : wd_end;
                for (uint64_t wd = s_lo[ef]; wd < hi && keep; ++wd) {
                    uint64_t v = rows[(uint64_t)ef * W + wd];
                    if (wd * 64 + 64 > lim) v &= (1ull << (lim - wd * 64)) - 1;
#pragma unroll
                    for (int ww = 0; ww < MW; ++ww) {
                        uint64_t x = m.w[ww];
                        while (x && v) {
                            const uint32_t e = ww * 64 + (__ffsll((long long)x) - 1);
                            x &= x - 1;
                            v &= rows[(uint64_t)e * W + wd];
                        }
                    }
                    keep = v == 0;
                }
            }
            p.keep[slot] = keep ? 1 : 0;
            if (!keep) atomicSub(&p.task_kept[t], 1u);
        }
    }
}

// ------------------------------------------------------------------ gather
// One warp per task: its kept candidates, in emission order, to dst.
template <int MW> __global__ void __launch_bounds__(128) wgather_kernel(WGatherParams p) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = warp; t < p.n_tasks; t += n_warps) {
        const uint64_t src = p.task_off[t];
        const uint32_t n = p.task_cnt[t];
        uint64_t dst = p.task_dst[t];
        if (dst == ~0ull) continue;
        for (uint32_t b = 0; b < n; b += 32) {
            const uint32_t i = b + lane;
            const bool keep = i < n && (!p.keep || p.keep[src + i]);
            const uint32_t bal = __ballot_sync(kFull, keep);
            if (keep) {
                const uint64_t pos = dst + __popc(bal & ((1u << lane) - 1));
                m_store<MW>(p.dst_m + pos * MW, m_load<MW>(p.out_m + (src + i) * MW));
                p.dst_s[pos] = p.out_s[src + i];
            }
            dst += __popc(bal);
        }
    }
}

int wmine_depth() { return kWDepth; }

int wtask_blocks_per_sm(bool vertical) {
    int blocks = 0;
    if (vertical) SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, wvtask_kernel<2>, 128, 0));
    else SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, wtask_kernel<2>, 128, 0));
    return blocks > 0 ? blocks : 1;
}
size_t wmine_level_bytes(int mw) { return mw == 2 ? sizeof(WLevel<2>) * kWDepth : 0; }
size_t wmine_root_bytes(int mw) { return mw == 2 ? sizeof(WRoot<2>) : 0; }

void launch_wroot(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "batched window miner supports 2 mask words", __FILE__, __LINE__);
    wroot_kernel<2><<<blocks, 128, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}
void launch_wsub(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "batched window miner supports 2 mask words", __FILE__, __LINE__);
    wsub_kernel<2><<<blocks, 128, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}
void launch_wtask(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "batched window miner supports 2 mask words", __FILE__, __LINE__);
    if (p.vbuf)
        wvtask_kernel<2><<<blocks, 128, 0, st>>>(p);
    else
        wtask_kernel<2><<<blocks, 128, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}
void launch_wfilter(const WFilterParams &p, int mw, unsigned blocks, unsigned threads, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "batched window miner supports 2 mask words", __FILE__, __LINE__);
    if (threads != 256 && threads != 1024)
        throw CudaError(cudaErrorInvalidValue, "filter blocks are 256 or 1,024 threads", __FILE__, __LINE__);
    wfilter_kernel<2><<<blocks, threads, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}
void launch_wgather(const WGatherParams &p, int mw, unsigned blocks, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "batched window miner supports 2 mask words", __FILE__, __LINE__);
    wgather_kernel<2><<<blocks, 128, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}

}  // namespace sg
