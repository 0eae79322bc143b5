// kernels_wmine.cu -- batched per-window MFI miner: one warp mines one window.
//
// The reference mines one window per engine process (code/pipeline/
// skab_spike.py:61-80 builds the windows; the engines' DFS is
// kernel_bitmap.cu:841-894); its result for a window is the MFI set of that
// window's transactions at the window's floor, which this kernel reproduces.
//
// Representation.  Items are the ring's dense ids 0..d-1 (d <= 64*MW); an
// itemset is an MW-word mask.  A search node (H, T) holds its projected
// database: one MW-word entry per transaction of t(H) that still contains a
// tail item, restricted to T (transactions whose restriction is empty add
// nothing to any count below the node and are dropped).  The root's database
// is the window itself, read from the ring's horizontal masks.
//
// Search.  Sequential depth-first over the set-enumeration tree, one node at
// a time, children in ascending (support, id) order -- the order under which
// a candidate found later is never a proper superset of one found earlier:
// child j's subtree lacks item f_i of every earlier sibling i < j, which all
// candidates of sibling i contain.  Every node applies
//   counts  c_e = |t(H u {e})|, e in T       (ballot popcounts over entries)
//   PEP     c_e == sup(H) (and >= thr)       -> e joins H
//   leaf    F = {e : thr <= c_e < sup(H)} empty: H is a candidate
//   HUT     H u F inside a known MFI          -> nothing new below
//   FHUT    |t(H u F)| >= thr                  -> H u F is the only candidate
// and candidates are checked against the MFIs found so far that contain the
// node's head (the "local MFI" list: the parent's list filtered to members
// containing the child's head, plus everything found inside the parent's
// subtree, which contains the parent's head by construction).  A candidate
// that passes is maximal, so the window's pool is its exact MFI set.
//
// Work is distributed by an atomic window counter (largest windows first);
// every loop is bounded by list lengths, and any capacity overflow (list
// stack, local-MFI stack, pool, depth) marks the window for the host-driven
// wave miner instead of producing a partial result.
#include "common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <int MW> struct Mask {
    uint64_t w[MW];
};

template <int MW> __device__ __forceinline__ bool m_has(const Mask<MW> &m, uint32_t e) {
    uint64_t x = 0;
#pragma unroll
    for (int k = 0; k < MW; ++k)
        if ((uint32_t)k == (e >> 6)) x = m.w[k];
    return (x >> (e & 63)) & 1ull;
}
template <int MW> __device__ __forceinline__ void m_set(Mask<MW> &m, uint32_t e) {
#pragma unroll
    for (int k = 0; k < MW; ++k)
        if ((uint32_t)k == (e >> 6)) m.w[k] |= 1ull << (e & 63);
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
// word i of m without a dynamically indexed register array
template <int MW> __device__ __forceinline__ uint64_t m_word(const Mask<MW> &m, uint32_t i) {
    uint64_t r = 0;
#pragma unroll
    for (int k = 0; k < MW; ++k)
        if ((uint32_t)k == i) r = m.w[k];
    return r;
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
    uint64_t hp[MW];      // head after PEP
    uint64_t list_off;    // first entry of this node's projected database (levels >= 1)
    uint32_t list_n;
    uint32_t lm_off, lm_n;  // local-MFI list (pool indices)
    uint32_t entry;       // pool size when the node was entered
    uint32_t k, j;        // frequent tail size, next child
    uint8_t f[128];       // frequent tail, ascending (support, id)
    uint32_t c[128];      // supports of f
};

// The search stack holds itemsets of up to kWDepth - 1 items.
constexpr int kWDepth = 48;
// chunks of 32 entries loaded before any is processed (memory-level parallelism)
constexpr int kU = 4;

}  // namespace

template <int MW> __global__ void __launch_bounds__(128) wmine_kernel(WMineParams p) {
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
    const uint32_t d = p.d;

    for (;;) {
        uint32_t wi = 0;
        if (lane == 0) wi = atomicAdd(p.next, 1u);
        wi = __shfl_sync(kFull, wi, 0);
        if (wi >= p.n_win) break;
        const uint32_t w = p.order[wi];
        const uint64_t start = p.starts[w];
        const uint32_t n = p.lens[w];
        const uint32_t thr = p.thrs[w] ? p.thrs[w] : 1;
        int status = 0;
        uint32_t np = 0;
        uint64_t nodes = 0;

        // current node
        int l = 0;
        Mask<MW> H = m_zero<MW>(), T = m_zero<MW>();
        for (uint32_t e = 0; e < d; ++e) m_set(T, e);
        uint32_t sup = n;
        uint64_t list_off = 0;
        uint32_t list_n = n;       // root: the window in the ring
        uint32_t lm_off = 0, lm_n = 0, entry = 0;
        bool expand = true;

        while (status == 0) {
            if (expand) {
                expand = false;
                ++nodes;
                const bool root = l == 0;
                // ---- counts over the projected database
                for (uint32_t q = lane; q < 128; q += 32) cnt[q] = 0;
                __syncwarp();
                for (uint32_t b = 0; b < list_n; b += 32 * kU) {
                    Mask<MW> m[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t i = b + u * 32 + lane;
                        m[u] = m_zero<MW>();
                        if (i < list_n) {
                            const uint64_t *src =
                                root ? p.hm + ((start + i) & p.cap_mask) * MW : lists + (list_off + i) * MW;
                            m[u] = m_and(m_load<MW>(src), T);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const Mask<MW> om = warp_or(m[u]);
#pragma unroll
                        for (int ww = 0; ww < MW; ++ww) {
                            uint64_t x = om.w[ww];
                            while (x) {
                                const uint32_t bit = __ffsll((long long)x) - 1;
                                x &= x - 1;
                                const uint32_t c = __popc(__ballot_sync(kFull, (m[u].w[ww] >> bit) & 1ull));
                                if (lane == 0) cnt[ww * 64 + bit] += c;
                            }
                        }
                    }
                }
                __syncwarp();
                // ---- PEP and the frequent tail
                Mask<MW> P = m_zero<MW>(), F = m_zero<MW>();
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
                uint32_t cf = 0;
                for (uint32_t b = 0; b < list_n; b += 32 * kU) {
                    bool h[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t i = b + u * 32 + lane;
                        h[u] = false;
                        if (i < list_n) {
                            const uint64_t *src =
                                root ? p.hm + ((start + i) & p.cap_mask) * MW : lists + (list_off + i) * MW;
                            h[u] = m_sub(F, m_load<MW>(src));
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kU; ++u) cf += __popc(__ballot_sync(kFull, h[u]));
                }
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
#pragma unroll
                for (int q = 0; q < 2 * MW; ++q) {
                    const uint32_t e = q * 32 + lane;
                    const bool isF = (F.w[q >> 1] >> ((q & 1) * 32 + lane)) & 1ull;
                    const uint32_t ce = isF ? cnt[e] : 0;
                    uint32_t rank = 0;
#pragma unroll
                    for (int ww = 0; ww < MW; ++ww) {
                        uint64_t x = F.w[ww];
                        while (x) {
                            const uint32_t e2 = ww * 64 + (__ffsll((long long)x) - 1);
                            x &= x - 1;
                            const uint32_t c2 = cnt[e2];
                            rank += (c2 < ce) || (c2 == ce && e2 < e);
                        }
                    }
                    if (isF) {
                        A.f[rank] = (uint8_t)e;
                        A.c[rank] = ce;
                    }
                }
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
            for (uint32_t q = j + 1 + lane; q < k; q += 32) {
                m_set(Tc, A.f[q]);
            }
            Tc = warp_or(Tc);
            Mask<MW> Hc = m_load<MW>(A.hp);
            m_set(Hc, e);
            const bool proot = l == 0;
            const uint64_t p_off = A.list_off;
            const uint32_t p_n = A.list_n;
            // child database: entries with e, restricted to the child's tail, non-empty
            const uint64_t c_off = proot ? 0 : p_off + p_n;
            uint32_t cn = 0;
            if (m_nz(Tc)) {
                for (uint32_t b = 0; b < p_n; b += 32 * kU) {
                    Mask<MW> m[kU];
                    bool keep[kU];
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t i = b + u * 32 + lane;
                        m[u] = m_zero<MW>();
                        keep[u] = false;
                        if (i < p_n) {
                            const uint64_t *src =
                                proot ? p.hm + ((start + i) & p.cap_mask) * MW : lists + (p_off + i) * MW;
                            const Mask<MW> r = m_load<MW>(src);
                            m[u] = m_and(r, Tc);
                            keep[u] = m_has(r, e) && m_nz(m[u]);
                        }
                    }
                    // the child's entries go after the parent's: writes never touch entries still to be read
#pragma unroll
                    for (int u = 0; u < kU; ++u) {
                        const uint32_t bal = __ballot_sync(kFull, keep[u]);
                        const uint64_t pos = c_off + cn + __popc(bal & ((1u << lane) - 1));
                        if (keep[u] && pos < p.list_cap) m_store(lists + pos * MW, m[u]);
                        cn += __popc(bal);
                    }
                }
                if (c_off + cn > p.list_cap) { status = 1; break; }
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

        // ---- publish the window's MFIs
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
            p.win_off[w] = off;
            p.win_cnt[w] = status == 0 ? np : 0;
            p.win_status[w] = status;
            p.win_nodes[w] = nodes;
        }
        __syncwarp();
    }
}

size_t wmine_level_bytes(int mw) {
    return mw == 2 ? sizeof(WLevel<2>) * kWDepth : 0;
}

void launch_wmine(const WMineParams &p, int mw, unsigned blocks, cudaStream_t st) {
    if (mw != 2) throw CudaError(cudaErrorInvalidValue, "wmine supports 2 mask words", __FILE__, __LINE__);
    wmine_kernel<2><<<blocks, 128, 0, st>>>(p);
    SG_CUDA_TRY(cudaGetLastError());
}

}  // namespace sg
