// kernels_lane.cu -- batched supports with one lane per candidate.
//
// Reference counterpart: the per-candidate AND-popcount loop of
// getResFrequencyCudaKernel (code/engine_tensorfim/code/engine/src/kernel_bitmap.cu:412-442,
// one launch per DFS node there) and the wave engine's counting
// (kernel_bmma.cu:603-768); here a million arbitrary k-item candidates share
// one launch and every bitmap chunk is staged once per CTA.
//
// Layout.  A CTA sweeps the transactions in chunks of 1,024 (16 words = 128
// bytes of every row).  TMA copies the chunk of all d rows into shared memory,
// row r at r * 128 bytes.  Each lane owns one candidate: it ANDs the 128-byte
// slices of the candidate's k rows in eight 16-byte pieces and accumulates the
// popcount.  Lane q of an 8-lane phase of a 128-bit shared load reads piece
// (i XOR q) at step i, so the eight lanes of a phase always touch eight
// distinct 16-byte bank groups -- conflict-free whatever rows they read.
//
// Candidates are sorted by k (descending) on the device, so the 32 lanes of a
// warp almost always share k and run one fully unrolled loop of 8k
// independent loads.  Groups of 32 consecutive sorted candidates ("sets") are
// dealt round-robin to the CTAs, so every CTA gets the same mix of k; inside a
// CTA, warps take sets from a shared counter, largest k first, once per chunk,
// and per-candidate totals live in shared memory.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sg {
namespace {

constexpr uint32_t kLaneRowsPerBox = 256;
constexpr uint32_t kLaneWords = 16;                                     // words per row per chunk
constexpr uint32_t kLaneBoxBytes = kLaneRowsPerBox * kLaneWords * 8;   // 32 KB
constexpr int kLaneThreads = 1024;
constexpr uint32_t kLaneBins = 8;       // k = 8 .. 1 (bin = 8 - k)
constexpr uint32_t kLaneTile = 256;     // candidates per prep tile (one per thread)
constexpr size_t kMaxSmem = 227 * 1024;
constexpr uint32_t kLaneMaxD = 4096;    // row ids travel in 12 bits of a record's first slot

// Record: eight 16-bit row ids; slots at and past k repeat item 0 (ANDing a
// row twice changes nothing); bits 12..15 of slot 0 hold k.
__device__ __forceinline__ int cand_bin(const uint64_t *__restrict__ cand_ptr, const uint32_t *__restrict__ items,
                                        uint64_t c, uint32_t d, uint16_t (&it)[8], uint32_t &k) {
    const uint64_t a = cand_ptr[c], b = cand_ptr[c + 1];
    const uint64_t kk = b - a;
    k = (uint32_t)kk;
    if (kk == 0) return -1;          // empty itemset: support n_txn
    if (kk > 8) return -2;           // streaming kernel
    for (uint32_t i = 0; i < 8; ++i) it[i] = 0;
    for (uint32_t i = 0; i < (uint32_t)kk; ++i) {
        const uint32_t x = items[a + i];
        if (x >= d) return -3;       // an id with no row: support 0
        it[i] = (uint16_t)x;
    }
    for (uint32_t i = (uint32_t)kk; i < 8; ++i) it[i] = it[0];
    return (int)(kLaneBins - (uint32_t)kk);
}

// Pass 1: per-bin candidate counts; empty, unknown-id and >8-item candidates
// are settled (or listed for the streaming kernel) here.
__global__ void __launch_bounds__(kLaneTile) lane_hist_kernel(const uint64_t *__restrict__ cand_ptr,
                                                              const uint32_t *__restrict__ items, uint64_t n,
                                                              uint32_t d, uint64_t n_txn, uint32_t *__restrict__ bins,
                                                              uint32_t *__restrict__ ovf_list,
                                                              unsigned long long *__restrict__ ovf_count,
                                                              uint32_t *__restrict__ out) {
    __shared__ uint32_t hist[kLaneBins];
    if (threadIdx.x < kLaneBins) hist[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        uint16_t it[8];
        uint32_t k;
        const int bin = cand_bin(cand_ptr, items, c, d, it, k);
        if (bin >= 0) {
            atomicAdd(&hist[bin], 1u);
        } else if (bin == -1) {
            out[c] = (uint32_t)n_txn;
        } else if (bin == -2) {
            ovf_list[atomicAdd(ovf_count, 1ull)] = (uint32_t)c;
        } else {
            out[c] = 0;
        }
    }
    __syncthreads();
    if (threadIdx.x < kLaneBins && hist[threadIdx.x]) atomicAdd(&bins[threadIdx.x], hist[threadIdx.x]);
}

// Pass 2: scatter records into k-descending order.  Each tile of 256
// candidates reserves its run inside every bin with one atomic per bin.
// bins[0..7] = counts, bins[8..15] = per-bin cursors.
__global__ void __launch_bounds__(kLaneTile) lane_scatter_kernel(const uint64_t *__restrict__ cand_ptr,
                                                                 const uint32_t *__restrict__ items, uint64_t n,
                                                                 uint32_t d, uint32_t *__restrict__ bins,
                                                                 uint4 *__restrict__ recs,
                                                                 uint32_t *__restrict__ perm) {
    __shared__ uint32_t start[kLaneBins], tile_n[kLaneBins], tile_base[kLaneBins];
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (uint32_t b = 0; b < kLaneBins; ++b) {
            start[b] = s;
            s += bins[b];
        }
    }
    const uint64_t stride = (uint64_t)gridDim.x * kLaneTile;
    for (uint64_t t0 = (uint64_t)blockIdx.x * kLaneTile; t0 < n; t0 += stride) {
        if (threadIdx.x < kLaneBins) tile_n[threadIdx.x] = 0;
        __syncthreads();
        const uint64_t c = t0 + threadIdx.x;
        uint16_t it[8];
        uint32_t k = 0, rank = 0;
        int bin = -1;
        if (c < n) {
            bin = cand_bin(cand_ptr, items, c, d, it, k);
            if (bin >= 0) rank = atomicAdd(&tile_n[bin], 1u);
        }
        __syncthreads();
        if (threadIdx.x < kLaneBins && tile_n[threadIdx.x])
            tile_base[threadIdx.x] = atomicAdd(&bins[kLaneBins + threadIdx.x], tile_n[threadIdx.x]);
        __syncthreads();
        if (bin >= 0) {
            const uint32_t pos = start[bin] + tile_base[bin] + rank;
            uint4 r;
            r.x = ((uint32_t)it[0] | (k << 12)) | ((uint32_t)it[1] << 16);
            r.y = (uint32_t)it[2] | ((uint32_t)it[3] << 16);
            r.z = (uint32_t)it[4] | ((uint32_t)it[5] << 16);
            r.w = (uint32_t)it[6] | ((uint32_t)it[7] << 16);
            recs[pos] = r;
            perm[pos] = (uint32_t)c;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ uint4 lds128(const uint8_t *p) { return *reinterpret_cast<const uint4 *>(p); }

// Popcount of the AND of K rows of the staged chunk: o[j] is row j's byte
// offset with the lane's piece rotation folded into bits 4..6.
template <int K>
__device__ __forceinline__ uint32_t lane_popc(const uint8_t *stage, const uint32_t (&o)[8]) {
    uint32_t tot = 0;
    if (K <= 4) {
        // two pieces per iteration: 2K loads in flight per warp, still without spills
#pragma unroll 2
        for (uint32_t i = 0; i < 8; ++i) {
            uint4 m = lds128(stage + (o[0] ^ (i << 4)));
#pragma unroll
            for (int j = 1; j < K; ++j) m = and4(m, lds128(stage + (o[j] ^ (i << 4))));
            tot += popc4(m);
        }
    } else {
        // one piece per iteration: larger K spill at two pieces under 64 registers
#pragma unroll 1
        for (uint32_t i = 0; i < 8; ++i) {
            uint4 m = lds128(stage + (o[0] ^ (i << 4)));
#pragma unroll
            for (int j = 1; j < K; ++j) m = and4(m, lds128(stage + (o[j] ^ (i << 4))));
            tot += popc4(m);
        }
    }
    return tot;
}

__global__ void __launch_bounds__(kLaneThreads, 1)
    k1_lane_kernel(const __grid_constant__ CUtensorMap bm_map, uint32_t n_boxes, uint64_t n_words,
                   const uint4 *__restrict__ recs, const uint32_t *__restrict__ perm, const uint32_t *__restrict__ bins,
                   uint32_t l_cap, uint32_t *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *stage = smem;                                           // n_boxes * 32 KB
    const uint32_t stage_bytes = n_boxes * kLaneBoxBytes;
    uint4 *rec_s = reinterpret_cast<uint4 *>(smem + stage_bytes);    // l_cap * 32 records
    uint32_t *acc_s = reinterpret_cast<uint32_t *>(rec_s + (size_t)l_cap * 32);
    uint64_t *bar = reinterpret_cast<uint64_t *>(acc_s + (size_t)l_cap * 32);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(bar + 1);          // two set counters

    const uint32_t tid = threadIdx.x, lane = tid & 31;
    uint32_t n_valid = 0;
#pragma unroll
    for (uint32_t b = 0; b < kLaneBins; ++b) n_valid += bins[b];
    const uint32_t n_sets = (n_valid + 31) / 32, G = gridDim.x, cta = blockIdx.x;
    if (cta >= n_sets) return;
    uint32_t nl = (n_sets - cta + G - 1) / G;   // sets cta, cta + G, ...
    if (nl > l_cap) nl = l_cap;                  // l_cap is the host's bound on nl

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        ctr[0] = 0;
        ctr[1] = 0;
    }
    for (uint32_t i = tid; i < nl * 32; i += kLaneThreads) {
        const uint32_t pos = (cta + (i >> 5) * G) * 32 + (i & 31);
        rec_s[i] = pos < n_valid ? recs[pos] : make_uint4(1u << 12, 0, 0, 0);   // row 0, k = 1
        acc_s[i] = 0;
    }
    __syncthreads();

    const uint32_t rot = (lane & 7) << 4;
    const uint64_t n_chunks = (n_words + kLaneWords - 1) / kLaneWords;
    uint32_t phase = 0;
    for (uint64_t ch = 0; ch < n_chunks; ++ch) {
        if (tid == 0) {
            mbar_arrive_expect_tx(bar, stage_bytes);
            for (uint32_t b = 0; b < n_boxes; ++b)
                tma_load_2d(stage + (size_t)b * kLaneBoxBytes, &bm_map, (int32_t)(ch * kLaneWords),
                            (int32_t)(b * kLaneRowsPerBox), bar);
        }
        const bool ok = mbar_wait_bounded(bar, phase, err);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            // give in-flight copies one more bounded chance to land before leaving
            mbar_wait_bounded(bar, phase ^ 1, err);
            return;
        }
        uint32_t *my_ctr = ctr + (ch & 1);
        for (;;) {
            uint32_t l = 0;
            if (lane == 0) l = atomicAdd(my_ctr, 1u);
            l = __shfl_sync(0xffffffffu, l, 0);
            if (l >= nl) break;
            const uint4 r = rec_s[l * 32 + lane];
            const uint32_t k = (r.x >> 12) & 15u;
            uint32_t o[8];
            o[0] = ((r.x & 0x0fffu) << 7) | rot;
            o[1] = ((r.x >> 16) << 7) | rot;
            o[2] = ((r.y & 0xffffu) << 7) | rot;
            o[3] = ((r.y >> 16) << 7) | rot;
            o[4] = ((r.z & 0xffffu) << 7) | rot;
            o[5] = ((r.z >> 16) << 7) | rot;
            o[6] = ((r.w & 0xffffu) << 7) | rot;
            o[7] = ((r.w >> 16) << 7) | rot;
            const uint32_t kmax = __reduce_max_sync(0xffffffffu, k);
            uint32_t v;
            switch (kmax) {
                case 1: v = lane_popc<1>(stage, o); break;
                case 2: v = lane_popc<2>(stage, o); break;
                case 3: v = lane_popc<3>(stage, o); break;
                case 4: v = lane_popc<4>(stage, o); break;
                case 5: v = lane_popc<5>(stage, o); break;
                case 6: v = lane_popc<6>(stage, o); break;
                case 7: v = lane_popc<7>(stage, o); break;
                default: v = lane_popc<8>(stage, o); break;
            }
            acc_s[l * 32 + lane] += v;
        }
        __syncthreads();   // every warp is done with this chunk before TMA overwrites it
        if (tid == 0) *my_ctr = 0;   // next used by chunk ch + 2, after the next barrier
    }
    for (uint32_t i = tid; i < nl * 32; i += kLaneThreads) {
        const uint32_t pos = (cta + (i >> 5) * G) * 32 + (i & 31);
        if (pos < n_valid) out[perm[pos]] = acc_s[i];
    }
}

// ---------------------------------------------------------------- TMEM form
// The same lanes, with the candidate records and totals in tensor memory
// instead of shared memory: shared memory then holds a ring of 32-KB box
// slots (seven for d <= 1,024: a chunk's four boxes plus three boxes of the
// next chunk, loaded while the current one is counted), and one CTA per SM
// can own a whole wave's worth of sets.
//
// TMEM layout: warp w reaches lanes 32 * (w % 4) .. +31 (its quadrant).  The
// CTA's sets l = q, q + 4, ... belong to quadrant q; the m-th of them sits in
// columns 5m .. 5m+3 (the 16-byte record of lane j's candidate in TMEM lane
// 32q + j) and 5m + 4 (its running total).  The eight warps of a quadrant
// take its sets from a per-quadrant counter, largest k first.
constexpr uint32_t kTmColsPerSet = 5;

__device__ __forceinline__ void tm_ld_rec(uint32_t taddr, uint4 &r, uint32_t &acc) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%5];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%4}, [%6];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w), "=r"(acc)
        : "r"(taddr), "r"(taddr + 4)
        : "memory");
}
__device__ __forceinline__ uint32_t tm_ld1(uint32_t taddr) {
    uint32_t v;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v)
        : "r"(taddr)
        : "memory");
    return v;
}
__device__ __forceinline__ void tm_st4(uint32_t taddr, uint4 v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w)
                 : "memory");
}
__device__ __forceinline__ void tm_st1(uint32_t taddr, uint32_t v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(v) : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tm_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tm_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__global__ void __launch_bounds__(kLaneThreads, 1)
    k1_lane_tm_kernel(const __grid_constant__ CUtensorMap bm_map, uint32_t n_boxes, uint32_t n_slots,
                      uint64_t n_words, const uint4 *__restrict__ recs, const uint32_t *__restrict__ perm,
                      const uint32_t *__restrict__ bins, uint32_t l_cap, uint32_t tm_cols,
                      uint32_t *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)n_slots * kLaneBoxBytes);  // one per slot
    unsigned long long *issued_s = reinterpret_cast<unsigned long long *>(full + n_slots);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(issued_s + 1);   // [quadrant][chunk parity]
    uint32_t *tslot = ctr + 8;

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, quad = warp & 3;
    uint32_t n_valid = 0;
#pragma unroll
    for (uint32_t b = 0; b < kLaneBins; ++b) n_valid += bins[b];
    const uint32_t n_sets = (n_valid + 31) / 32, G = gridDim.x, cta = blockIdx.x;
    if (cta >= n_sets) return;
    uint32_t nl = (n_sets - cta + G - 1) / G;
    if (nl > l_cap) nl = l_cap;                        // l_cap bounds the TMEM columns
    const uint32_t nq = nl > quad ? (nl - quad + 3) / 4 : 0;   // this quadrant's sets

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(tm_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (uint32_t s = 0; s < n_slots; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        for (int i = 0; i < 8; ++i) ctr[i] = 0;
        *issued_s = 0;
    }
    tm_fence_before();
    __syncthreads();
    tm_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t tq = tbase + ((quad * 32u) << 16);

    for (uint32_t m = warp >> 2; m < nq; m += 8) {
        const uint32_t pos = (cta + (quad + 4 * m) * G) * 32 + lane;
        const uint4 r = pos < n_valid ? recs[pos] : make_uint4(1u << 12, 0, 0, 0);   // row 0, k = 1
        tm_st4(tq + kTmColsPerSet * m, r);
        tm_st1(tq + kTmColsPerSet * m + 4, 0u);
    }
    tm_wait_st();

    const uint32_t rot = (lane & 7) << 4;
    const uint64_t n_chunks = (n_words + kLaneWords - 1) / kLaneWords;
    const uint64_t total = n_chunks * n_boxes;
    bool ok = true;
    for (uint64_t ch = 0; ch < n_chunks; ++ch) {
        if (tid == 0) {
            // slot g % n_slots is free once the chunk of box g - n_slots is done:
            // every chunk before ch is
            uint64_t g = *issued_s;
            const uint64_t lim = min(total, ch * n_boxes + n_slots);
            for (; g < lim; ++g) {
                const uint32_t sl = (uint32_t)(g % n_slots);
                mbar_arrive_expect_tx(&full[sl], kLaneBoxBytes);
                tma_load_2d(smem + (size_t)sl * kLaneBoxBytes, &bm_map, (int32_t)((g / n_boxes) * kLaneWords),
                            (int32_t)((g % n_boxes) * kLaneRowsPerBox), &full[sl]);
            }
            *issued_s = g;
        }
        for (uint32_t b = 0; b < n_boxes && ok; ++b) {
            const uint64_t g = ch * n_boxes + b;
            ok = mbar_wait_bounded(&full[g % n_slots], (uint32_t)((g / n_slots) & 1), err);
        }
        tm_fence_before();
        if (__syncthreads_or(!ok)) {
            ok = false;   // the same for every thread: the paths below hold warp-wide TMEM operations
            break;
        }
        tm_fence_after();
        const uint32_t base_s = (uint32_t)((ch * n_boxes) % n_slots);
        uint32_t *my_ctr = ctr + quad * 2 + (uint32_t)(ch & 1);
        for (;;) {
            uint32_t m = 0;
            if (lane == 0) m = atomicAdd(my_ctr, 1u);
            m = __shfl_sync(0xffffffffu, m, 0);
            if (m >= nq) break;
            uint4 r;
            uint32_t acc;
            tm_ld_rec(tq + kTmColsPerSet * m, r, acc);
            const uint32_t k = (r.x >> 12) & 15u;
            const uint32_t it[8] = {r.x & 0x0fffu, r.x >> 16, r.y & 0xffffu, r.y >> 16,
                                    r.z & 0xffffu, r.z >> 16, r.w & 0xffffu, r.w >> 16};
            uint32_t o[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                uint32_t sl = base_s + (it[j] >> 8);
                if (sl >= n_slots) sl -= n_slots;
                o[j] = (sl << 15) | ((it[j] & 255u) << 7) | rot;
            }
            const uint32_t kmax = __reduce_max_sync(0xffffffffu, k);
            uint32_t v;
            switch (kmax) {
                case 1: v = lane_popc<1>(smem, o); break;
                case 2: v = lane_popc<2>(smem, o); break;
                case 3: v = lane_popc<3>(smem, o); break;
                case 4: v = lane_popc<4>(smem, o); break;
                case 5: v = lane_popc<5>(smem, o); break;
                case 6: v = lane_popc<6>(smem, o); break;
                case 7: v = lane_popc<7>(smem, o); break;
                default: v = lane_popc<8>(smem, o); break;
            }
            tm_st1(tq + kTmColsPerSet * m + 4, acc + v);
        }
        tm_wait_st();
        tm_fence_before();
        __syncthreads();   // every warp is done with this chunk's slots and totals
        tm_fence_after();
        if (tid < 4) ctr[tid * 2 + (uint32_t)(ch & 1)] = 0;   // next used by chunk ch + 2
    }
    if (ok) {
        for (uint32_t m = warp >> 2; m < nq; m += 8) {
            const uint32_t pos = (cta + (quad + 4 * m) * G) * 32 + lane;
            const uint32_t acc = tm_ld1(tq + kTmColsPerSet * m + 4);
            if (pos < n_valid) out[perm[pos]] = acc;
        }
    } else {
        // a wait ran out: let the copies still in flight land (bounded) before
        // the CTA's shared memory goes away
        const uint64_t g1 = *issued_s;
        for (uint64_t g = g1 > n_slots ? g1 - n_slots : 0; g < g1; ++g)
            mbar_wait_bounded(&full[g % n_slots], (uint32_t)((g / n_slots) & 1), err);
    }
    tm_fence_before();
    __syncthreads();
    if (warp == 0) {
        tm_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(tm_cols) : "memory");
    }
}

size_t lane_tm_smem_bytes(uint32_t n_slots) { return (size_t)n_slots * kLaneBoxBytes + (size_t)n_slots * 8 + 64; }

size_t lane_smem_bytes(uint32_t n_boxes, uint32_t l_cap) {
    return (size_t)n_boxes * kLaneBoxBytes + (size_t)l_cap * 32 * (16 + 4) + 16;
}

}  // namespace

int lane_tm_supports_device(const CUtensorMap *map, uint32_t d, uint64_t n_words, const uint64_t *cand_ptr,
                            const uint32_t *cand_items, uint64_t n_cand, uint64_t n_txn, uint32_t *out, void *scratch,
                            size_t scratch_bytes, uint32_t waves, uint32_t *dev_err, cudaStream_t st, int n_sm,
                            uint32_t **ovf_list, unsigned long long **ovf_count, uint64_t *launches,
                            cudaEvent_t *ev) {
    if (!lane_supported(d) || n_cand == 0 || n_cand > 0xffffffffull) return -1;
    if (scratch_bytes < support_scratch_bytes_for(n_cand)) return -1;
    const uint32_t n_boxes = (d + kLaneRowsPerBox - 1) / kLaneRowsPerBox;
    uint32_t n_slots = 0;
    while (lane_tm_smem_bytes(n_slots + 1) <= kMaxSmem) ++n_slots;
    if (n_slots < n_boxes) return -1;
    const uint64_t n_sets = (n_cand + 31) / 32;
    uint64_t grid = 0, l_cap = 0;
    for (uint32_t w = std::max<uint32_t>(1, waves); w <= 64; ++w) {
        grid = std::min<uint64_t>((uint64_t)n_sm * w, n_sets);
        l_cap = (n_sets + grid - 1) / grid;
        if (kTmColsPerSet * ((l_cap + 3) / 4) <= 512) break;
        grid = 0;
    }
    if (grid == 0) return -1;
    uint32_t tm_cols = 32;
    while (tm_cols < kTmColsPerSet * ((l_cap + 3) / 4)) tm_cols *= 2;
    uint8_t *sb = static_cast<uint8_t *>(scratch);
    uint4 *recs = reinterpret_cast<uint4 *>(sb);
    uint32_t *ovf = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16));
    uint32_t *perm = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + align256(n_cand * 4));
    uint32_t *bins = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + 2 * align256(n_cand * 4));
    unsigned long long *ovf_n = reinterpret_cast<unsigned long long *>(
        sb + align256(n_cand * 16) + 2 * align256(n_cand * 4) + align256(kSupportSortBins * 4));
    SG_CUDA_TRY(cudaMemsetAsync(bins, 0, 2 * kLaneBins * 4, st));
    SG_CUDA_TRY(cudaMemsetAsync(ovf_n, 0, 8, st));
    const unsigned prep_blocks = (unsigned)std::min<uint64_t>((n_cand + kLaneTile - 1) / kLaneTile, (uint64_t)n_sm * 8);
    lane_hist_kernel<<<prep_blocks, kLaneTile, 0, st>>>(cand_ptr, cand_items, n_cand, d, n_txn, bins, ovf, ovf_n, out);
    SG_CUDA_TRY(cudaGetLastError());
    lane_scatter_kernel<<<prep_blocks, kLaneTile, 0, st>>>(cand_ptr, cand_items, n_cand, d, bins, recs, perm);
    SG_CUDA_TRY(cudaGetLastError());
    const size_t smem = lane_tm_smem_bytes(n_slots);
    SG_CUDA_TRY(cudaFuncSetAttribute(k1_lane_tm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (ev) SG_CUDA_TRY(cudaEventRecord(ev[1], st));
    k1_lane_tm_kernel<<<(unsigned)grid, kLaneThreads, smem, st>>>(*map, n_boxes, n_slots, n_words, recs, perm, bins,
                                                                  (uint32_t)l_cap, tm_cols, out, dev_err);
    SG_CUDA_TRY(cudaGetLastError());
    if (ev) SG_CUDA_TRY(cudaEventRecord(ev[2], st));
    if (launches) *launches += 3;
    *ovf_list = ovf;
    *ovf_count = ovf_n;
    return 0;
}

bool lane_supported(uint32_t d) { return d > 0 && d <= kLaneMaxD && lane_smem_bytes((d + 255) / 256, 1) <= kMaxSmem; }

int lane_supports_device(const CUtensorMap *map, uint32_t d, uint64_t n_words, const uint64_t *cand_ptr,
                         const uint32_t *cand_items, uint64_t n_cand, uint64_t n_txn, uint32_t *out, void *scratch,
                         size_t scratch_bytes, uint32_t waves, uint32_t *dev_err, cudaStream_t st, int n_sm,
                         uint32_t **ovf_list, unsigned long long **ovf_count, uint64_t *launches,
                         cudaEvent_t *ev) {
    if (!lane_supported(d) || n_cand == 0 || n_cand > 0xffffffffull) return -1;
    if (scratch_bytes < support_scratch_bytes_for(n_cand)) return -1;
    const uint32_t n_boxes = (d + kLaneRowsPerBox - 1) / kLaneRowsPerBox;
    const uint64_t n_sets = (n_cand + 31) / 32;
    uint64_t grid = 0, l_cap = 0;
    for (uint32_t w = std::max<uint32_t>(1, waves); w <= 64; ++w) {
        grid = std::min<uint64_t>((uint64_t)n_sm * w, n_sets);
        l_cap = (n_sets + grid - 1) / grid;
        if (lane_smem_bytes(n_boxes, (uint32_t)l_cap) <= kMaxSmem) break;
        grid = 0;
    }
    if (grid == 0) return -1;
    uint8_t *sb = static_cast<uint8_t *>(scratch);
    uint4 *recs = reinterpret_cast<uint4 *>(sb);
    uint32_t *ovf = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16));
    uint32_t *perm = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + align256(n_cand * 4));
    uint32_t *bins = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + 2 * align256(n_cand * 4));
    unsigned long long *ovf_n = reinterpret_cast<unsigned long long *>(
        sb + align256(n_cand * 16) + 2 * align256(n_cand * 4) + align256(kSupportSortBins * 4));
    SG_CUDA_TRY(cudaMemsetAsync(bins, 0, 2 * kLaneBins * 4, st));
    SG_CUDA_TRY(cudaMemsetAsync(ovf_n, 0, 8, st));
    const unsigned prep_blocks = (unsigned)std::min<uint64_t>((n_cand + kLaneTile - 1) / kLaneTile, (uint64_t)n_sm * 8);
    lane_hist_kernel<<<prep_blocks, kLaneTile, 0, st>>>(cand_ptr, cand_items, n_cand, d, n_txn, bins, ovf, ovf_n, out);
    SG_CUDA_TRY(cudaGetLastError());
    lane_scatter_kernel<<<prep_blocks, kLaneTile, 0, st>>>(cand_ptr, cand_items, n_cand, d, bins, recs, perm);
    SG_CUDA_TRY(cudaGetLastError());
    const size_t smem = lane_smem_bytes(n_boxes, (uint32_t)l_cap);
    SG_CUDA_TRY(cudaFuncSetAttribute(k1_lane_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (ev) SG_CUDA_TRY(cudaEventRecord(ev[1], st));
    k1_lane_kernel<<<(unsigned)grid, kLaneThreads, smem, st>>>(*map, n_boxes, n_words, recs, perm, bins,
                                                               (uint32_t)l_cap, out, dev_err);
    SG_CUDA_TRY(cudaGetLastError());
    if (ev) SG_CUDA_TRY(cudaEventRecord(ev[2], st));
    if (launches) *launches += 3;
    *ovf_list = ovf;
    *ovf_count = ovf_n;
    return 0;
}

}  // namespace sg
