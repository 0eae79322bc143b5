// kernels_tc.cu -- co-occurrence on the 5th-generation tensor cores (tcgen05).
//
// C[i][j] = popc(bv_i & bv_j) is the dot product of two 0/1 vectors.  Bits
// are expanded to fp8 e4m3 bytes (1.0 = 0x38, 0.0 = 0x00; both exact) inside
// the kernel and multiplied with tcgen05.mma .kind::f8f6f4, accumulating in
// fp32 in tensor memory: every partial sum is an integer below 2^24 (a CTA
// covers at most 2^20 transactions per split), so fp32 holds it exactly.
// The reference does this product with b1 AND-POPC wmma fragments
// (code/engine_tensorfim/code/microbench/bmma_bench.cu:99-152); GB300 has no
// b1 tcgen05 kind and its int8 tensor rate is cut, hence e4m3.
//
// Tiling: a CTA owns one upper-triangle 128 x 128 tile (rows bi, columns bj)
// and a slice of the transactions.  Per stage, 256 threads expand a 256-bit
// slice of 128 + 128 rows into two 128B-swizzled K-major atoms per operand
// (row r, byte b at r*128 + ((b/16) ^ (r%8))*16 + b%16), fence the async
// proxy, and one thread issues 8 MMAs of K=32; tcgen05.commit arrives on the
// stage's mbarrier when the tensor core is done reading it.  The epilogue
// reads the 128 x 128 fp32 accumulator from TMEM (tcgen05.ld 32x32b) and
// adds the integer counts into C (and its mirror) with atomics.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcStages = 2;
constexpr int kTcAtom = 128 * 128;             // one 128-row x 128-byte swizzle atom
constexpr int kTcOperand = 2 * kTcAtom;        // two atoms along K per operand
constexpr int kTcStageBytes = 2 * kTcOperand;  // A and B
constexpr uint32_t kTcCols = 128;              // TMEM columns (fp32 accumulators)

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    // sm_100 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading
    // byte offset >> 4 (16-29, unused for swizzled K-major: 1), stride byte
    // offset >> 4 (32-45: 1024 B between 8-row groups), version 1 (46-47),
    // base offset 0 (49-51), layout SWIZZLE_128B = 2 (61-63).
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3fff);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor, kind::f8f6f4: D = f32 (bits 4-5 = 1), A = B = e4m3
// (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kTcIdesc = (1u << 4) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 4 bits -> 4 bytes of e4m3 (0x38 = 1.0 where the bit is set).
__device__ __forceinline__ uint32_t nib4(uint32_t n) { return ((n * 0x00204081u) & 0x01010101u) * 0x38u; }

// Expand 128 bits (two u64) into one 128-byte swizzled row of an atom.
__device__ __forceinline__ void expand_row(uint8_t *atom, uint32_t r, uint64_t lo, uint64_t hi) {
    uint8_t *row = atom + r * 128;
    const uint32_t x = r & 7;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint64_t w = c < 4 ? lo : hi;
        const uint32_t bits = (uint32_t)(w >> ((c & 3) * 16)) & 0xffffu;
        const uint4 v = make_uint4(nib4(bits & 15), nib4((bits >> 4) & 15), nib4((bits >> 8) & 15), nib4(bits >> 12));
        *reinterpret_cast<uint4 *>(row + ((c ^ x) << 4)) = v;
    }
}

// Bit slices arrive by TMA (box 4 words x 128 rows per operand) into a ring of
// kTcRing slots issued kTcRing steps ahead; expansion reads them from shared
// memory, and the two fp8 stages alternate so that expanding step i+1
// overlaps the tensor core's MMAs on step i.
constexpr int kTcRing = 6;
constexpr int kTcBitTile = 128 * 32;       // one operand's bit slice: 128 rows x 4 words
constexpr int kTcBitSlot = 2 * kTcBitTile;

__global__ void __launch_bounds__(kTcThreads, 1)
    cooc_tc_kernel(const __grid_constant__ CUtensorMap bm_map, uint64_t n_words, uint32_t d, uint32_t n_tiles,
                   uint64_t words_per_split, uint32_t *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mma_bar[kTcStages];
    __shared__ uint64_t bit_bar[kTcRing];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    uint32_t t = blockIdx.x, bi = 0;
    while (t >= n_tiles - bi) { t -= n_tiles - bi; ++bi; }
    const uint32_t bj = bi + t;
    const uint64_t w_begin = (uint64_t)blockIdx.y * words_per_split;
    const uint64_t w_end = min(n_words, w_begin + words_per_split);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem) + 1023) & ~uintptr_t(1023));
    uint8_t *ring = base + (size_t)kTcStages * kTcStageBytes;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) mbar_init(&mma_bar[s], 1);
        for (int s = 0; s < kTcRing; ++s) mbar_init(&bit_bar[s], 1);
        mbar_init(&done_bar, 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    const uint64_t n_steps = w_begin < w_end ? (w_end - w_begin + 3) / 4 : 0;  // 4 words = 256 bits per step
    auto issue = [&](uint64_t step) {
        const uint32_t slot = (uint32_t)(step % kTcRing);
        uint8_t *dst = ring + (size_t)slot * kTcBitSlot;
        mbar_arrive_expect_tx(&bit_bar[slot], kTcBitSlot);
        const int32_t x = (int32_t)(w_begin + step * 4);
        tma_load_2d(dst, &bm_map, x, (int32_t)(bi * 128), &bit_bar[slot]);
        tma_load_2d(dst + kTcBitTile, &bm_map, x, (int32_t)(bj * 128), &bit_bar[slot]);
    };
    if (tid == 0)
        for (uint64_t sidx = 0; sidx < n_steps && sidx < (uint64_t)kTcRing; ++sidx) issue(sidx);
    bool ok = true;
    for (uint64_t it = 0; it < n_steps; ++it) {
        const uint32_t slot = (uint32_t)(it % kTcRing);
        const uint32_t s = (uint32_t)(it % kTcStages);
        uint8_t *stage = base + (size_t)s * kTcStageBytes;
        ok = mbar_wait_bounded(&bit_bar[slot], (uint32_t)((it / kTcRing) & 1), err);
        if (ok && it >= kTcStages)
            ok = mbar_wait_bounded(&mma_bar[s], (uint32_t)((it / kTcStages - 1) & 1), err);
        if (__syncthreads_or(!ok)) break;
        {
            // thread -> one row of A (tid < 128) or B (tid >= 128): 4 words from the ring
            const uint32_t r = tid & 127;
            const uint8_t *src = ring + (size_t)slot * kTcBitSlot + (tid < 128 ? 0 : kTcBitTile) + r * 32;
            const uint4 x0 = *reinterpret_cast<const uint4 *>(src);
            const uint4 x1 = *reinterpret_cast<const uint4 *>(src + 16);
            uint8_t *op = stage + (tid < 128 ? 0 : kTcOperand);
            expand_row(op, r, (uint64_t)x0.x | ((uint64_t)x0.y << 32), (uint64_t)x0.z | ((uint64_t)x0.w << 32));
            expand_row(op + kTcAtom, r, (uint64_t)x1.x | ((uint64_t)x1.y << 32),
                       (uint64_t)x1.z | ((uint64_t)x1.w << 32));
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_addr(stage), b0 = smem_addr(stage + kTcOperand);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint32_t off = (uint32_t)(k >> 2) * kTcAtom + (uint32_t)(k & 3) * 32;
                tc_mma(tmem, smem_desc_sw128(a0 + off), smem_desc_sw128(b0 + off), (it > 0 || k > 0) ? 1u : 0u);
            }
            tc_commit(&mma_bar[s]);
            // every thread has read this ring slot: refill it kTcRing steps ahead
            if (it + kTcRing < n_steps) issue(it + kTcRing);
        }
    }
    // wait for every MMA before reading the accumulator
    if (tid == 0 && n_steps > 0) tc_commit(&done_bar);
    __syncthreads();
    if (ok && n_steps > 0) ok = mbar_wait_bounded(&done_bar, 0, err);
    tc_fence_after();
    if (__syncthreads_or(!ok) == 0 && n_steps > 0 && warp < 4) {
        const uint32_t lane_base = warp * 32;
        const uint32_t row = bi * 128 + lane_base + (tid & 31);
#pragma unroll 1
        for (uint32_t cb = 0; cb < kTcCols; cb += 32) {
            uint32_t v[32];
            const uint32_t taddr = tmem + (lane_base << 16) + cb;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < d) {
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const uint32_t col = bj * 128 + cb + q;
                    const uint32_t cnt = (uint32_t)__uint_as_float(v[q]);
                    if (col < d && cnt) {
                        atomicAdd(&out[(uint64_t)row * d + col], cnt);
                        if (bi != bj) atomicAdd(&out[(uint64_t)col * d + row], cnt);
                    }
                }
            }
        }
    }
    if (!ok) {
        // let copies still in flight land before the CTA's shared memory goes away
        for (int sidx = 0; sidx < kTcRing; ++sidx) mbar_wait_bounded(&bit_bar[sidx], 0, err);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
    }
}

// ---------------------------------------------------------------- 256 x 256 blocks
// The same product with a CTA per upper-triangle 256 x 256 block.  Per step
// (128 transactions) the bit slices of the block's 256 A rows and 256 B rows
// are expanded into one 128B-swizzled K-major atom per operand (B's atom is
// 256 rows tall), and per K = 32 substep two MMAs M = 128 (the two halves of
// A) x N = 256 accumulate into two 256-column fp32 accumulators (all 512 TMEM
// columns).  Each expanded slice feeds twice the MMA work of the 128 x 128
// form, and a diagonal block expands its rows once and uses them as A and B.
//
// Warp roles, coordinated by mbarriers only (no CTA-wide barrier per step):
//   warps 0..15  expansion: a row of A (warps 0..7) or of B (8..15) per thread
//                (half a row of the shared operand on the diagonal); wait ring_full and
//                stage_empty, expand, fence the async proxy, arrive on
//                ring_empty and stage_full (one arrival per warp);
//   warp 16      one thread issues the MMAs of a step once stage_full completes
//                and commits them to stage_empty;
//   warp 17      one thread keeps the TMA ring of bit slices (2 words x 256
//                rows per operand, 16-byte rows read row-wise) kT2Ring steps ahead.
// Three 64-KB stages let the expansion run two steps ahead of the tensor core.
constexpr int kT2Rows = 256;
constexpr int kT2ExpWarps = 16;
constexpr int kT2Threads = 32 * (kT2ExpWarps + 2);
constexpr int kT2Cols = 512;                        // two 128 x 256 fp32 accumulators
constexpr int kT2AtomA = 256 * 128;                 // A: 256 rows x 128 B (two M halves)
constexpr int kT2AtomB = 256 * 128;                 // B: 256 rows x 128 B
constexpr int kT2StageBytes = kT2AtomA + kT2AtomB;  // 64 KB
constexpr int kT2Stages = 3;
constexpr int kT2Ring = 3;
constexpr int kT2BitBox = 256 * 16;                 // one operand's slice: 256 rows x 2 words
constexpr int kT2BitSlot = 2 * kT2BitBox;
constexpr uint32_t kT2Idesc = (1u << 4) | ((256u >> 3) << 17) | ((128u >> 4) << 24);   // D f32, e4m3, N=256, M=128

__device__ __forceinline__ void tc_mma_n256(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kT2Idesc), "r"(acc)
        : "memory");
}

// Expand 64 bits (chunks 4*half .. 4*half+3 of a 128-byte swizzled row).
__device__ __forceinline__ void expand_half(uint8_t *atom, uint32_t r, uint32_t half, uint64_t w) {
    uint8_t *row = atom + r * 128;
    const uint32_t x = r & 7;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const uint32_t bits = (uint32_t)(w >> (c * 16)) & 0xffffu;
        const uint4 v = make_uint4(nib4(bits & 15), nib4((bits >> 4) & 15), nib4((bits >> 8) & 15), nib4(bits >> 12));
        *reinterpret_cast<uint4 *>(row + (((half * 4 + c) ^ x) << 4)) = v;
    }
}

__global__ void __launch_bounds__(kT2Threads, 1)
    cooc_tc256_kernel(const __grid_constant__ CUtensorMap bm_map, uint64_t n_words, uint32_t d, uint32_t n_blocks,
                      uint64_t words_per_split, uint32_t *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t ring_full[kT2Ring], ring_empty[kT2Ring], stage_full[kT2Stages], stage_empty[kT2Stages];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile uint32_t failed;              // a role gave up on a wait: the others stop
    __shared__ unsigned long long issued_n;           // ring steps issued (producer)
    uint32_t t = blockIdx.x, bi = 0;
    while (t >= n_blocks - bi) { t -= n_blocks - bi; ++bi; }
    const uint32_t bj = bi + t;
    const bool diag = bi == bj;
    const uint64_t w_begin = (uint64_t)blockIdx.y * words_per_split;
    const uint64_t w_end = min(n_words, w_begin + words_per_split);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem) + 1023) & ~uintptr_t(1023));
    uint8_t *ring = base + (size_t)kT2Stages * kT2StageBytes;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kT2Cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kT2Ring; ++s) {
            mbar_init(&ring_full[s], 1);
            mbar_init(&ring_empty[s], kT2ExpWarps);
        }
        for (int s = 0; s < kT2Stages; ++s) {
            mbar_init(&stage_full[s], kT2ExpWarps);
            mbar_init(&stage_empty[s], 1);
        }
        mbar_init(&done_bar, 1);
        fence_mbar_init();
        failed = 0;
        issued_n = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t n_steps = w_begin < w_end ? (w_end - w_begin + 1) / 2 : 0;   // 2 words = 128 bits per step

    if (warp < kT2ExpWarps) {
        // ---- expansion
        // warps 0..7: row tid of A; warps 8..15: row tid - 256 of B (on the diagonal,
        // half tid >> 8 of row tid & 255 of the shared operand)
        const uint32_t r = tid & 255, sel = tid >> 8;
        for (uint64_t it = 0; it < n_steps; ++it) {
            if (__any_sync(0xffffffffu, failed != 0)) break;   // the same decision for the whole warp
            const uint32_t slot = (uint32_t)(it % kT2Ring), s = (uint32_t)(it % kT2Stages);
            uint8_t *stage = base + (size_t)s * kT2StageBytes;
            bool ok = mbar_wait_bounded(&ring_full[slot], (uint32_t)((it / kT2Ring) & 1), err);
            uint4 a = make_uint4(0, 0, 0, 0);
            if (ok) {
                const uint8_t *src = ring + (size_t)slot * kT2BitSlot + r * 16;
                if (!diag) {
                    a = *reinterpret_cast<const uint4 *>(src + sel * kT2BitBox);
                } else {
                    const uint2 hw = *reinterpret_cast<const uint2 *>(src + sel * 8);
                    a.x = hw.x;
                    a.y = hw.y;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&ring_empty[slot]);   // the slot's bits are in registers
            if (ok && it >= kT2Stages)
                ok = mbar_wait_bounded(&stage_empty[s], (uint32_t)((it / kT2Stages - 1) & 1), err);
            if (!__all_sync(0xffffffffu, ok)) {
                failed = 1;
                break;
            }
            if (!diag)
                expand_row(stage + sel * kT2AtomA, r, (uint64_t)a.x | ((uint64_t)a.y << 32),
                           (uint64_t)a.z | ((uint64_t)a.w << 32));
            else
                expand_half(stage, r, sel, (uint64_t)a.x | ((uint64_t)a.y << 32));
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&stage_full[s]);
        }
    } else if (warp == kT2ExpWarps) {
        // ---- MMA issue (one thread)
        if (lane == 0) {
            for (uint64_t it = 0; it < n_steps && !failed; ++it) {
                const uint32_t s = (uint32_t)(it % kT2Stages);
                if (!mbar_wait_bounded(&stage_full[s], (uint32_t)((it / kT2Stages) & 1), err)) {
                    failed = 1;
                    break;
                }
                tc_fence_after();
                uint8_t *stage = base + (size_t)s * kT2StageBytes;
                const uint32_t a0 = smem_addr(stage), b0 = diag ? a0 : smem_addr(stage + kT2AtomA);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        tc_mma_n256(tmem + (uint32_t)h * 256u,
                                    smem_desc_sw128(a0 + (uint32_t)h * 128u * 128u + k * 32),
                                    smem_desc_sw128(b0 + k * 32), (it > 0 || k > 0) ? 1u : 0u);
                }
                tc_commit(&stage_empty[s]);
            }
            // every MMA issued so far, also after a failed wait (they still read the stages)
            if (n_steps > 0) tc_commit(&done_bar);
        }
    } else {
        // ---- TMA producer (one thread)
        if (lane == 0) {
            const uint32_t slot_bytes = diag ? kT2BitBox : kT2BitSlot;
            for (uint64_t it = 0; it < n_steps && !failed; ++it) {
                const uint32_t slot = (uint32_t)(it % kT2Ring);
                if (it >= kT2Ring &&
                    !mbar_wait_bounded(&ring_empty[slot], (uint32_t)((it / kT2Ring - 1) & 1), err)) {
                    failed = 1;
                    break;
                }
                uint8_t *dst = ring + (size_t)slot * kT2BitSlot;
                mbar_arrive_expect_tx(&ring_full[slot], slot_bytes);
                const int32_t x = (int32_t)(w_begin + it * 2);
                tma_load_2d(dst, &bm_map, x, (int32_t)(bi * kT2Rows), &ring_full[slot]);
                if (!diag) tma_load_2d(dst + kT2BitBox, &bm_map, x, (int32_t)(bj * kT2Rows), &ring_full[slot]);
                issued_n = it + 1;
            }
        }
    }
    __syncthreads();
    bool ok = !failed;
    if (n_steps > 0 && !mbar_wait_bounded(&done_bar, 0, err)) ok = false;
    tc_fence_after();
    if (__syncthreads_or(!ok) == 0 && n_steps > 0 && warp < kT2ExpWarps) {
        // warp w reads the 32 TMEM lanes of quadrant w % 4 in accumulator (w / 4) % 2,
        // columns 128 * (w / 8) .. +127
        const uint32_t q = warp & 3, h = (warp >> 2) & 1, c0 = (warp >> 3) * 128;
        const uint32_t row = bi * kT2Rows + h * 128 + q * 32 + lane;
#pragma unroll 1
        for (uint32_t cb = c0; cb < c0 + 128; cb += 32) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((q * 32) << 16) + h * 256 + cb;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < d) {
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const uint32_t col = bj * kT2Rows + cb + c;
                    const uint32_t cnt = (uint32_t)__uint_as_float(v[c]);
                    if (col < d && cnt) {
                        atomicAdd(&out[(uint64_t)row * d + col], cnt);
                        if (!diag) atomicAdd(&out[(uint64_t)col * d + row], cnt);
                    }
                }
            }
        }
    }
    if (!ok) {
        // let the copies still in flight land before the CTA's shared memory goes
        // away: the last issued step of every ring slot, with its own phase
        const uint64_t g1 = issued_n;
        for (uint64_t g = g1 > (uint64_t)kT2Ring ? g1 - kT2Ring : 0; g < g1; ++g)
            mbar_wait_bounded(&ring_full[g % kT2Ring], (uint32_t)((g / kT2Ring) & 1), err);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kT2Cols) : "memory");
    }
}

bool encode_bits_map_box(CUtensorMap *map, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                         uint64_t row_stride, uint32_t box_words, uint32_t box_rows);

bool encode_bits_map(CUtensorMap *map, const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride) {
    return encode_bits_map_box(map, bitmaps, d, n_words, row_stride, 4, 128);
}

bool encode_bits_map_box(CUtensorMap *map, const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                         uint64_t row_stride, uint32_t box_words, uint32_t box_rows) {
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return false;
        fn = reinterpret_cast<EncodeFn>(p);
    }
    cuuint64_t dims[2] = {(cuuint64_t)n_words, (cuuint64_t)d};
    cuuint64_t strides[1] = {(cuuint64_t)row_stride * 8};
    cuuint32_t box[2] = {box_words, box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<uint64_t *>(bitmaps), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t tc_smem_bytes() { return (size_t)kTcStages * kTcStageBytes + (size_t)kTcRing * kTcBitSlot + 1024; }
size_t tc256_smem_bytes() { return (size_t)kT2Stages * kT2StageBytes + (size_t)kT2Ring * kT2BitSlot + 1024; }

int cooc_tc256_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out,
                      cudaStream_t st, int n_sm, uint32_t *dev_err, uint64_t *launches) {
    if (d == 0) return 0;
    if ((reinterpret_cast<uintptr_t>(bitmaps) & 15) || (row_stride & 1)) return -1;
    SG_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)d * d * 4, st));
    const uint32_t n_blocks = (d + kT2Rows - 1) / kT2Rows;
    const uint32_t pairs = n_blocks * (n_blocks + 1) / 2;
    // one wave: split the transactions so that pairs x splits <= SMs; each split
    // covers at most 2^20 transactions (fp32 exactness of the partial counts);
    // splits start on an even word (TMA boxes of two words)
    uint64_t splits = std::max<uint64_t>(1, (uint64_t)n_sm / pairs);
    uint64_t wps = (n_words + splits - 1) / splits;
    wps = std::min<uint64_t>(wps, (1ull << 20) / 64);
    wps = (wps + 1) / 2 * 2;
    splits = (n_words + wps - 1) / wps;
    CUtensorMap map;
    if (!encode_bits_map_box(&map, bitmaps, d, n_words, row_stride, 2, kT2Rows)) return -1;
    const size_t smem = tc256_smem_bytes();
    SG_CUDA_TRY(cudaFuncSetAttribute(cooc_tc256_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(pairs, (unsigned)splits);
    cooc_tc256_kernel<<<grid, kT2Threads, smem, st>>>(map, n_words, d, n_blocks, wps, out, dev_err);
    SG_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 1;
    return 0;
}

int cooc_tc_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out,
                   cudaStream_t st, int n_sm, uint32_t *dev_err, uint64_t *launches) {
    if (d == 0) return 0;
    if ((reinterpret_cast<uintptr_t>(bitmaps) & 15) || (row_stride & 1)) return -1;
    SG_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)d * d * 4, st));
    const uint32_t n_tiles = (d + 127) / 128;
    const uint32_t pairs = n_tiles * (n_tiles + 1) / 2;
    // one wave: split the transactions so that pairs x splits <= SMs; each split
    // covers at most 2^20 transactions (fp32 exactness of the partial counts)
    uint64_t splits = std::max<uint64_t>(1, (uint64_t)n_sm / pairs);
    uint64_t wps = (n_words + splits - 1) / splits;
    wps = std::min<uint64_t>(wps, (1ull << 20) / 64);
    wps = (wps + 3) / 4 * 4;
    splits = (n_words + wps - 1) / wps;
    CUtensorMap map;
    if (!encode_bits_map(&map, bitmaps, d, n_words, row_stride)) return -1;
    const size_t smem = tc_smem_bytes();
    SG_CUDA_TRY(cudaFuncSetAttribute(cooc_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(pairs, (unsigned)splits);
    cooc_tc_kernel<<<grid, kTcThreads, smem, st>>>(map, n_words, d, n_tiles, wps, out, dev_err);
    SG_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 1;
    return 0;
}

}  // namespace sg
