// kernels_cooc.cu -- pairwise co-occurrence C[i][j] = popc(bv_i & bv_j).
//
// Reference counterparts: the b1 AND-POPC GEMMs of
// code/engine_tensorfim/code/microbench/bmma_bench.cu:50-152 (wmma b1 naive and
// smem-tiled) and bitmap_kernel (:159-174, CUDA-core popcount), run with A = B =
// the item bitmaps.  C is symmetric, so only tiles with bi <= bj are computed;
// each such tile is written to both (bi,bj) and (bj,bi).  The transaction
// (k) dimension is split across CTAs so the few upper-triangle tiles still
// fill all SMs; partial tiles are summed with 32-bit atomics into a zeroed C.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sg {

// ---------------------------------------------------------------- CUDA-core
// CTA tile 128 x 128, 256 threads, 8 x 8 outputs per thread.  k chunk = 16
// 32-bit words per row staged in shared memory (padded rows avoid conflicts).
constexpr int kPT = 128;      // tile edge
constexpr int kPK = 16;       // u32 words per k chunk

// Shared tiles are stored k-major ([word][row], rows padded to 129) so that a
// warp's 16 distinct B columns (tx + 16 j) hit 16 distinct banks and the A rows
// (ty + 16 i, two values per warp) are broadcasts.
__global__ void __launch_bounds__(256) cooc_popc_kernel(const uint32_t *__restrict__ bm32, uint64_t stride32,
                                                        uint64_t n32, uint32_t d, uint32_t n_tiles,
                                                        uint64_t k_per_split, uint32_t *__restrict__ out) {
    __shared__ uint32_t As[kPK][kPT + 1];
    __shared__ uint32_t Bs[kPK][kPT + 1];
    // decode upper-triangle tile pair from blockIdx.x
    uint32_t t = blockIdx.x, bi = 0;
    while (t >= n_tiles - bi) { t -= n_tiles - bi; ++bi; }
    const uint32_t bj = bi + t;
    const uint64_t k0 = (uint64_t)blockIdx.y * k_per_split;
    const uint64_t k1 = min(n32, k0 + k_per_split);
    const uint32_t tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    uint32_t acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0;
    for (uint64_t kc = k0; kc < k1; kc += kPK) {
        for (int idx = threadIdx.x; idx < kPT * kPK; idx += 256) {
            const int r = idx / kPK, c = idx % kPK;
            const uint64_t kk = kc + c;
            const uint32_t ra = bi * kPT + r, rb = bj * kPT + r;
            As[c][r] = (ra < d && kk < k1) ? bm32[ra * stride32 + kk] : 0u;
            Bs[c][r] = (rb < d && kk < k1) ? bm32[rb * stride32 + kk] : 0u;
        }
        __syncthreads();
#pragma unroll 4
        for (int c = 0; c < kPK; ++c) {
            uint32_t a[8], b[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] = As[c][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 8; ++j) b[j] = Bs[c][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] += __popc(a[i] & b[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t r = bi * kPT + ty + 16 * i;
        if (r >= d) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t c = bj * kPT + tx + 16 * j;
            if (c >= d || acc[i][j] == 0) continue;
            atomicAdd(&out[(uint64_t)r * d + c], acc[i][j]);
            if (bi != bj) atomicAdd(&out[(uint64_t)c * d + r], acc[i][j]);
        }
    }
}

// ---------------------------------------------------------------- b1 mma.sync
// mma.sync.m16n8k256 .b1 AND.POPC: CTA tile 128 x 128 (8 warps, each 64 x 32
// = 4 x 4 mma tiles), k chunk = 512 bits (16 u32) per row in shared memory.
// Fragment layout (PTX ISA, m16n8k256 .b1): A a0/a2 row = group, a1/a3 row =
// group + 8; a0/a1 hold k bits [32*tig, +32), a2/a3 bits [128 + 32*tig, +32).
// B b0 holds k bits [32*tig, +32) and b1 [128 + 32*tig, +32) of column group.
// C c0/c1 row group, cols 2*tig + {0,1}; c2/c3 row group + 8.
constexpr int kBK = 16;     // u32 per row per chunk (512 bits)
constexpr int kBKpad = 20;  // padded row (80 B) -> rows 0..7 land on distinct bank quads

__device__ __forceinline__ void mma_b1(uint32_t (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(256) cooc_bmma_kernel(const uint32_t *__restrict__ bm32, uint64_t stride32,
                                                        uint64_t n32, uint32_t d, uint32_t n_tiles,
                                                        uint64_t k_per_split, uint32_t *__restrict__ out) {
    __shared__ uint32_t As[kPT][kBKpad];
    __shared__ uint32_t Bs[kPT][kBKpad];
    uint32_t t = blockIdx.x, bi = 0;
    while (t >= n_tiles - bi) { t -= n_tiles - bi; ++bi; }
    const uint32_t bj = bi + t;
    const uint64_t k0 = (uint64_t)blockIdx.y * k_per_split;
    const uint64_t k1 = min(n32, k0 + k_per_split);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t grp = lane >> 2, tig = lane & 3;
    const uint32_t wm = (warp >> 2) * 64;  // warp row offset in tile (0 / 64)
    const uint32_t wn = (warp & 3) * 32;   // warp col offset (0..96)
    uint32_t acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0;
    for (uint64_t kc = k0; kc < k1; kc += kBK) {
        for (int idx = threadIdx.x; idx < kPT * kBK / 4; idx += 256) {
            const int r = idx / (kBK / 4), c4 = (idx % (kBK / 4)) * 4;
            const uint64_t kk = kc + c4;
            const uint32_t ra = bi * kPT + r, rb = bj * kPT + r;
            uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
            if (kk + 3 < k1) {
                if (ra < d) va = *reinterpret_cast<const uint4 *>(bm32 + ra * stride32 + kk);
                if (rb < d) vb = *reinterpret_cast<const uint4 *>(bm32 + rb * stride32 + kk);
            } else {
                uint32_t ta[4] = {0, 0, 0, 0}, tb[4] = {0, 0, 0, 0};
                for (int q = 0; q < 4; ++q) {
                    if (kk + q < k1) {
                        if (ra < d) ta[q] = bm32[ra * stride32 + kk + q];
                        if (rb < d) tb[q] = bm32[rb * stride32 + kk + q];
                    }
                }
                va = make_uint4(ta[0], ta[1], ta[2], ta[3]);
                vb = make_uint4(tb[0], tb[1], tb[2], tb[3]);
            }
            As[r][c4 + 0] = va.x; As[r][c4 + 1] = va.y; As[r][c4 + 2] = va.z; As[r][c4 + 3] = va.w;
            Bs[r][c4 + 0] = vb.x; Bs[r][c4 + 1] = vb.y; Bs[r][c4 + 2] = vb.z; Bs[r][c4 + 3] = vb.w;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kBK / 8; ++ks) {  // two 256-bit k steps per chunk
            uint32_t af[4][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t r0 = wm + i * 16 + grp;
                af[i][0] = As[r0][ks * 8 + tig];
                af[i][1] = As[r0 + 8][ks * 8 + tig];
                af[i][2] = As[r0][ks * 8 + 4 + tig];
                af[i][3] = As[r0 + 8][ks * 8 + 4 + tig];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t c0 = wn + j * 8 + grp;
                bf[j][0] = Bs[c0][ks * 8 + tig];
                bf[j][1] = Bs[c0][ks * 8 + 4 + tig];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_b1(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const uint32_t row = bi * kPT + wm + i * 16 + grp + (r >= 2 ? 8 : 0);
                const uint32_t col = bj * kPT + wn + j * 8 + tig * 2 + (r & 1);
                const uint32_t v = acc[i][j][r];
                if (row < d && col < d && v) {
                    atomicAdd(&out[(uint64_t)row * d + col], v);
                    if (bi != bj) atomicAdd(&out[(uint64_t)col * d + row], v);
                }
            }
}

size_t cooc_scratch_bytes(uint32_t d, uint64_t n_words, int kind) {
    (void)d; (void)n_words; (void)kind;
    return 0;
}

int cooc_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride, uint32_t *out, int kind,
                cudaStream_t st, int n_sm, void *scratch, size_t scratch_bytes, uint64_t *launches, uint32_t *dev_err) {
    (void)scratch; (void)scratch_bytes;
    if (d == 0) return 0;
    if (kind == 3) return cooc_tc_device(bitmaps, d, n_words, row_stride, out, st, n_sm, dev_err, launches);
    if (kind == 4) return cooc_tc256_device(bitmaps, d, n_words, row_stride, out, st, n_sm, dev_err, launches);
    SG_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)d * d * 4, st));
    const uint32_t n_tiles = (d + kPT - 1) / kPT;
    const uint32_t pairs = n_tiles * (n_tiles + 1) / 2;
    const uint64_t n32 = n_words * 2, stride32 = row_stride * 2;
    // split k so that the grid covers ~4 CTAs per SM
    const uint64_t target = (uint64_t)n_sm * 4;
    uint64_t splits = std::max<uint64_t>(1, (target + pairs - 1) / pairs);
    const uint64_t chunk = (kind == 2) ? kBK : kPK;
    uint64_t kps = (n32 + splits - 1) / splits;
    kps = (kps + chunk - 1) / chunk * chunk;
    splits = (n32 + kps - 1) / kps;
    dim3 grid(pairs, (unsigned)splits);
    const uint32_t *bm32 = reinterpret_cast<const uint32_t *>(bitmaps);
    if (kind == 2) {
        cooc_bmma_kernel<<<grid, 256, 0, st>>>(bm32, stride32, n32, d, n_tiles, kps, out);
    } else {
        cooc_popc_kernel<<<grid, 256, 0, st>>>(bm32, stride32, n32, d, n_tiles, kps, out);
    }
    SG_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 1;
    return 0;
}

}  // namespace sg
