// kernels_bitmap.cu -- bitmap build and AND-popcount support counting.
//
// Reference counterparts (paths relative to the reference project root):
//   transpose_kernel   buildBitmap, code/engine_tensorfim/code/engine/src/kernel_bitmap.cu:342-380
//                      (host scatter there; one CTA per transaction tile here)
//   query_kernel       getResFrequencyCudaKernel, kernel_bitmap.cu:412-442 (one launch per
//                      DFS node there; thousands of queries per launch here)
//   k1_staged_kernel   the wave engine's maskBuild + BMMA counting, kernel_bmma.cu:603-768,
//                      restated for arbitrary k-item candidates with the bitmap chunk staged
//                      once per CTA in shared memory by TMA
#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace sg {

// ---------------------------------------------------------------- transpose
// CSR transactions -> vertical bitmaps.  A CTA owns a tile of TW*64
// transactions and builds the d x TW-word tile in shared memory with 32-bit
// shared atomics, then writes each row's TW words (one 8*TW-byte run) and
// adds the tile's popcounts to the singleton counts.
__global__ void transpose_kernel(const uint64_t *__restrict__ row_ptr, const uint32_t *__restrict__ items,
                                 uint64_t n_txn, const int32_t *__restrict__ remap, uint32_t n_ids, uint32_t d,
                                 uint64_t *__restrict__ bm, uint64_t stride, uint32_t *__restrict__ counts,
                                 uint32_t tw) {
    extern __shared__ uint32_t tile[];  // d * 2*tw
    const uint32_t tw32 = 2 * tw;
    const uint64_t t0 = (uint64_t)blockIdx.x * tw * 64;
    const uint64_t t1 = min(n_txn, t0 + (uint64_t)tw * 64);
    for (uint32_t i = threadIdx.x; i < d * tw32; i += blockDim.x) tile[i] = 0;
    __syncthreads();
    for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const uint32_t local = (uint32_t)(t - t0);
        for (uint64_t j = row_ptr[t]; j < row_ptr[t + 1]; ++j) {
            const uint32_t id = items[j];
            int32_t e = -1;
            if (remap) {
                if (id < n_ids) e = remap[id];
            } else if (id < d) {
                e = (int32_t)id;
            }
            if (e >= 0) atomicOr(&tile[(uint32_t)e * tw32 + (local >> 5)], 1u << (local & 31));
        }
    }
    __syncthreads();
    const uint64_t w0 = t0 / 64;
    for (uint32_t i = threadIdx.x; i < d * tw; i += blockDim.x) {
        const uint32_t e = i / tw, wl = i - e * tw;
        const uint64_t gw = w0 + wl;
        if (gw < stride) {
            const uint64_t v = (uint64_t)tile[e * tw32 + 2 * wl] | ((uint64_t)tile[e * tw32 + 2 * wl + 1] << 32);
            bm[(uint64_t)e * stride + gw] = v;
        }
    }
    if (counts) {
        for (uint32_t e = threadIdx.x; e < d; e += blockDim.x) {
            uint32_t s = 0;
            for (uint32_t k = 0; k < tw32; ++k) s += __popc(tile[e * tw32 + k]);
            if (s) atomicAdd(&counts[e], s);
        }
    }
}

// Fallback for very wide item spaces: global 64-bit atomics, one thread per transaction.
__global__ void transpose_global_kernel(const uint64_t *__restrict__ row_ptr, const uint32_t *__restrict__ items,
                                        uint64_t n_txn, const int32_t *__restrict__ remap, uint32_t n_ids,
                                        uint32_t d, unsigned long long *__restrict__ bm, uint64_t stride) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n_txn;
         t += (uint64_t)gridDim.x * blockDim.x) {
        for (uint64_t j = row_ptr[t]; j < row_ptr[t + 1]; ++j) {
            const uint32_t id = items[j];
            int32_t e = -1;
            if (remap) {
                if (id < n_ids) e = remap[id];
            } else if (id < d) {
                e = (int32_t)id;
            }
            if (e >= 0) atomicOr(&bm[(uint64_t)e * stride + (t >> 6)], 1ull << (t & 63));
        }
    }
}

__global__ void row_popc_kernel(const uint64_t *__restrict__ rows, uint64_t stride, uint64_t n_words, uint32_t d,
                                uint32_t *__restrict__ counts) {
    const uint32_t e = blockIdx.x;
    if (e >= d) return;
    uint32_t s = 0;
    for (uint64_t w = threadIdx.x; w < n_words; w += blockDim.x) s += popc64(rows[e * stride + w]);
    s = warp_sum(s);
    __shared__ uint32_t part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0;
        v = warp_sum(v);
        if (threadIdx.x == 0) counts[e] = v;
    }
}

void launch_transpose(const uint64_t *row_ptr, const uint32_t *items, uint64_t n_txn, const int32_t *remap,
                      uint32_t d, uint64_t *bitmaps, uint64_t stride, uint32_t *counts, cudaStream_t st,
                      int n_sm) {
    (void)n_sm;
    if (n_txn == 0 || d == 0) return;
    // n_ids of the remap table is passed through `counts` sizing by the caller; the
    // remap array covers every id that occurs (the caller builds it from the max id).
    const uint32_t n_ids = 0xffffffffu;
    const size_t budget = 160 * 1024;
    uint32_t tw = 32;
    while (tw > 1 && (size_t)d * tw * 8 > budget) tw >>= 1;
    SG_CUDA_TRY(cudaMemsetAsync(bitmaps, 0, (size_t)d * stride * 8, st));
    if ((size_t)d * tw * 8 > budget) {
        transpose_global_kernel<<<1024, 256, 0, st>>>(row_ptr, items, n_txn, remap, n_ids, d,
                                                      reinterpret_cast<unsigned long long *>(bitmaps), stride);
        SG_CUDA_TRY(cudaGetLastError());
        if (counts) launch_row_popc(bitmaps, stride, stride, d, counts, st);
        return;
    }
    const size_t smem = (size_t)d * tw * 8;
    SG_CUDA_TRY(cudaFuncSetAttribute(transpose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (counts) SG_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)d * 4, st));
    const uint64_t tiles = (n_txn + (uint64_t)tw * 64 - 1) / ((uint64_t)tw * 64);
    transpose_kernel<<<(unsigned)tiles, 512, smem, st>>>(row_ptr, items, n_txn, remap, n_ids, d, bitmaps, stride,
                                                          counts, tw);
    SG_CUDA_TRY(cudaGetLastError());
}

namespace {
// Candidate CSR from the host, checked and mapped on the device: bad[0] |= 1 when
// cand_ptr decreases anywhere; items become dense rows (ids that never occur map
// past the last row, where every support is 0).  remap null = identity on [0, n_ids).
__global__ void cand_prep_kernel(const uint64_t *__restrict__ cand_ptr, uint64_t n_cand, uint32_t *__restrict__ items,
                                 uint64_t n_items, const int32_t *__restrict__ remap, uint32_t n_ids,
                                 uint32_t *__restrict__ bad) {
    const uint64_t n = n_cand > n_items ? n_cand : n_items;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < n_cand && cand_ptr[i + 1] < cand_ptr[i]) atomicOr(bad, 1u);
        if (i < n_items) {
            const uint32_t id = items[i];
            uint32_t r = 0xfffffffeu;
            if (id < n_ids) {
                const int32_t m = remap ? remap[id] : (int32_t)id;
                if (m >= 0) r = (uint32_t)m;
            }
            items[i] = r;
        }
    }
}
}  // namespace

void launch_cand_prep(const uint64_t *cand_ptr, uint64_t n_cand, uint32_t *items, uint64_t n_items,
                      const int32_t *remap, uint32_t n_ids, uint32_t *bad, cudaStream_t st, int n_sm) {
    const uint64_t n = std::max<uint64_t>(std::max(n_cand, n_items), 1);
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)n_sm * 8);
    cand_prep_kernel<<<blocks, 256, 0, st>>>(cand_ptr, n_cand, items, n_items, remap, n_ids, bad);
    SG_CUDA_TRY(cudaGetLastError());
}

void launch_row_popc(const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t d, uint32_t *counts,
                     cudaStream_t st) {
    if (d == 0) return;
    row_popc_kernel<<<d, 256, 0, st>>>(rows, stride, n_words, d, counts);
    SG_CUDA_TRY(cudaGetLastError());
}

// ---------------------------------------------------------------- streaming queries
// One warp per query; each lane streams 16-byte words of the mask and of the
// query's rows with non-coherent 128-bit loads, ANDs them and popcounts.
__global__ void __launch_bounds__(256) query_kernel(QueryBatch qb) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t n_q = qb.n_q_device ? *qb.n_q_device : qb.n_q;
    for (uint64_t j = warp; j < n_q; j += n_warps) {
        const uint64_t q = qb.q_index ? qb.q_index[j] : j;
        const uint64_t a = qb.q_ptr[q], b = qb.q_ptr[q + 1];
        const uint64_t *mask = nullptr;
        if (qb.mask_slot) {
            const uint32_t s = qb.mask_slot[q];
            if (s != kNoSlot) mask = qb.arena + (uint64_t)s * qb.arena_stride;
        }
        if (a == b && mask == nullptr) {
            if (lane == 0) qb.out[q] = (uint32_t)qb.empty_value;
            continue;
        }
        bool bad = false;
        for (uint64_t i = a + lane; i < b; i += 32) bad |= qb.q_items[i] >= qb.d;
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) qb.out[q] = 0;
            continue;
        }
        uint32_t acc = 0;
        const uint64_t w_first = qb.q_w0 ? (qb.q_w0[q] & ~1ull) : 0;
        for (uint64_t base = w_first; base < qb.n_words; base += 64) {
            const uint64_t w = base + 2 * lane;
            if (w < qb.n_words) {
                uint4 v = mask ? ld_nc_v4(mask + w) : make_uint4(~0u, ~0u, ~0u, ~0u);
                for (uint64_t i = a; i < b; ++i) {
                    // once the AND is empty the remaining rows cannot add a bit
                    if ((v.x | v.y | v.z | v.w) == 0) break;
                    v = and4(v, ld_nc_v4(qb.rows + (uint64_t)qb.q_items[i] * qb.row_stride + w));
                }
                acc += popc4(v);
            }
            if (qb.mode == QUERY_ANY && __any_sync(0xffffffffu, acc != 0)) break;
            if (qb.mode == QUERY_ANY2 && __reduce_add_sync(0xffffffffu, acc) >= 2) break;
        }
        acc = warp_sum(acc);
        if (lane == 0) qb.out[q] = acc;
    }
}

// Tail counts of a wave's nodes: entry j of the concatenated tails belongs to
// node i (tail_ptr[i] <= j < tail_ptr[i+1]); out[j] = popc(mask(slot[i]) AND
// row(items[j])).  One warp per entry, the node found by binary search, so
// the host builds one record per node instead of one query per tail item.
__global__ void __launch_bounds__(256) tail_count_kernel(const uint64_t *__restrict__ rows, uint64_t row_stride,
                                                        uint64_t n_words, const uint64_t *__restrict__ arena,
                                                        uint64_t arena_stride, const uint32_t *__restrict__ slot,
                                                        const uint64_t *__restrict__ tail_ptr, uint32_t n_nodes,
                                                        const uint32_t *__restrict__ items, uint32_t *__restrict__ out) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t total = tail_ptr[n_nodes];
    for (uint64_t j = warp; j < total; j += n_warps) {
        uint32_t lo = 0, hi = n_nodes - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (tail_ptr[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        const uint64_t *mask = arena + (uint64_t)slot[lo] * arena_stride;
        const uint64_t *row = rows + (uint64_t)items[j] * row_stride;
        uint32_t acc = 0;
        for (uint64_t w = 2 * lane; w < n_words; w += 64) acc += popc4(and4(ld_nc_v4(mask + w), ld_nc_v4(row + w)));
        acc = warp_sum(acc);
        if (lane == 0) out[j] = acc;
    }
}

void launch_tail_counts(const uint64_t *rows, uint64_t row_stride, uint64_t n_words, const uint64_t *arena,
                        uint64_t arena_stride, const uint32_t *slot, const uint64_t *tail_ptr, uint32_t n_nodes,
                        uint64_t n_entries, const uint32_t *items, uint32_t *out, cudaStream_t st, int n_sm) {
    if (n_nodes == 0 || n_entries == 0) return;
    const uint64_t blocks = std::min<uint64_t>((n_entries + 7) / 8, (uint64_t)n_sm * 64);
    tail_count_kernel<<<(unsigned)blocks, 256, 0, st>>>(rows, row_stride, n_words, arena, arena_stride, slot, tail_ptr,
                                                        n_nodes, items, out);
    SG_CUDA_TRY(cudaGetLastError());
}

void launch_queries(const QueryBatch &qb, cudaStream_t st, int n_sm) {
    uint64_t blocks;
    if (qb.n_q_device) {
        blocks = (uint64_t)n_sm * 8;
    } else {
        if (qb.n_q == 0) return;
        blocks = std::min<uint64_t>((qb.n_q + 7) / 8, (uint64_t)n_sm * 64);
    }
    query_kernel<<<(unsigned)blocks, 256, 0, st>>>(qb);
    SG_CUDA_TRY(cudaGetLastError());
}

// ---------------------------------------------------------------- staged batch supports
// Candidate records: 8 x uint16 row ids; 0xffff marks unused slots and an
// all-0xffff record marks a candidate whose support was written elsewhere.
constexpr uint16_t kRecNone = 0xffffu;
constexpr uint32_t kStagedRowsPerBox = 256;
constexpr uint32_t kStagedWords = 16;   // words per row per chunk (128 bytes)

__global__ void prep_records_kernel(const uint64_t *__restrict__ cand_ptr, const uint32_t *__restrict__ cand_items,
                                    uint64_t n, uint32_t d, uint64_t n_txn, uint4 *__restrict__ recs,
                                    uint32_t *__restrict__ ovf_list, unsigned long long *__restrict__ ovf_count,
                                    uint32_t *__restrict__ out) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = cand_ptr[c], b = cand_ptr[c + 1];
        const uint64_t k = b - a;
        uint32_t h[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
        if (k == 0) {
            out[c] = (uint32_t)n_txn;
        } else if (k > 8) {
            const unsigned long long slot = atomicAdd(ovf_count, 1ull);
            ovf_list[slot] = (uint32_t)c;
        } else {
            bool zero = false;
            uint16_t it[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) it[i] = kRecNone;
            for (uint64_t i = 0; i < k; ++i) {
                const uint32_t x = cand_items[a + i];
                if (x >= d) zero = true;
                it[i] = (uint16_t)x;
            }
            if (zero) {
                out[c] = 0;
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) h[i] = (uint32_t)it[2 * i] | ((uint32_t)it[2 * i + 1] << 16);
            }
        }
        recs[c] = make_uint4(h[0], h[1], h[2], h[3]);
    }
}

// 8-lane transpose-reduce: lane l (of an aligned group of 8) enters with
// partials p[0..7] for 8 candidates and leaves with the group-wide sum of p[l].
__device__ __forceinline__ uint32_t treduce8(const uint32_t (&p)[8], uint32_t l) {
    uint32_t q[4], r[2];
    const bool h4 = l & 4, h2 = l & 2, h1 = l & 1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t send = h4 ? p[k] : p[k + 4];
        const uint32_t keep = h4 ? p[k + 4] : p[k];
        q[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t send = h2 ? q[k] : q[k + 2];
        const uint32_t keep = h2 ? q[k + 2] : q[k];
        r[k] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    const uint32_t send = h1 ? r[0] : r[1];
    const uint32_t keep = h1 ? r[1] : r[0];
    return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

// Each CTA owns `cpc` consecutive candidates and sweeps the whole transaction
// range in chunks of 16 words (1024 transactions).  Per chunk, TMA copies the
// 128-byte slice of every bitmap row into shared memory (rows r*128 bytes
// apart); a group of 8 lanes then evaluates one candidate at a time, each
// lane ANDing a 16-byte piece of the k rows, so a warp reads 4 rows x 128
// contiguous bytes per step (4 conflict-free wavefronts).  Partial popcounts
// of 8 candidates are transpose-reduced into one register per lane, which
// accumulates across chunks: each support is written once, at the end.
template <int THREADS, int SMAX>
__global__ void __launch_bounds__(THREADS, 1)
    k1_staged_kernel(const __grid_constant__ CUtensorMap bm_map, uint32_t n_boxes, uint64_t n_words,
                     const uint4 *__restrict__ recs, uint64_t n_cand, uint32_t cpc, uint32_t *__restrict__ out,
                     uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr uint32_t G = THREADS / 8;             // groups of 8 lanes
    uint8_t *chunk = smem;                           // n_boxes * 256 rows * 128 B
    const uint32_t chunk_bytes = n_boxes * kStagedRowsPerBox * kStagedWords * 8;
    uint4 *rec_s = reinterpret_cast<uint4 *>(smem + chunk_bytes);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + chunk_bytes + (size_t)cpc * 16);

    const uint32_t tid = threadIdx.x;
    const uint32_t g = tid >> 3, l = tid & 7;
    const uint64_t base = (uint64_t)blockIdx.x * cpc;
    if (base >= n_cand) return;
    const uint64_t left = n_cand - base;
    const uint32_t ncta = left < cpc ? (uint32_t)left : cpc;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    for (uint32_t i = tid; i < ncta; i += THREADS) rec_s[i] = recs[base + i];
    __syncthreads();

    uint32_t acc[SMAX];
#pragma unroll
    for (int s = 0; s < SMAX; ++s) acc[s] = 0;
    const uint32_t n_sets = (ncta + 8 * G - 1) / (8 * G);
    const uint64_t n_chunks = (n_words + kStagedWords - 1) / kStagedWords;
    uint32_t phase = 0;
    for (uint64_t ch = 0; ch < n_chunks; ++ch) {
        if (tid == 0) {
            mbar_arrive_expect_tx(bar, chunk_bytes);
            for (uint32_t b = 0; b < n_boxes; ++b)
                tma_load_2d(chunk + (size_t)b * kStagedRowsPerBox * kStagedWords * 8, &bm_map,
                            (int32_t)(ch * kStagedWords), (int32_t)(b * kStagedRowsPerBox), bar);
        }
        const bool ok = mbar_wait_bounded(bar, phase, err);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            // give in-flight copies one more bounded chance to land before leaving
            mbar_wait_bounded(bar, phase ^ 1, err);
            return;
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s) {
            if ((uint32_t)s < n_sets) {
                uint32_t p[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t c = ((uint32_t)s * 8 + j) * G + g;
                    uint32_t v = 0;
                    if (c < ncta) {
                        const uint4 r = rec_s[c];
                        const uint32_t h[4] = {r.x, r.y, r.z, r.w};
                        uint32_t it0 = h[0] & 0xffffu;
                        if (it0 != kRecNone) {
                            uint4 m = *reinterpret_cast<const uint4 *>(chunk + (size_t)it0 * 128 + l * 16);
#pragma unroll
                            for (int k = 1; k < 8; ++k) {
                                const uint32_t it = (h[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
                                if (it == kRecNone) break;
                                m = and4(m, *reinterpret_cast<const uint4 *>(chunk + (size_t)it * 128 + l * 16));
                            }
                            v = popc4(m);
                        }
                    }
                    p[j] = v;
                }
                acc[s] += treduce8(p, l);
            }
        }
        __syncthreads();  // every group is done with this chunk before TMA overwrites it
    }
#pragma unroll
    for (int s = 0; s < SMAX; ++s) {
        const uint32_t c = ((uint32_t)s * 8 + l) * G + g;
        if ((uint32_t)s < n_sets && c < ncta) {
            const uint32_t it0 = rec_s[c].x & 0xffffu;
            if (it0 != kRecNone) out[base + c] = acc[s];
        }
    }
}

// 4-lane transpose-reduce: lane l (of an aligned group of 4) enters with
// partials p[0..3] for 4 candidates and leaves with the group-wide sum of p[l].
__device__ __forceinline__ uint32_t treduce4(const uint32_t (&p)[4], uint32_t l) {
    uint32_t q[2];
    const bool h2 = l & 2, h1 = l & 1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t send = h2 ? p[k] : p[k + 2];
        const uint32_t keep = h2 ? p[k + 2] : p[k];
        q[k] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    const uint32_t send = h1 ? q[0] : q[1];
    const uint32_t keep = h1 ? q[1] : q[0];
    return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

// k1_staged_kernel with groups of 4 lanes: each lane ANDs 32 bytes of a row
// (two 16-byte pieces, 64 bytes apart), so a candidate's record is decoded by
// 4 lanes instead of 8 and a warp evaluates 8 candidates per step.  Even
// groups read the row's first half first and odd groups its second half
// first: the two groups of an 8-lane phase of a 128-bit shared load then hit
// disjoint banks.
template <int THREADS, int SMAX>
__global__ void __launch_bounds__(THREADS, 1)
    k1_staged4_kernel(const __grid_constant__ CUtensorMap bm_map, uint32_t n_boxes, uint64_t n_words,
                      const uint4 *__restrict__ recs, uint64_t n_cand, uint32_t cpc, uint32_t *__restrict__ out,
                      uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr uint32_t G = THREADS / 4;             // groups of 4 lanes
    uint8_t *chunk = smem;                           // n_boxes * 256 rows * 128 B
    const uint32_t chunk_bytes = n_boxes * kStagedRowsPerBox * kStagedWords * 8;
    uint4 *rec_s = reinterpret_cast<uint4 *>(smem + chunk_bytes);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + chunk_bytes + (size_t)cpc * 16);

    const uint32_t tid = threadIdx.x;
    const uint32_t g = tid >> 2, l = tid & 3;
    const uint32_t off_a = ((g & 1) ? 64u : 0u) + l * 16, off_b = ((g & 1) ? 0u : 64u) + l * 16;
    const uint64_t base = (uint64_t)blockIdx.x * cpc;
    if (base >= n_cand) return;
    const uint64_t left = n_cand - base;
    const uint32_t ncta = left < cpc ? (uint32_t)left : cpc;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    for (uint32_t i = tid; i < ncta; i += THREADS) rec_s[i] = recs[base + i];
    __syncthreads();

    uint32_t acc[SMAX];
#pragma unroll
    for (int s = 0; s < SMAX; ++s) acc[s] = 0;
    const uint32_t n_sets = (ncta + 4 * G - 1) / (4 * G);
    const uint64_t n_chunks = (n_words + kStagedWords - 1) / kStagedWords;
    uint32_t phase = 0;
    for (uint64_t ch = 0; ch < n_chunks; ++ch) {
        if (tid == 0) {
            mbar_arrive_expect_tx(bar, chunk_bytes);
            for (uint32_t b = 0; b < n_boxes; ++b)
                tma_load_2d(chunk + (size_t)b * kStagedRowsPerBox * kStagedWords * 8, &bm_map,
                            (int32_t)(ch * kStagedWords), (int32_t)(b * kStagedRowsPerBox), bar);
        }
        const bool ok = mbar_wait_bounded(bar, phase, err);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            // give in-flight copies one more bounded chance to land before leaving
            mbar_wait_bounded(bar, phase ^ 1, err);
            return;
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s) {
            if ((uint32_t)s < n_sets) {
                uint32_t p[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t c = ((uint32_t)s * 4 + j) * G + g;
                    uint32_t v = 0;
                    if (c < ncta) {
                        const uint4 r = rec_s[c];
                        const uint32_t h[4] = {r.x, r.y, r.z, r.w};
                        const uint32_t it0 = h[0] & 0xffffu;
                        if (it0 != kRecNone) {
                            const uint8_t *row = chunk + (size_t)it0 * 128;
                            uint4 ma = *reinterpret_cast<const uint4 *>(row + off_a);
                            uint4 mb = *reinterpret_cast<const uint4 *>(row + off_b);
#pragma unroll
                            for (int k = 1; k < 8; ++k) {
                                const uint32_t it = (h[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
                                if (it == kRecNone) break;
                                const uint8_t *rk = chunk + (size_t)it * 128;
                                ma = and4(ma, *reinterpret_cast<const uint4 *>(rk + off_a));
                                mb = and4(mb, *reinterpret_cast<const uint4 *>(rk + off_b));
                            }
                            v = popc4(ma) + popc4(mb);
                        }
                    }
                    p[j] = v;
                }
                acc[s] += treduce4(p, l);
            }
        }
        __syncthreads();  // every group is done with this chunk before TMA overwrites it
    }
#pragma unroll
    for (int s = 0; s < SMAX; ++s) {
        const uint32_t c = ((uint32_t)s * 4 + l) * G + g;
        if ((uint32_t)s < n_sets && c < ncta) {
            const uint32_t it0 = rec_s[c].x & 0xffffu;
            if (it0 != kRecNone) out[base + c] = acc[s];
        }
    }
}

// ---------------------------------------------------------------- sorted batch supports
// Candidates are counting-sorted by key = (k - 1) * 4096 + first item, so that
// (a) the four 8-lane groups of a warp almost always share k and run one fully
// unrolled, branch-free K-load AND (unused record slots point at an all-ones
// row in shared memory), and (b) consecutive candidates of a group usually
// share their first item, whose 16-byte piece then stays in registers.
// Sorted record: item0 in bits 0..11 and k in bits 12..15 of .x, items 1..7
// as 16-bit fields; pad items = the all-ones row index.
constexpr uint32_t kSortItemMax = 4096;
constexpr uint32_t kSortBins = 8 * kSortItemMax;
constexpr uint32_t kSortCompactMax = 1024;  // 10-bit ids in the 12-byte sorted records

__global__ void sort_count_kernel(const uint64_t *__restrict__ cand_ptr, const uint32_t *__restrict__ cand_items,
                                  uint64_t n, uint32_t d, uint64_t n_txn, uint32_t *__restrict__ bins,
                                  uint32_t *__restrict__ ovf_list, unsigned long long *__restrict__ ovf_count,
                                  uint32_t *__restrict__ out) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = cand_ptr[c], b = cand_ptr[c + 1];
        const uint64_t k = b - a;
        if (k == 0) {
            out[c] = (uint32_t)n_txn;
        } else if (k > 8) {
            ovf_list[atomicAdd(ovf_count, 1ull)] = (uint32_t)c;
        } else {
            uint32_t mn = 0xffffffffu;
            bool zero = false;
            for (uint64_t i = a; i < b; ++i) {
                const uint32_t x = cand_items[i];
                zero |= x >= d;
                mn = min(mn, x);
            }
            if (zero) out[c] = 0;
            else atomicAdd(&bins[(uint32_t)(k - 1) * kSortItemMax + mn], 1u);
        }
    }
}

// Exclusive scan of the bins in place (one CTA of 1024 threads); total -> *n_valid.
__global__ void __launch_bounds__(1024) sort_scan_kernel(uint32_t *__restrict__ bins, uint64_t *__restrict__ n_valid) {
    constexpr uint32_t per = kSortBins / 1024;
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    uint32_t s = 0;
    for (uint32_t i = 0; i < per; ++i) s += bins[t * per + i];
    part[t] = s;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1) {
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t ? part[t - 1] : 0u;
    for (uint32_t i = 0; i < per; ++i) {
        const uint32_t v = bins[t * per + i];
        bins[t * per + i] = run;
        run += v;
    }
    if (t == 1023) *n_valid = part[1023];
}

// Sorted record (12 bytes, ids < 1024): lo = items 0..5 as 10-bit fields and
// k in bits 60..63; hi = items 6..7 as 10-bit fields.  Slots beyond k repeat
// item 0 (AND is idempotent), so no padding row is needed.
__global__ void sort_scatter_kernel(const uint64_t *__restrict__ cand_ptr, const uint32_t *__restrict__ cand_items,
                                    uint64_t n, uint32_t d, uint32_t *__restrict__ cursor,
                                    uint64_t *__restrict__ rec_lo, uint32_t *__restrict__ rec_hi,
                                    uint32_t *__restrict__ perm) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = cand_ptr[c], b = cand_ptr[c + 1];
        const uint64_t k = b - a;
        if (k == 0 || k > 8) continue;
        uint32_t it[8];
        uint32_t mn = 0xffffffffu, at = 0;
        bool zero = false;
        for (uint64_t i = a; i < b; ++i) {
            const uint32_t x = cand_items[i];
            zero |= x >= d;
            if (x < mn) { mn = x; at = (uint32_t)(i - a); }
            it[i - a] = x;
        }
        if (zero) continue;
        // the smallest item goes first (it is the sort key and the reused row)
        it[at] = it[0];
        it[0] = mn;
        for (uint64_t i = k; i < 8; ++i) it[i] = mn;
        const uint32_t pos = atomicAdd(&cursor[(uint32_t)(k - 1) * kSortItemMax + mn], 1u);
        uint64_t lo = (uint64_t)k << 60;
#pragma unroll
        for (int i = 0; i < 6; ++i) lo |= (uint64_t)it[i] << (10 * i);
        rec_lo[pos] = lo;
        rec_hi[pos] = it[6] | (it[7] << 10);
        perm[pos] = (uint32_t)c;
    }
}

__device__ __forceinline__ uint32_t rec_item(uint64_t lo, uint32_t hi, int i) {
    return i < 6 ? (uint32_t)(lo >> (10 * i)) & 1023u : (hi >> (10 * (i - 6))) & 1023u;
}

template <int K>
__device__ __forceinline__ uint4 and_tail(const uint8_t *base, uint64_t lo, uint32_t hi, uint4 m) {
#pragma unroll
    for (int i = 1; i < K; ++i) m = and4(m, *reinterpret_cast<const uint4 *>(base + (size_t)rec_item(lo, hi, i) * 128));
    return m;
}

// Same chunk pipeline as k1_staged_kernel.  Group g owns a contiguous run of
// the CTA's sorted candidates, so consecutive candidates usually share k
// (one unrolled K-load AND per warp, K = the warp's largest k) and their
// first item, whose 16-byte piece stays in registers.  Slots past a group's
// run issue no shared loads.
template <int THREADS, int SMAX>
__global__ void __launch_bounds__(THREADS, 1)
    k1_sorted_kernel(const __grid_constant__ CUtensorMap bm_map, uint32_t n_boxes, uint64_t n_words,
                     const uint64_t *__restrict__ rec_lo, const uint32_t *__restrict__ rec_hi,
                     const uint32_t *__restrict__ perm, const uint64_t *__restrict__ n_valid, uint32_t cpc,
                     uint32_t *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr uint32_t G = THREADS / 8;
    const uint32_t chunk_bytes = n_boxes * kStagedRowsPerBox * kStagedWords * 8;
    uint8_t *chunk = smem;
    uint64_t *lo_s = reinterpret_cast<uint64_t *>(smem + chunk_bytes);
    uint32_t *hi_s = reinterpret_cast<uint32_t *>(lo_s + cpc);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + chunk_bytes + (size_t)cpc * 12 + 16 - ((size_t)cpc * 12) % 16);

    const uint32_t tid = threadIdx.x, g = tid >> 3, l = tid & 7;
    const uint64_t nv = *n_valid;
    const uint64_t base = (uint64_t)blockIdx.x * cpc;
    if (base >= nv) return;
    const uint32_t ncta = (uint32_t)min((uint64_t)cpc, nv - base);
    const uint32_t per_g = (ncta + G - 1) / G;
    const uint32_t g_lo = min(g * per_g, ncta), g_hi = min(g_lo + per_g, ncta);
    const uint32_t n_sets = (per_g + 7) / 8;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    for (uint32_t i = tid; i < ncta; i += THREADS) {
        lo_s[i] = rec_lo[base + i];
        hi_s[i] = rec_hi[base + i];
    }
    __syncthreads();

    uint32_t acc[SMAX];
#pragma unroll
    for (int s = 0; s < SMAX; ++s) acc[s] = 0;
    const uint64_t n_chunks = (n_words + kStagedWords - 1) / kStagedWords;
    const uint8_t *lane_base = chunk + l * 16;
    uint32_t phase = 0;
    for (uint64_t ch = 0; ch < n_chunks; ++ch) {
        if (tid == 0) {
            mbar_arrive_expect_tx(bar, chunk_bytes);
            for (uint32_t b = 0; b < n_boxes; ++b)
                tma_load_2d(chunk + (size_t)b * kStagedRowsPerBox * kStagedWords * 8, &bm_map,
                            (int32_t)(ch * kStagedWords), (int32_t)(b * kStagedRowsPerBox), bar);
        }
        const bool ok = mbar_wait_bounded(bar, phase, err);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            mbar_wait_bounded(bar, phase ^ 1, err);
            return;
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s) {
            if ((uint32_t)s < n_sets) {
                uint32_t p[8];
                uint32_t cur0 = 0xffffffffu;
                uint4 row0 = make_uint4(0, 0, 0, 0);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t c = g_lo + (uint32_t)s * 8 + j;
                    const bool valid = c < g_hi;
                    uint64_t lo = 0;
                    uint32_t hi = 0;
                    if (valid) {
                        lo = lo_s[c];
                        hi = hi_s[c];
                    }
                    const uint32_t k = (uint32_t)(lo >> 60);
                    const uint32_t kmax = __reduce_max_sync(0xffffffffu, k);
                    uint32_t v = 0;
                    if (valid) {
                        const uint32_t it0 = (uint32_t)lo & 1023u;
                        if (it0 != cur0) {
                            row0 = *reinterpret_cast<const uint4 *>(lane_base + (size_t)it0 * 128);
                            cur0 = it0;
                        }
                        uint4 m = row0;
                        switch (kmax) {
                            case 2: m = and_tail<2>(lane_base, lo, hi, m); break;
                            case 3: m = and_tail<3>(lane_base, lo, hi, m); break;
                            case 4: m = and_tail<4>(lane_base, lo, hi, m); break;
                            case 5: m = and_tail<5>(lane_base, lo, hi, m); break;
                            case 6: m = and_tail<6>(lane_base, lo, hi, m); break;
                            case 7: m = and_tail<7>(lane_base, lo, hi, m); break;
                            case 8: m = and_tail<8>(lane_base, lo, hi, m); break;
                            default: break;
                        }
                        v = popc4(m);
                    }
                    p[j] = v;
                }
                acc[s] += treduce8(p, l);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int s = 0; s < SMAX; ++s) {
        const uint32_t c = g_lo + (uint32_t)s * 8 + l;
        if ((uint32_t)s < n_sets && c < g_hi) out[perm[base + c]] = acc[s];
    }
}

constexpr int kStagedThreads = 1024;
constexpr int kStagedSmax = 8;
constexpr int kStagedSmax4 = 8;   // 4-lane groups: 8 sets x 4 candidates x 256 groups = 8,192
constexpr int kSortedSmax = 8;
constexpr uint32_t kSortedMaxCpc = kStagedThreads / 8 * 8 * kSortedSmax;  // 8192

size_t sorted_smem_bytes(uint32_t d, uint32_t cpc) {
    const uint32_t n_boxes = (d + kStagedRowsPerBox - 1) / kStagedRowsPerBox;
    return (size_t)n_boxes * kStagedRowsPerBox * kStagedWords * 8 + (size_t)cpc * 12 + 16 + 64;
}
constexpr uint32_t kStagedMaxCpc = kStagedThreads / 8 * 8 * kStagedSmax;  // 8192

size_t staged_smem_bytes(uint32_t d, uint32_t cpc) {
    const uint32_t n_boxes = (d + kStagedRowsPerBox - 1) / kStagedRowsPerBox;
    return (size_t)n_boxes * kStagedRowsPerBox * kStagedWords * 8 + (size_t)cpc * 16 + 64;
}

bool encode_bitmap_map(CUtensorMap *map, const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride) {
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
    if ((reinterpret_cast<uintptr_t>(bitmaps) & 15) || (row_stride & 1)) return false;
    cuuint64_t dims[2] = {(cuuint64_t)n_words, (cuuint64_t)d};
    cuuint64_t strides[1] = {(cuuint64_t)row_stride * 8};
    cuuint32_t box[2] = {kStagedWords, kStagedRowsPerBox};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<uint64_t *>(bitmaps), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

size_t support_scratch_bytes(uint64_t n_cand) { return support_scratch_bytes_for(n_cand); }

int support_batch_device(const uint64_t *bitmaps, uint32_t d, uint64_t n_words, uint64_t row_stride,
                         uint64_t n_txn, const uint64_t *cand_ptr, const uint32_t *cand_items, uint64_t n_cand,
                         uint32_t *out, const SupportScratch &scratch, const SupportPlan &plan,
                         const CUtensorMap *map, uint32_t *dev_err, cudaStream_t st, int n_sm, uint64_t *launches,
                         cudaEvent_t *ev) {
    if (n_cand == 0) return 0;
    auto mark = [&](int i) {
        if (ev) SG_CUDA_TRY(cudaEventRecord(ev[i], st));
    };
    const uint64_t n_words_even = (n_words + 1) & ~1ull;
    // default grid: one wave of CTAs for the sorted kernel (its 12-byte records leave room
    // for ~6,600 candidates per CTA), two for the staged kernel
    auto pick_cpc = [&](uint32_t cap, size_t (*smem_fn)(uint32_t, uint32_t), uint32_t waves) -> uint32_t {
        const uint64_t ctas_target = (uint64_t)n_sm * std::max<uint32_t>(1, plan.waves ? plan.waves : waves);
        uint32_t cpc = plan.cands_per_cta;
        if (cpc == 0) cpc = (uint32_t)std::min<uint64_t>(cap, (n_cand + ctas_target - 1) / ctas_target);
        cpc = std::max<uint32_t>(1, std::min(cpc, cap));
        while (cpc > 1 && smem_fn(d, cpc) > 227 * 1024) cpc = cpc * 3 / 4;
        return smem_fn(d, cpc) <= 227 * 1024 ? cpc : 0;
    };
    int kind = plan.kernel;
    if (map == nullptr || d == 0) kind = SUPPORT_STREAM;
    // measured on GB300 at 1M candidates x 1,024 rows: lane with TMEM records 22.3 ms, lane
    // with shared-memory records 23.2 ms, staged with 4-lane groups 30.0 ms, staged with 8-lane
    // groups 30.9 ms, sorted 30.8-46 ms (depending on its grid).  AUTO falls through to the
    // shared-memory lane form, then STAGED4, when a layout does not fit.
    if (kind == SUPPORT_AUTO) kind = lane_supported(d) ? SUPPORT_LANE_TM : SUPPORT_STAGED4;
    if (kind == SUPPORT_LANE || kind == SUPPORT_LANE_TM) {
        uint32_t *ovf_l = nullptr;
        unsigned long long *ovf_c = nullptr;
        mark(0);
        int rc = -1;
        if (kind == SUPPORT_LANE_TM)
            rc = lane_tm_supports_device(map, d, n_words_even, cand_ptr, cand_items, n_cand, n_txn, out,
                                         scratch.base, scratch.bytes, plan.waves ? plan.waves : 1, dev_err, st, n_sm,
                                         &ovf_l, &ovf_c, launches, ev);
        if (rc != 0)
            rc = lane_supports_device(map, d, n_words_even, cand_ptr, cand_items, n_cand, n_txn, out, scratch.base,
                                      scratch.bytes, kind == SUPPORT_LANE && plan.waves ? plan.waves : 2, dev_err, st,
                                      n_sm, &ovf_l, &ovf_c, launches, ev);
        if (rc == 0) {
            QueryBatch qb;
            qb.rows = bitmaps; qb.row_stride = row_stride; qb.n_words = n_words_even; qb.d = d;
            qb.q_ptr = cand_ptr; qb.q_items = cand_items; qb.n_q_device = reinterpret_cast<const uint64_t *>(ovf_c);
            qb.q_index = ovf_l; qb.out = out; qb.empty_value = n_txn;
            launch_queries(qb, st, n_sm);
            mark(3);
            if (launches) *launches += 1;
            return 0;
        }
        if (scratch.bytes < support_scratch_bytes(n_cand)) return -1;
        kind = SUPPORT_STAGED4;
    }
    if (kind == SUPPORT_SORTED && d > kSortCompactMax) kind = SUPPORT_STAGED;
    if ((kind == SUPPORT_STAGED || kind == SUPPORT_STAGED4) && d > 65535) kind = SUPPORT_STREAM;
    uint32_t cpc = 0;
    if (kind == SUPPORT_SORTED) {
        cpc = pick_cpc(kSortedMaxCpc, sorted_smem_bytes, 1);
        if (!cpc) kind = SUPPORT_STREAM;
    } else if (kind == SUPPORT_STAGED || kind == SUPPORT_STAGED4) {
        cpc = pick_cpc(kStagedMaxCpc, staged_smem_bytes, 2);
        if (!cpc) kind = SUPPORT_STREAM;
    }
    if (kind == SUPPORT_STREAM) {
        QueryBatch qb;
        qb.rows = bitmaps; qb.row_stride = row_stride; qb.n_words = n_words_even; qb.d = d;
        qb.q_ptr = cand_ptr; qb.q_items = cand_items; qb.n_q = n_cand; qb.out = out; qb.empty_value = n_txn;
        mark(0);
        mark(1);
        launch_queries(qb, st, n_sm);
        mark(2);
        mark(3);
        if (launches) *launches += 1;
        return 0;
    }
    if (scratch.bytes < support_scratch_bytes(n_cand)) return -1;
    uint8_t *sb = static_cast<uint8_t *>(scratch.base);
    uint4 *recs = reinterpret_cast<uint4 *>(sb);
    uint32_t *ovf = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16));
    uint32_t *perm = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + align256(n_cand * 4));
    uint32_t *bins = reinterpret_cast<uint32_t *>(sb + align256(n_cand * 16) + 2 * align256(n_cand * 4));
    unsigned long long *ovf_n = reinterpret_cast<unsigned long long *>(
        sb + align256(n_cand * 16) + 2 * align256(n_cand * 4) + align256(kSupportSortBins * 4));
    uint64_t *n_valid = reinterpret_cast<uint64_t *>(ovf_n + 1);
    const uint32_t n_boxes = (d + kStagedRowsPerBox - 1) / kStagedRowsPerBox;
    const unsigned prep_blocks = (unsigned)std::min<uint64_t>((n_cand + 255) / 256, (uint64_t)n_sm * 16);
    const uint64_t ctas = (n_cand + cpc - 1) / cpc;
    mark(0);
    SG_CUDA_TRY(cudaMemsetAsync(ovf_n, 0, 8, st));
    if (kind == SUPPORT_SORTED) {
        SG_CUDA_TRY(cudaMemsetAsync(bins, 0, kSupportSortBins * 4, st));
        sort_count_kernel<<<prep_blocks, 256, 0, st>>>(cand_ptr, cand_items, n_cand, d, n_txn, bins, ovf, ovf_n, out);
        SG_CUDA_TRY(cudaGetLastError());
        sort_scan_kernel<<<1, 1024, 0, st>>>(bins, n_valid);
        SG_CUDA_TRY(cudaGetLastError());
        uint64_t *rec_lo = reinterpret_cast<uint64_t *>(recs);
        uint32_t *rec_hi = reinterpret_cast<uint32_t *>(rec_lo + n_cand);
        sort_scatter_kernel<<<prep_blocks, 256, 0, st>>>(cand_ptr, cand_items, n_cand, d, bins, rec_lo, rec_hi, perm);
        SG_CUDA_TRY(cudaGetLastError());
        const size_t smem = sorted_smem_bytes(d, cpc);
        auto kern = k1_sorted_kernel<kStagedThreads, kSortedSmax>;
        SG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        mark(1);
        kern<<<(unsigned)ctas, kStagedThreads, smem, st>>>(*map, n_boxes, n_words_even, rec_lo, rec_hi, perm, n_valid,
                                                           cpc, out, dev_err);
        SG_CUDA_TRY(cudaGetLastError());
        mark(2);
        if (launches) *launches += 4;
    } else {
        prep_records_kernel<<<prep_blocks, 256, 0, st>>>(cand_ptr, cand_items, n_cand, d, n_txn, recs, ovf, ovf_n,
                                                         out);
        SG_CUDA_TRY(cudaGetLastError());
        const size_t smem = staged_smem_bytes(d, cpc);
        auto kern = kind == SUPPORT_STAGED4 ? k1_staged4_kernel<kStagedThreads, kStagedSmax4>
                                            : k1_staged_kernel<kStagedThreads, kStagedSmax>;
        SG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        mark(1);
        kern<<<(unsigned)ctas, kStagedThreads, smem, st>>>(*map, n_boxes, n_words_even, recs, n_cand, cpc, out,
                                                           dev_err);
        SG_CUDA_TRY(cudaGetLastError());
        mark(2);
        if (launches) *launches += 2;
    }
    // candidates with more than 8 items
    QueryBatch qb;
    qb.rows = bitmaps; qb.row_stride = row_stride; qb.n_words = n_words_even; qb.d = d;
    qb.q_ptr = cand_ptr; qb.q_items = cand_items; qb.n_q_device = reinterpret_cast<const uint64_t *>(ovf_n);
    qb.q_index = ovf; qb.out = out; qb.empty_value = n_txn;
    launch_queries(qb, st, n_sm);
    mark(3);
    if (launches) *launches += 1;
    return 0;
}

// ---------------------------------------------------------------- wait self-test
// An mbarrier that nothing ever arrives at: every thread's bounded wait runs
// out, records DEVERR_MBAR_TIMEOUT and returns.  No copy or MMA is issued, so
// nothing is in flight when the CTA leaves.
__global__ void wait_probe_kernel(uint32_t *err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    mbar_wait_bounded(&bar, 0, err);
}

void launch_wait_probe(uint32_t *err, cudaStream_t st) {
    wait_probe_kernel<<<1, 32, 0, st>>>(err);
    SG_CUDA_TRY(cudaGetLastError());
}

// ---------------------------------------------------------------- projected databases
// Exclusive prefix popcounts of a row's words (one CTA): ofs[w] = set bits of
// words 0 .. w-1, the position of word w's first transaction in the projection.
__global__ void __launch_bounds__(1024) row_prefix_kernel(const uint64_t *__restrict__ row, uint64_t n_words,
                                                          uint32_t *__restrict__ ofs) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    const uint64_t per = (n_words + 1023) / 1024;
    const uint64_t w0 = min(n_words, (uint64_t)t * per), w1 = min(n_words, w0 + per);
    uint32_t s = 0;
    for (uint64_t w = w0; w < w1; ++w) s += popc64(row[w]);
    part[t] = s;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1) {   // inclusive scan
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - s;
    for (uint64_t w = w0; w < w1; ++w) {
        ofs[w] = run;
        run += popc64(row[w]);
    }
}

// The move masks of the compress (generalized extract) of each root word m,
// after H. S. Warren, Hacker's Delight, 2nd ed., section 7-4: six steps, step i
// shifting the bits in masks[i] right by 2^i, pack the bits of x under m to the
// low end in order.  The masks depend on m alone, so they are computed once per
// root and used for every projected row (masks[i * n_words + w]).
__global__ void root_masks_kernel(const uint64_t *__restrict__ root, uint64_t n_words, uint64_t *__restrict__ masks) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < n_words; w += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t m = root[w];
        uint64_t mk = ~m << 1;   // ones at positions whose lower neighbour is a zero of m
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            uint64_t mp = mk ^ (mk << 1);   // parallel suffix (prefix xor towards the high end)
            mp ^= mp << 2;
            mp ^= mp << 4;
            mp ^= mp << 8;
            mp ^= mp << 16;
            mp ^= mp << 32;
            const uint64_t mv = mp & m;     // bits that move by 2^i in this step
            m = (m ^ mv) | (mv >> (1 << i));
            mk &= ~mp;
            masks[(uint64_t)i * n_words + w] = mv;
        }
    }
}

// Row items[blockIdx.y] of the projection: the bits of that bitmap row at the set
// positions of `root`, packed in transaction order (out rows zeroed beforehand).
__global__ void project_rows_kernel(const uint64_t *__restrict__ rows, uint64_t stride, uint64_t n_words,
                                    const uint64_t *__restrict__ root, const uint32_t *__restrict__ ofs,
                                    const uint64_t *__restrict__ masks, const uint32_t *__restrict__ items,
                                    unsigned long long *__restrict__ out, uint64_t out_stride) {
    const uint32_t e = items[blockIdx.y];
    const uint64_t *src = rows + (uint64_t)e * stride;
    unsigned long long *dst = out + (uint64_t)e * out_stride;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < n_words; w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t m = root[w];
        if (!m) continue;
        uint64_t p = src[w] & m;
        if (!p) continue;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const uint64_t t = p & masks[(uint64_t)i * n_words + w];
            p = (p ^ t) | (t >> (1 << i));
        }
        const uint32_t nb = popc64(m);
        const uint32_t o = ofs[w], sh = o & 63;
        atomicOr(dst + (o >> 6), (unsigned long long)(p << sh));
        if (sh && sh + nb > 64) atomicOr(dst + (o >> 6) + 1, (unsigned long long)(p >> (64 - sh)));
    }
}

void launch_projection(const uint64_t *rows, uint64_t stride, uint64_t n_words, uint32_t root_row,
                       const uint32_t *items, uint32_t n_items, uint32_t *ofs, uint64_t *masks, uint64_t *out,
                       uint64_t out_stride, uint64_t out_words, uint32_t d, cudaStream_t st, int n_sm) {
    SG_CUDA_TRY(cudaMemset2DAsync(out, out_stride * 8, 0, out_words * 8, d, st));
    if (n_items == 0 || n_words == 0) return;
    const uint64_t *root = rows + (uint64_t)root_row * stride;
    row_prefix_kernel<<<1, 1024, 0, st>>>(root, n_words, ofs);
    SG_CUDA_TRY(cudaGetLastError());
    root_masks_kernel<<<(unsigned)std::min<uint64_t>((n_words + 255) / 256, (uint64_t)n_sm * 8), 256, 0, st>>>(
        root, n_words, masks);
    SG_CUDA_TRY(cudaGetLastError());
    const unsigned bx = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n_words + 255) / 256,
                                                                            (uint64_t)n_sm * 16 / std::max(1u, n_items) + 1));
    project_rows_kernel<<<dim3(bx, n_items), 256, 0, st>>>(rows, stride, n_words, root, ofs, masks, items,
                                                           reinterpret_cast<unsigned long long *>(out), out_stride);
    SG_CUDA_TRY(cudaGetLastError());
}

// ---------------------------------------------------------------- miner helpers
__global__ void child_mask_kernel(uint64_t *__restrict__ arena, uint64_t astride, uint64_t n_words,
                                  const uint64_t *__restrict__ rows, uint64_t rstride, const uint64_t *__restrict__ ptr,
                                  const uint32_t *__restrict__ items, const uint32_t *__restrict__ parent_slot,
                                  const uint32_t *__restrict__ child_slot, uint32_t n) {
    const uint64_t n_vec = n_words / 2;
    const uint64_t total = (uint64_t)n * n_vec;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(i / n_vec);
        const uint64_t v = i - (uint64_t)c * n_vec;
        const uint32_t ps = parent_slot[c];
        uint4 r = make_uint4(~0u, ~0u, ~0u, ~0u);
        if (ps != kNoSlot) r = *reinterpret_cast<const uint4 *>(arena + (uint64_t)ps * astride + 2 * v);
        for (uint64_t j = ptr[c]; j < ptr[c + 1]; ++j) r = and4(r, ld_nc_v4(rows + (uint64_t)items[j] * rstride + 2 * v));
        *reinterpret_cast<uint4 *>(arena + (uint64_t)child_slot[c] * astride + 2 * v) = r;
    }
}

void launch_child_masks(uint64_t *arena, uint64_t arena_stride, uint64_t n_words, const uint64_t *rows,
                        uint64_t row_stride, const uint64_t *ptr, const uint32_t *items, const uint32_t *parent_slot,
                        const uint32_t *child_slot, uint32_t n, cudaStream_t st, int n_sm) {
    if (n == 0) return;
    const uint64_t total = (uint64_t)n * (n_words / 2);
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)n_sm * 32);
    child_mask_kernel<<<blocks, 256, 0, st>>>(arena, arena_stride, n_words, rows, row_stride, ptr, items, parent_slot,
                                              child_slot, n);
    SG_CUDA_TRY(cudaGetLastError());
}

__global__ void pool_append_kernel(unsigned long long *__restrict__ pool, uint64_t pstride,
                                   const uint64_t *__restrict__ set_ptr, const uint32_t *__restrict__ set_items,
                                   uint64_t first, uint32_t n_sets, const uint64_t *__restrict__ set_col) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n_sets; s += gridDim.x * blockDim.x) {
        const uint64_t m = set_col ? set_col[s] : first + s;
        for (uint64_t i = set_ptr[s]; i < set_ptr[s + 1]; ++i)
            atomicOr(&pool[(uint64_t)set_items[i] * pstride + (m >> 6)], 1ull << (m & 63));
    }
}

void launch_pool_append(uint64_t *pool_rows, uint64_t pool_stride, const uint64_t *set_ptr, const uint32_t *set_items,
                        uint64_t first_member, uint32_t n_sets, cudaStream_t st, const uint64_t *set_col) {
    if (n_sets == 0) return;
    const unsigned blocks = std::min<unsigned>((n_sets + 255) / 256, 1024);
    pool_append_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<unsigned long long *>(pool_rows), pool_stride,
                                               set_ptr, set_items, first_member, n_sets, set_col);
    SG_CUDA_TRY(cudaGetLastError());
}

}  // namespace sg
