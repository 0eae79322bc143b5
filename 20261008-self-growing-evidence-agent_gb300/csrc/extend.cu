// extend.cu -- frequent single-item extensions of many itemsets (the maximality check).
//
// Reference counterpart: the maximality rule of mine_mfi
// (code/pipeline/skab_spike.py:129-135: a set is kept when no other frequent
// set contains it) and of the engines (code/engine_tensorfim/code/engine/src/
// kernel_bitmap.cu:870: a node is maximal when its number of frequent
// extensions equals its size).  Here the rule is evaluated for a batch of
// arbitrary itemsets S: which items e (not in S) have sup(S u {e}) >= t.
// An empty answer means S is maximal at t.
//
// Per batch of sets:
//   1. ext_bound_kernel (a warp per set): bound(e) = min over s in S of the
//      pairwise co-occurrence C[s][e] (an upper bound of sup(S u {e}), the
//      matrix computed once per dataset on the tensor cores); the items with
//      bound >= t, not in S, are listed per set in ascending row order.
//   2. ext_count_kernel (a CTA per set and group of 16 listed items): every
//      thread ANDs the set's rows word by word (the set's tidset is never
//      stored) and counts the AND with each listed item's row; a block
//      reduction gives the exact supports, and the frequent items set their
//      bit in the set's output mask (atomicOr).
// Both steps are exact: the bound only skips items whose support cannot reach t.
#include <algorithm>
#include <numeric>

#include "common.cuh"
#include "engine.h"

namespace sg {
namespace {

constexpr int kExtThreads = 256;
constexpr int kExtGroup = 16;   // listed items counted per CTA

// One warp per set.  list[s * d + j] (j < n_list[s]) = dense rows of the
// candidate extensions, ascending.
__global__ void ext_bound_kernel(const uint32_t *__restrict__ cooc, uint32_t d, const uint64_t *__restrict__ ptr,
                                 const uint32_t *__restrict__ rows, uint32_t n_sets, uint32_t thr,
                                 uint16_t *__restrict__ list, uint32_t *__restrict__ n_list) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n_sets) return;
    const uint64_t a = ptr[warp], b = ptr[warp + 1];
    uint32_t cnt = 0;
    for (uint32_t e0 = 0; e0 < d; e0 += 32) {
        const uint32_t e = e0 + lane;
        bool ok = e < d;
        if (ok) {
            uint32_t bound = cooc[(uint64_t)e * d + e];   // sup({e}): the bound of the empty set
            for (uint64_t i = a; i < b && bound >= thr; ++i) {
                const uint32_t s = rows[i];
                if (s >= d || s == e) {   // an absent item (support 0), or e already in S
                    bound = 0;
                    break;
                }
                bound = min(bound, cooc[(uint64_t)s * d + e]);
            }
            ok = bound >= thr;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, ok);
        if (ok) list[(uint64_t)warp * d + cnt + __popc(m & ((1u << lane) - 1))] = (uint16_t)e;
        cnt += __popc(m);
    }
    if (lane == 0) n_list[warp] = cnt;
}

// blockIdx.x = group of kExtGroup listed items, blockIdx.y = set.
__global__ void __launch_bounds__(kExtThreads) ext_count_kernel(
    const uint64_t *__restrict__ bm, uint64_t stride, uint64_t n_words, uint32_t d, const uint64_t *__restrict__ ptr,
    const uint32_t *__restrict__ rows, const uint16_t *__restrict__ list, const uint32_t *__restrict__ n_list,
    const uint32_t *__restrict__ d2o, uint32_t thr, unsigned long long *__restrict__ out, uint32_t out_words) {
    const uint32_t set = blockIdx.y, g0 = blockIdx.x * kExtGroup;
    const uint32_t nl = n_list[set];
    if (g0 >= nl) return;
    const uint32_t ng = min((uint32_t)kExtGroup, nl - g0);
    const uint64_t a = ptr[set], b = ptr[set + 1];
    __shared__ uint32_t part[kExtThreads / 32][kExtGroup];
    const uint64_t *ext[kExtGroup];
#pragma unroll
    for (int j = 0; j < kExtGroup; ++j)
        ext[j] = bm + (uint64_t)list[(uint64_t)set * d + g0 + min((uint32_t)j, ng - 1)] * stride;
    uint32_t acc[kExtGroup];
#pragma unroll
    for (int j = 0; j < kExtGroup; ++j) acc[j] = 0;
    for (uint64_t w = threadIdx.x; w < n_words; w += kExtThreads) {
        uint64_t m = ~0ull;
        for (uint64_t i = a; i < b; ++i) m &= __ldg(bm + (uint64_t)rows[i] * stride + w);
        if (m == 0) continue;
#pragma unroll
        for (int j = 0; j < kExtGroup; ++j)
            if ((uint32_t)j < ng) acc[j] += popc64(m & __ldg(ext[j] + w));
    }
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kExtGroup; ++j) {
        const uint32_t v = warp_sum(acc[j]);
        if (lane == 0) part[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < ng) {
        uint32_t s = 0;
        for (int w = 0; w < kExtThreads / 32; ++w) s += part[w][threadIdx.x];
        if (s >= thr) {
            const uint32_t id = d2o[list[(uint64_t)set * d + g0 + threadIdx.x]];
            atomicOr(out + (uint64_t)set * out_words + (id >> 6), 1ull << (id & 63));
        }
    }
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sgfim_frequent_extensions(sgfim_handle *h, const uint64_t *set_ptr, const uint32_t *set_items,
                                         uint64_t n_sets, uint32_t min_count, uint64_t *masks, uint32_t mask_words) {
    if (!h || (n_sets && (!set_ptr || !masks))) return fail(h, SGFIM_EINVAL, "null argument");
    if (!h->ds.loaded) return fail(h, SGFIM_ESTATE, "no dataset loaded");
    Dataset &ds = h->ds;
    if (mask_words < (ds.n_ids + 63) / 64) return fail(h, SGFIM_EINVAL, "mask_words below ceil(n_ids / 64)");
    if (n_sets == 0) return SGFIM_OK;
    if (set_ptr[0] != 0) return fail(h, SGFIM_EINVAL, "set_ptr[0] must be 0");
    for (uint64_t s = 0; s < n_sets; ++s)
        if (set_ptr[s + 1] < set_ptr[s]) return fail(h, SGFIM_EINVAL, "set_ptr must be non-decreasing");
    API_GUARD_BEGIN
    cudaSetDevice(h->device);
    std::fill(masks, masks + n_sets * mask_words, 0ull);
    const uint32_t d = ds.d;
    const uint32_t thr = std::max<uint32_t>(1, min_count);
    if (d == 0 || ds.n_txn == 0) return SGFIM_OK;
    cudaStream_t st = h->stream;
    // pairwise co-occurrence of the rows, once per dataset
    if (!ds.ext_cooc_ready) {
        ds.ext_cooc.reserve((size_t)d * d * 4, st);
        int rc = sgfim_cooccurrence_device(h, ds.bitmaps.as<uint64_t>(), d, ds.n_words, ds.stride,
                                           ds.ext_cooc.as<uint32_t>(), SGFIM_COOC_AUTO, st);
        if (rc) return rc;
        ds.ext_d2o.reserve((size_t)d * 4, st);
        SG_CUDA_TRY(cudaMemcpyAsync(ds.ext_d2o.ptr, ds.d2o.data(), (size_t)d * 4, cudaMemcpyHostToDevice, st));
        SG_CUDA_TRY(cudaStreamSynchronize(st));
        int drc = check_device_error(h);
        if (drc) return drc;
        ds.ext_cooc_ready = true;
    }
    // batches bounded by the candidate lists (d entries per set) and the output masks
    const uint64_t batch = std::max<uint64_t>(1, std::min<uint64_t>(32768, (256ull << 20) / ((uint64_t)d * 2 + 64)));
    ExtWorkspace &w = h->ext;
    w.list.reserve((size_t)batch * d * 2, st);
    w.n_list.reserve((size_t)batch * 4, st);
    w.out.reserve((size_t)batch * mask_words * 8, st);
    std::vector<uint64_t> bp;
    std::vector<uint32_t> br;
    for (uint64_t s0 = 0; s0 < n_sets; s0 += batch) {
        const uint64_t nb = std::min(batch, n_sets - s0);
        const uint64_t i0 = set_ptr[s0], i1 = set_ptr[s0 + nb];
        bp.resize(nb + 1);
        br.resize(std::max<uint64_t>(1, i1 - i0));
        for (uint64_t s = 0; s <= nb; ++s) bp[s] = set_ptr[s0 + s] - i0;
        for (uint64_t i = i0; i < i1; ++i) {
            const uint32_t id = set_items[i];
            const int32_t r = id < ds.o2d.size() ? ds.o2d[id] : -1;
            br[i - i0] = r < 0 ? 0xffffffffu : (uint32_t)r;   // absent: the kernels treat it as support 0
        }
        const uint64_t *d_ptr = w.ptr.put(bp.data(), nb + 1, st);
        const uint32_t *d_rows = w.rows.put(br.data(), br.size(), st);
        SG_CUDA_TRY(cudaMemsetAsync(w.out.ptr, 0, nb * mask_words * 8, st));
        const unsigned warps_per_block = 8;
        ext_bound_kernel<<<(unsigned)((nb + warps_per_block - 1) / warps_per_block), 32 * warps_per_block, 0, st>>>(
            ds.ext_cooc.as<uint32_t>(), d, d_ptr, d_rows, (uint32_t)nb, thr, w.list.as<uint16_t>(),
            w.n_list.as<uint32_t>());
        SG_CUDA_TRY(cudaGetLastError());
        dim3 grid((d + kExtGroup - 1) / kExtGroup, (unsigned)nb);
        ext_count_kernel<<<grid, kExtThreads, 0, st>>>(ds.bitmaps.as<uint64_t>(), ds.stride, ds.n_words, d, d_ptr,
                                                      d_rows, w.list.as<uint16_t>(), w.n_list.as<uint32_t>(),
                                                      ds.ext_d2o.as<uint32_t>(), thr,
                                                      w.out.as<unsigned long long>(), mask_words);
        SG_CUDA_TRY(cudaGetLastError());
        h->launches += 2;
        SG_CUDA_TRY(cudaMemcpyAsync(masks + s0 * mask_words, w.out.ptr, nb * mask_words * 8, cudaMemcpyDeviceToHost,
                                    st));
        SG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return check_device_error(h);
    API_GUARD_END(h)
}
