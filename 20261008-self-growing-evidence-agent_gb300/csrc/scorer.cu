// scorer.cu -- frontier-scoring MLP weights on the device (learned order).
//
// No reference counterpart: the reference orders its search by singleton
// support only (kernel_bitmap.cu:276-283).  The scorer ranks candidate
// extensions; it changes the order in which subtrees are searched, never the
// counts or the final MFI set.
#include <cstring>

#include "common.cuh"
#include "engine.h"

using namespace sg;

extern "C" int sgfim_load_scorer(sgfim_handle *h, uint32_t in_dim, uint32_t hidden, const uint16_t *w1_bf16,
                                 const float *b1, const uint16_t *w2_bf16, const float *b2, const uint16_t *w3_bf16,
                                 const float *b3) {
    if (!h || !w1_bf16 || !b1 || !w2_bf16 || !b2 || !w3_bf16 || !b3) return fail(h, SGFIM_EINVAL, "null argument");
    if (in_dim == 0 || in_dim > 64 || hidden == 0 || hidden > 256 || (hidden % 16) != 0)
        return fail(h, SGFIM_EINVAL, "scorer shape: in_dim 1..64, hidden a multiple of 16 up to 256");
    try {
        cudaSetDevice(h->device);
        Scorer &s = h->scorer;
        s.in_dim = in_dim;
        s.hidden = hidden;
        s.w1.reserve((size_t)hidden * in_dim * 2, h->stream);
        s.b1.reserve((size_t)hidden * 4, h->stream);
        s.w2.reserve((size_t)hidden * hidden * 2, h->stream);
        s.b2.reserve((size_t)hidden * 4, h->stream);
        s.w3.reserve((size_t)hidden * 2, h->stream);
        s.b3.reserve(4, h->stream);
        SG_CUDA_TRY(cudaMemcpyAsync(s.w1.ptr, w1_bf16, (size_t)hidden * in_dim * 2, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(s.b1.ptr, b1, (size_t)hidden * 4, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(s.w2.ptr, w2_bf16, (size_t)hidden * hidden * 2, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(s.b2.ptr, b2, (size_t)hidden * 4, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(s.w3.ptr, w3_bf16, (size_t)hidden * 2, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaMemcpyAsync(s.b3.ptr, b3, 4, cudaMemcpyHostToDevice, h->stream));
        SG_CUDA_TRY(cudaStreamSynchronize(h->stream));
        s.loaded = true;
        return SGFIM_OK;
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }
}
