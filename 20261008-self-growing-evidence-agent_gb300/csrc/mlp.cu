// mlp.cu -- the frontier-scoring MLP: fused forward, backward and Adam kernels.
//
// No reference counterpart (the reference orders its search by singleton
// support only, kernel_bitmap.cu:276-283).  Network: in_dim -> H -> H -> 1,
// ReLU, sigmoid output; weights are bf16 (row-major [out][in]), biases,
// activations and accumulation fp32.  Training keeps fp32 master weights
// and refreshes the bf16 copy after every Adam step.  The layers are small
// (H = 128): one CTA of H threads owns a tile of rows, thread j owns output
// column j, and the bf16 weights of layer 2 sit in shared memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "engine.h"

namespace sg {

constexpr int kMlpRows = 16;   // rows per CTA
constexpr int kMlpMaxIn = 64;

__device__ __forceinline__ float bf2f(uint16_t b) { return __uint_as_float(((uint32_t)b) << 16); }

// Forward.  Z1/Z2 (pre-activations) are written when non-null (training).
__global__ void mlp_fwd_kernel(const float *__restrict__ X, uint32_t n, uint32_t F, uint32_t H,
                               const uint16_t *__restrict__ W1, const float *__restrict__ b1,
                               const uint16_t *__restrict__ W2, const float *__restrict__ b2,
                               const uint16_t *__restrict__ w3, const float *__restrict__ b3, float *__restrict__ Z1,
                               float *__restrict__ Z2, float *__restrict__ P) {
    extern __shared__ float sm[];
    float *xs = sm;                               // [R][F]
    float *h1 = xs + kMlpRows * F;                // [R][H]
    uint16_t *w2t = reinterpret_cast<uint16_t *>(h1 + kMlpRows * H);  // [H(in)][H(out)]
    __shared__ float red[kMlpRows][8];
    const uint32_t j = threadIdx.x;
    const uint64_t r0 = (uint64_t)blockIdx.x * kMlpRows;
    for (uint32_t idx = j; idx < kMlpRows * F; idx += H) {
        const uint64_t r = r0 + idx / F;
        xs[idx] = r < n ? X[r * F + idx % F] : 0.f;
    }
    for (uint32_t idx = j; idx < H * H; idx += H) {
        const uint32_t o = idx / H, i = idx % H;   // W2[o][i] -> w2t[i][o]
        w2t[i * H + o] = W2[idx];
    }
    __syncthreads();
    // layer 1
    {
        float w[kMlpMaxIn];
#pragma unroll 8
        for (uint32_t i = 0; i < F; ++i) w[i] = bf2f(W1[j * F + i]);
        const float bj = b1[j];
        for (int r = 0; r < kMlpRows; ++r) {
            float z = bj;
            for (uint32_t i = 0; i < F; ++i) z = fmaf(w[i], xs[r * F + i], z);
            h1[r * H + j] = fmaxf(z, 0.f);
            if (Z1 && r0 + r < n) Z1[(r0 + r) * H + j] = z;
        }
    }
    __syncthreads();
    // layer 2
    float acc[kMlpRows];
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) acc[r] = 0.f;
    for (uint32_t i = 0; i < H; ++i) {
        const float w = bf2f(w2t[i * H + j]);
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) acc[r] = fmaf(w, h1[r * H + i], acc[r]);
    }
    const float bj2 = b2[j], wj3 = bf2f(w3[j]);
    const uint32_t lane = j & 31, warp = j >> 5;
#pragma unroll
    for (int r = 0; r < kMlpRows; ++r) {
        const float z = acc[r] + bj2;
        if (Z2 && r0 + r < n) Z2[(r0 + r) * H + j] = z;
        float v = wj3 * fmaxf(z, 0.f);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[r][warp] = v;
    }
    __syncthreads();
    if (j < kMlpRows && r0 + j < n) {
        float s = b3[0];
        for (uint32_t w = 0; w < H / 32; ++w) s += red[j][w];
        P[r0 + j] = 1.f / (1.f + expf(-s));
    }
}

// Backward of the mean (weighted) binary cross-entropy.  Gradients are
// accumulated with fp32 atomics into zeroed buffers; loss gets the summed
// weighted BCE.  scale = 1 / batch size.
__global__ void mlp_bwd_kernel(const float *__restrict__ X, uint32_t n, uint32_t F, uint32_t H,
                               const uint16_t *__restrict__ W2, const uint16_t *__restrict__ w3,
                               const float *__restrict__ Z1, const float *__restrict__ Z2,
                               const float *__restrict__ P, const float *__restrict__ Y,
                               const float *__restrict__ WT, float scale, float *__restrict__ dW1,
                               float *__restrict__ db1, float *__restrict__ dW2, float *__restrict__ db2,
                               float *__restrict__ dw3, float *__restrict__ db3, float *__restrict__ loss) {
    extern __shared__ float sm[];
    float *xs = sm;                              // [R][F]
    float *h1 = xs + kMlpRows * F;               // [R][H]
    float *dz2 = h1 + kMlpRows * H;              // [R][H]
    float *dz3 = dz2 + kMlpRows * H;             // [R]
    uint16_t *w2s = reinterpret_cast<uint16_t *>(dz3 + kMlpRows);  // [H(out)][H(in)]
    const uint32_t j = threadIdx.x;
    const uint64_t r0 = (uint64_t)blockIdx.x * kMlpRows;
    for (uint32_t idx = j; idx < kMlpRows * F; idx += H) {
        const uint64_t r = r0 + idx / F;
        xs[idx] = r < n ? X[r * F + idx % F] : 0.f;
    }
    for (uint32_t idx = j; idx < H * H; idx += H) w2s[idx] = W2[idx];
    if (j < kMlpRows) {
        const uint64_t r = r0 + j;
        float g = 0.f;
        if (r < n) {
            const float wt = WT ? WT[r] : 1.f;
            const float p = P[r], y = Y[r];
            g = scale * wt * (p - y);
            const float pc = fminf(fmaxf(p, 1e-7f), 1.f - 1e-7f);
            atomicAdd(loss, -scale * wt * (y * logf(pc) + (1.f - y) * logf(1.f - pc)));
        }
        dz3[j] = g;
    }
    __syncthreads();
    // layer 3 and the ReLU of layer 2
    {
        const float wj3 = bf2f(w3[j]);
        float gw3 = 0.f, gb2 = 0.f, gb3 = 0.f;
        for (int r = 0; r < kMlpRows; ++r) {
            const uint64_t row = r0 + r;
            float z2 = 0.f, z1 = 0.f;
            if (row < n) {
                z2 = Z2[row * H + j];
                z1 = Z1[row * H + j];
            }
            const float h2 = fmaxf(z2, 0.f);
            gw3 = fmaf(dz3[r], h2, gw3);
            gb3 += dz3[r];
            const float g2 = z2 > 0.f ? dz3[r] * wj3 : 0.f;
            dz2[r * H + j] = g2;
            gb2 += g2;
            h1[r * H + j] = fmaxf(z1, 0.f);
        }
        atomicAdd(&dw3[j], gw3);
        atomicAdd(&db2[j], gb2);
        if (j == 0) atomicAdd(db3, gb3);
    }
    __syncthreads();
    // dW2[j][i] = sum_r dz2[r][j] h1[r][i]
    {
        float g[kMlpRows];
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) g[r] = dz2[r * H + j];
        for (uint32_t i = 0; i < H; ++i) {
            float s = 0.f;
#pragma unroll
            for (int r = 0; r < kMlpRows; ++r) s = fmaf(g[r], h1[r * H + i], s);
            if (s != 0.f) atomicAdd(&dW2[j * H + i], s);
        }
    }
    // dh1[r][i] = sum_j dz2[r][j] W2[j][i]  (this thread plays i = j)
    {
        const uint32_t i = j;
        float acc[kMlpRows];
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) acc[r] = 0.f;
        for (uint32_t o = 0; o < H; ++o) {
            const float w = bf2f(w2s[o * H + i]);
#pragma unroll
            for (int r = 0; r < kMlpRows; ++r) acc[r] = fmaf(dz2[r * H + o], w, acc[r]);
        }
        float gb1 = 0.f;
        float gw[kMlpMaxIn];
        for (uint32_t f = 0; f < F; ++f) gw[f] = 0.f;
#pragma unroll
        for (int r = 0; r < kMlpRows; ++r) {
            const uint64_t row = r0 + r;
            const float z1 = row < n ? Z1[row * H + i] : 0.f;
            const float g1 = z1 > 0.f ? acc[r] : 0.f;
            gb1 += g1;
            for (uint32_t f = 0; f < F; ++f) gw[f] = fmaf(g1, xs[r * F + f], gw[f]);
        }
        atomicAdd(&db1[i], gb1);
        for (uint32_t f = 0; f < F; ++f)
            if (gw[f] != 0.f) atomicAdd(&dW1[i * F + f], gw[f]);
    }
}

// Adam on fp32 master weights; refreshes the bf16 copy (round to nearest even).
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, uint16_t *__restrict__ p16, uint32_t n, float lr, float beta1,
                            float beta2, float eps, float bc1, float bc2, float wd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * p[i];
        const float mi = beta1 * m[i] + (1.f - beta1) * gi;
        const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        p[i] = pi;
        if (p16) p16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(pi));
    }
}

size_t mlp_fwd_smem(uint32_t F, uint32_t H) { return (size_t)kMlpRows * (F + H) * 4 + (size_t)H * H * 2; }
size_t mlp_bwd_smem(uint32_t F, uint32_t H) {
    return (size_t)kMlpRows * (F + 2 * H + 1) * 4 + (size_t)H * H * 2;
}

void launch_mlp_forward(const float *X, uint32_t n, uint32_t F, uint32_t H, const uint16_t *W1, const float *b1,
                        const uint16_t *W2, const float *b2, const uint16_t *w3, const float *b3, float *Z1,
                        float *Z2, float *P, cudaStream_t st) {
    if (n == 0) return;
    const size_t smem = mlp_fwd_smem(F, H);
    SG_CUDA_TRY(cudaFuncSetAttribute(mlp_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mlp_fwd_kernel<<<(n + kMlpRows - 1) / kMlpRows, H, smem, st>>>(X, n, F, H, W1, b1, W2, b2, w3, b3, Z1, Z2, P);
    SG_CUDA_TRY(cudaGetLastError());
}

}  // namespace sg

using namespace sg;

namespace {
bool mlp_shape_ok(uint32_t F, uint32_t H) { return F >= 1 && F <= kMlpMaxIn && H >= 32 && H <= 256 && H % 32 == 0; }
}  // namespace

extern "C" {

int sgfim_mlp_forward(sgfim_handle *h, const float *X, uint32_t n, uint32_t in_dim, uint32_t hidden,
                      const uint16_t *W1, const float *b1, const uint16_t *W2, const float *b2, const uint16_t *w3,
                      const float *b3, float *Z1, float *Z2, float *P, void *stream) {
    if (!h || (n && (!X || !P)) || !W1 || !b1 || !W2 || !b2 || !w3 || !b3)
        return fail(h, SGFIM_EINVAL, "null argument");
    if (!mlp_shape_ok(in_dim, hidden)) return fail(h, SGFIM_EINVAL, "mlp shape: in_dim 1..64, hidden 32..256 step 32");
    try {
        cudaSetDevice(h->device);
        launch_mlp_forward(X, n, in_dim, hidden, W1, b1, W2, b2, w3, b3, Z1, Z2, P,
                           stream ? (cudaStream_t)stream : (cudaStream_t)0);
        h->launches++;
        return SGFIM_OK;
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }
}

int sgfim_mlp_backward(sgfim_handle *h, const float *X, uint32_t n, uint32_t in_dim, uint32_t hidden,
                       const uint16_t *W2, const uint16_t *w3, const float *Z1, const float *Z2, const float *P,
                       const float *Y, const float *WT, float scale, float *dW1, float *db1, float *dW2, float *db2,
                       float *dw3, float *db3, float *loss, void *stream) {
    if (!h || (n && (!X || !Z1 || !Z2 || !P || !Y)) || !W2 || !w3 || !dW1 || !db1 || !dW2 || !db2 || !dw3 || !db3 ||
        !loss)
        return fail(h, SGFIM_EINVAL, "null argument");
    if (!mlp_shape_ok(in_dim, hidden)) return fail(h, SGFIM_EINVAL, "mlp shape: in_dim 1..64, hidden 32..256 step 32");
    try {
        cudaSetDevice(h->device);
        if (n == 0) return SGFIM_OK;
        cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)0;
        const size_t smem = mlp_bwd_smem(in_dim, hidden);
        SG_CUDA_TRY(cudaFuncSetAttribute(mlp_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        mlp_bwd_kernel<<<(n + kMlpRows - 1) / kMlpRows, hidden, smem, st>>>(X, n, in_dim, hidden, W2, w3, Z1, Z2, P, Y,
                                                                           WT, scale, dW1, db1, dW2, db2, dw3, db3,
                                                                           loss);
        SG_CUDA_TRY(cudaGetLastError());
        h->launches++;
        return SGFIM_OK;
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }
}

int sgfim_adam_step(sgfim_handle *h, float *param, const float *grad, float *m, float *v, uint16_t *param_bf16,
                    uint32_t n, float lr, float beta1, float beta2, float eps, uint32_t step, float weight_decay,
                    void *stream) {
    if (!h || !param || !grad || !m || !v || step == 0) return fail(h, SGFIM_EINVAL, "bad argument");
    try {
        cudaSetDevice(h->device);
        const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
        const unsigned blocks = std::min<unsigned>((n + 255) / 256, 1024);
        adam_kernel<<<blocks ? blocks : 1, 256, 0, stream ? (cudaStream_t)stream : (cudaStream_t)0>>>(
            param, grad, m, v, param_bf16, n, lr, beta1, beta2, eps, bc1, bc2, weight_decay);
        SG_CUDA_TRY(cudaGetLastError());
        h->launches++;
        return SGFIM_OK;
    } catch (const CudaError &e) {
        return fail(h, SGFIM_EDEVICE, e.what);
    }
}

}  // extern "C"
