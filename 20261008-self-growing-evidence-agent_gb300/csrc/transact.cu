// transact.cu -- sensor stream -> transactions on the GPU.
//
// Reference: code/pipeline/skab_spike.py
//   fit_bins            :38-52  per-sensor quantiles at linspace(0, 1, n_bins+1)
//                               (numpy "linear" method), unique edges, a
//                               constant column gets [e0 - 0.5, e0 + 0.5]
//   bin_index           :55-58  searchsorted(edges, v, side="right") - 1, clamped
//   window_transactions :62-80  windows s = 0, stride, ..., s + window <= n; the
//                               median of each sensor over the window picks one
//                               item per sensor; the label is the window's max
// Items are dense ids sensor * n_bins + bin.
//
// Device work: the row-major [n, S] matrix is transposed to columns; every
// order statistic numpy's quantile needs is found exactly by an 8-pass MSD
// radix select over order-preserving 64-bit keys of the doubles (one CTA per
// sensor x rank); the quantile interpolation runs in explicitly rounded
// double intrinsics, so no multiply-add is fused and the edges are the same
// doubles numpy computes; one thread per (window, sensor) sorts its window
// and bins the median.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "engine.h"

namespace sg {

namespace {

constexpr uint32_t kMaxWindow = 256;

__device__ __forceinline__ uint64_t dkey(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | (1ull << 63));
}
__device__ __forceinline__ double dkey_inv(uint64_t k) {
    const uint64_t b = (k >> 63) ? (k & ~(1ull << 63)) : ~k;
    return __longlong_as_double((long long)b);
}

__global__ void to_columns_kernel(const double *__restrict__ rows, uint64_t n, uint32_t S, double *__restrict__ cols,
                                  uint32_t *__restrict__ nan_count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n * S; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / S;
        const uint32_t c = (uint32_t)(i - r * S);
        const double v = rows[i];
        if (v != v) atomicAdd(nan_count, 1u);
        cols[(uint64_t)c * n + r] = v;
    }
}

// k-th smallest (0-based) of column blockIdx.y for rank ranks[blockIdx.y * R + blockIdx.x]
__global__ void __launch_bounds__(512) kth_kernel(const double *__restrict__ cols, uint64_t n, const uint64_t *__restrict__ ranks,
                                                  uint32_t R, double *__restrict__ out) {
    __shared__ uint32_t hist[256];
    __shared__ uint64_t s_prefix, s_mask, s_k;
    const uint32_t s = blockIdx.y, r = blockIdx.x;
    const double *col = cols + (uint64_t)s * n;
    if (threadIdx.x == 0) {
        s_prefix = 0;
        s_mask = 0;
        s_k = ranks[(uint64_t)s * R + r];
    }
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const uint64_t prefix = s_prefix, mask = s_mask;
        for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
            const uint64_t key = dkey(col[i]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t k = s_k, cum = 0;
            uint32_t dgt = 255;
            for (uint32_t d = 0; d < 256; ++d) {
                if (k < cum + hist[d]) {
                    dgt = d;
                    break;
                }
                cum += hist[d];
            }
            s_prefix = prefix | ((uint64_t)dgt << shift);
            s_mask = mask | (255ull << shift);
            s_k = k - cum;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[(uint64_t)s * R + r] = dkey_inv(s_prefix);
}

// numpy linear quantile for quantile q of sensor s: lo/hi are the order
// statistics at floor(h) and floor(h)+1 (both the last one when h >= n-1),
// gamma = h - floor(h) (h - (-1) above the bounds, where lo == hi), and
// lerp(a, b, g) = g >= 0.5 ? b - (b - a) * (1 - g) : a + (b - a) * g.
__global__ void quantile_kernel(const double *__restrict__ stats, uint32_t R, const uint32_t *__restrict__ lo_idx,
                                const uint32_t *__restrict__ hi_idx, const double *__restrict__ gamma, uint32_t nq,
                                uint32_t S, double *__restrict__ edges) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq * S) return;
    const uint32_t s = i / nq, q = i - s * nq;
    const double a = stats[(uint64_t)s * R + lo_idx[q]];
    const double b = stats[(uint64_t)s * R + hi_idx[q]];
    const double g = gamma[q];
    const double diff = __dsub_rn(b, a);
    double v = __dadd_rn(a, __dmul_rn(diff, g));
    if (g >= 0.5) v = __dsub_rn(b, __dmul_rn(diff, __dsub_rn(1.0, g)));
    edges[i] = v;
}

// numpy's median of `window` values `step` elements apart (insertion sort while
// loading; the mean of the two middle values for an even count).
__device__ __forceinline__ double window_median(const double *__restrict__ col, uint32_t window, uint64_t step = 1) {
    double buf[kMaxWindow];
    for (uint32_t j = 0; j < window; ++j) {
        const double v = col[j * step];
        uint32_t k = j;
        while (k > 0 && buf[k - 1] > v) {
            buf[k] = buf[k - 1];
            --k;
        }
        buf[k] = v;
    }
    return (window & 1) ? buf[window / 2] : __ddiv_rn(__dadd_rn(buf[window / 2 - 1], buf[window / 2]), 2.0);
}

// One thread per (window, sensor): median of the window's values, binned.
__global__ void window_bin_kernel(const double *__restrict__ cols, uint64_t n, uint32_t S, uint32_t window,
                                  uint32_t stride, uint64_t n_win, const double *__restrict__ edges,
                                  const uint32_t *__restrict__ n_edges, uint32_t edge_stride, uint32_t n_bins,
                                  const int32_t *__restrict__ anomaly, uint32_t *__restrict__ items,
                                  int32_t *__restrict__ labels) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_win * S) return;
    const uint64_t w = i / S;
    const uint32_t s = (uint32_t)(i - w * S);
    const uint64_t start = w * stride;
    const double med = window_median(cols + (uint64_t)s * n + start, window);
    const double *e = edges + (uint64_t)s * edge_stride;
    const uint32_t m = n_edges[s];
    uint32_t cnt = 0;   // edges <= med (searchsorted side="right")
    for (uint32_t j = 0; j < m; ++j) cnt += e[j] <= med;
    int32_t b = (int32_t)cnt - 1;
    if (b < 0) b = 0;
    if (b > (int32_t)m - 2) b = (int32_t)m - 2;
    items[w * S + s] = s * n_bins + (uint32_t)b;
    if (s == 0) {
        int32_t mx = 0;
        if (anomaly) {
            mx = anomaly[start];
            for (uint32_t j = 1; j < window; ++j) mx = max(mx, anomaly[start + j]);
        }
        labels[w] = mx;
    }
}

// ---------------------------------------------------------------- online (P²) edges
//
// code/pipeline/online_discretize.py: every sensor keeps n_bins-1 five-marker
// estimators (P2Quantile :22-71) at quantiles i/n_bins; run_file (:111-128)
// feeds every row of every window, in window order, to every estimator (rows
// shared by overlapping windows are fed again) and after each window bins the
// window median with the edges of that moment (OnlineBinner.edges :87-103).
// An estimator is a sequential recurrence, so the parallel axis is the chain
// (sensor, estimator).  A warp carries `lanes` chains (1..32): few chains run
// one to a warp, so that every chain has a scheduler's double pipe to itself;
// many chains share a warp.  All arithmetic is explicitly rounded (no fused
// multiply-add), in the reference's order, so the estimates are the
// reference's bit for bit.
//
// When the estimate stops changing.  The reference's value() is the middle
// marker qv[2], and its marker rule can never move markers 2 and 3 for most
// quantiles.  With gap_i = n[i+1] - n[i], the setup gives gaps (1+2q, 2q,
// 2-2q, 1-2q); a sample in cell k adds 1 to every position and 1 more to
// positions 1..k, so gap_0 grows by [k >= 1] and gap_i (i = 1..3) shrinks by
// [k == i] -- gaps 1..3 never grow.  Marker i is tested only when d = gap_{i-1}
// >= 1 and span = gap_{i-1} + gap_i > 1, and a move needs qv[i] + qp < qv[i+1]
// with qp = (d+1) (qv[i+1] - qv[i-1]) / span >= (d+1)/span (qv[i+1] - qv[i]),
// so it needs (d+1)/span < 1, i.e. gap_i > 1.  Marker 3 needs gap_3 = 1-2q > 1:
// never.  Marker 2 needs gap_1 = 2q >= 1 and gap_2 = 2-2q > 1: never for
// q != 1/2.  With q = j/n_bins and n_bins <= 64 both inequalities miss by at
// least 1/64, far beyond the rounding of the positions and of qp.  So for q !=
// 1/2 the estimate is fixed at the setup (the third smallest of the first five
// samples).  For q = 1/2 the positions are integers and marker 2 can be tested
// only while no sample fell in cell 1 or 2 (gap_1 = gap_2 = 1), or never when
// qv[1] = qv[2] = qv[3] (qp = 0).  The kernel runs the recurrence until its
// chain reaches such a state and then writes the fixed estimate for every
// remaining window; `full` turns the shortcut off (the tests compare both).

constexpr uint32_t kMaxOnlineBins = 64;

// stable insertion sort of five registers (Python's sorted on equal keys)
__device__ __forceinline__ void sort5(double (&a)[5]) {
#pragma unroll
    for (int i = 1; i < 5; ++i)
#pragma unroll
        for (int j = i; j > 0; --j)
            if (a[j - 1] > a[j]) {
                const double t = a[j - 1];
                a[j - 1] = a[j];
                a[j] = t;
            }
}

__global__ void nan_count_kernel(const double *__restrict__ v, uint64_t n, uint32_t *__restrict__ nan_count) {
    uint32_t c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        c += v[i] != v[i];
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(nan_count, c);
}

// est[(w * S + s) * m + j] = estimate j of sensor s after window w; chain c =
// s * m + j reads rows[t * S + s] (row-major values: neighbouring lanes read
// neighbouring sensors).
__global__ void __launch_bounds__(128) p2_kernel(const double *__restrict__ rows, uint32_t S, uint32_t m,
                                                 const double *__restrict__ quant, uint32_t window, uint32_t stride,
                                                 uint64_t n_win, uint32_t lanes, uint32_t full,
                                                 double *__restrict__ est) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t c = ((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) * lanes + lane;
    if (lane >= lanes || c >= (uint64_t)S * m) return;
    const uint32_t s = (uint32_t)(c / m), j = (uint32_t)(c - (uint64_t)s * m);
    const double q = quant[j];
    const bool half = q == 0.5;
    const uint64_t chains = (uint64_t)S * m;
    double qv[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double np_[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    uint32_t n_init = 0;   // the same for every chain: all see the same rows
    bool fixed = false;
    uint64_t w = 0;
    for (; w < n_win && !fixed; ++w) {
        const double *x_ptr = rows + w * stride * S + s;
        for (uint32_t t = 0; t < window; ++t) {
            const double x = x_ptr[(uint64_t)t * S];
            if (n_init < 5) {
#pragma unroll
                for (int i = 0; i < 5; ++i)
                    if ((uint32_t)i == n_init) qv[i] = x;
                if (++n_init == 5) {
                    sort5(qv);
                    np_[0] = 0.0;
                    np_[1] = __dadd_rn(1.0, __dmul_rn(2.0, q));
                    np_[2] = __dadd_rn(1.0, __dmul_rn(4.0, q));
                    np_[3] = __dadd_rn(3.0, __dmul_rn(2.0, q));
                    np_[4] = 4.0;
                    if (!full && (!half || (qv[1] == qv[2] && qv[2] == qv[3]))) {
                        fixed = true;
                        break;
                    }
                }
                continue;
            }
            int k;
            if (x < qv[0]) {
                qv[0] = x;
                k = 0;
            } else if (x < qv[1]) {
                k = 0;
            } else if (x < qv[2]) {
                k = 1;
            } else if (x < qv[3]) {
                k = 2;
            } else if (x <= qv[4]) {
                k = 3;
            } else {
                qv[4] = x;
                k = 3;
            }
#pragma unroll
            for (int i = 0; i < 5; ++i) np_[i] = __dadd_rn(np_[i], 1.0);
#pragma unroll
            for (int i = 1; i < 4; ++i)
                if (i <= k) np_[i] = __dadd_rn(np_[i], 1.0);
#pragma unroll
            for (int i = 1; i < 4; ++i) {
                const double d = __dsub_rn(np_[i], np_[i - 1]);
                const double span = __dsub_rn(np_[i + 1], np_[i - 1]);
                if (d >= 1.0 && span > 1.0) {
                    const double qp = __ddiv_rn(__dmul_rn(__dadd_rn(d, 1.0), __dsub_rn(qv[i + 1], qv[i - 1])), span);
                    const double moved = __dadd_rn(qv[i], qp);
                    if (qv[i - 1] < moved && moved < qv[i + 1]) qv[i] = moved;
                }
            }
            // q = 1/2: once a sample fell in cell 1 or 2, marker 2 is never tested again
            if (!full && (k == 1 || k == 2)) {
                fixed = true;
                break;
            }
        }
        double v;
        if (n_init >= 5) {
            v = qv[2];
        } else {
            // fewer than five samples: numpy's median of them (unused slots sort last)
            double a[5];
#pragma unroll
            for (int i = 0; i < 5; ++i) a[i] = (uint32_t)i < n_init ? qv[i] : __longlong_as_double(0x7ff0000000000000ll);
            sort5(a);
            v = a[0];
#pragma unroll
            for (int i = 1; i < 5; ++i)
                if ((uint32_t)i == n_init / 2) v = (n_init & 1) ? a[i] : __ddiv_rn(__dadd_rn(a[i - 1], a[i]), 2.0);
        }
        est[w * chains + c] = v;
    }
    // the estimate no longer changes: every remaining window gets it
    for (; w < n_win; ++w) est[w * chains + c] = qv[2];
}

// One thread per (window, sensor): edges from the sensor's estimates after the
// window, then the window median binned with them.
__global__ void online_bin_kernel(const double *__restrict__ rows, uint32_t S, uint32_t window, uint32_t stride,
                                  uint64_t n_win, const double *__restrict__ est, uint32_t n_bins,
                                  const int32_t *__restrict__ anomaly, double *__restrict__ edges,
                                  uint32_t *__restrict__ items, int32_t *__restrict__ labels) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_win * S) return;
    const uint64_t w = i / S;
    const uint32_t s = (uint32_t)(i - w * S);
    const uint32_t m = n_bins - 1;
    double q[kMaxOnlineBins - 1];
    const double *src = est + i * m;
    for (uint32_t j = 0; j < m; ++j) {
        const double v = src[j];
        uint32_t k = j;
        while (k > 0 && q[k - 1] > v) {
            q[k] = q[k - 1];
            --k;
        }
        q[k] = v;
    }
    double span = __dsub_rn(q[m - 1], q[0]);
    if (1e-9 > span) span = 1e-9;   // max(q[-1] - q[0], 1e-9)
    const double min_gap = __dmul_rn(0.05, span);
    if (n_bins == 3) {
        if (__dsub_rn(q[1], q[0]) < min_gap) {
            const double mid = __ddiv_rn(__dadd_rn(q[0], q[1]), 2.0);
            const double half = __ddiv_rn(min_gap, 2.0);
            q[0] = __dsub_rn(mid, half);
            q[1] = __dadd_rn(mid, half);
        }
    } else {
        for (uint32_t j = 1; j < m; ++j) {
            const double lo = __dadd_rn(q[j - 1], min_gap);
            if (q[j] < lo) q[j] = lo;
        }
    }
    double *e = edges + i * (n_bins + 1);
    e[0] = __dsub_rn(q[0], span);
    for (uint32_t j = 0; j < m; ++j) e[1 + j] = q[j];
    e[n_bins] = __dadd_rn(q[m - 1], span);
    const uint64_t start = w * stride;
    const double med = window_median(rows + start * S + s, window, S);
    uint32_t cnt = 0;   // edges <= med (searchsorted side="right")
    for (uint32_t j = 0; j <= n_bins; ++j) cnt += e[j] <= med;
    int32_t b = (int32_t)cnt - 1;
    if (b < 0) b = 0;
    if (b > (int32_t)n_bins - 1) b = (int32_t)n_bins - 1;
    items[i] = s * n_bins + (uint32_t)b;
    if (s == 0) {
        int32_t mx = 0;
        if (anomaly) {
            mx = anomaly[start];
            for (uint32_t j = 1; j < window; ++j) mx = max(mx, anomaly[start + j]);
        }
        labels[w] = mx;
    }
}

}  // namespace

}  // namespace sg

using namespace sg;

extern "C" int sgfim_transactionize_online(sgfim_handle *h, const double *values, uint64_t n_rows,
                                           uint32_t n_sensors, const int32_t *anomaly, uint32_t window,
                                           uint32_t stride, uint32_t n_bins, uint32_t flags, double *edges_out,
                                           uint32_t *items_out, int32_t *labels_out, uint64_t *n_windows_out) {
    if (!h) return SGFIM_EINVAL;
    if (!values && n_rows) return fail(h, SGFIM_EINVAL, "null values");
    if (n_sensors == 0 || window < 1 || stride < 1)
        return fail(h, SGFIM_EINVAL, "n_sensors, window and stride must be >= 1");
    if (n_bins < 2 || n_bins > kMaxOnlineBins) return fail(h, SGFIM_EINVAL, "n_bins must be in 2..64");
    if (window > kMaxWindow) return fail(h, SGFIM_EINVAL, "window longer than 256 rows");
    if ((uint64_t)n_sensors * n_bins > 0xffffffffull) return fail(h, SGFIM_EINVAL, "too many items");
    const uint64_t n_win = n_rows >= window ? (n_rows - window) / stride + 1 : 0;
    if (n_windows_out) *n_windows_out = n_win;
    if (n_win && (!items_out || !labels_out)) return fail(h, SGFIM_EINVAL, "null output");
    if ((n_win * n_sensors + 127) / 128 > 0x7fffffffull) return fail(h, SGFIM_EINVAL, "too many windows");
    API_GUARD_BEGIN
    SG_CUDA_TRY(cudaSetDevice(h->device));
    cudaStream_t st = h->stream;
    const uint32_t S = n_sensors, m = n_bins - 1;
    DevBuf d_rows, d_est, d_out, d_anom;
    struct Free {
        DevBuf *b[4];
        ~Free() {
            for (DevBuf *x : b) x->release();
        }
    } guard{{&d_rows, &d_est, &d_out, &d_anom}};
    if (n_win) {
        const size_t mat = (size_t)n_rows * S * 8;
        d_rows.reserve(mat, st);
        // out: nan count | quantiles | labels | items | edges
        size_t off = 0;
        auto carve = [&](size_t bytes) {
            const size_t o = off;
            off += (bytes + 255) & ~(size_t)255;
            return o;
        };
        const size_t o_nan = carve(4), o_q = carve((size_t)m * 8), o_lab = carve(n_win * 4),
                     o_items = carve(n_win * S * 4), o_edges = carve(n_win * S * (n_bins + 1) * 8);
        d_out.reserve(off, st);
        d_est.reserve(n_win * S * m * 8, st);
        char *base = d_out.as<char>();
        std::vector<double> quant(m);
        for (uint32_t j = 0; j < m; ++j) quant[j] = (double)(j + 1) / (double)n_bins;   // i / n_bins
        SG_CUDA_TRY(cudaMemcpyAsync(d_rows.ptr, values, mat, cudaMemcpyHostToDevice, st));
        SG_CUDA_TRY(cudaMemsetAsync(base + o_nan, 0, 4, st));
        SG_CUDA_TRY(cudaMemcpyAsync(base + o_q, quant.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st));
        const uint64_t total = n_rows * S;
        nan_count_kernel<<<(unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)h->n_sm * 8), 256, 0, st>>>(
            d_rows.as<double>(), total, reinterpret_cast<uint32_t *>(base + o_nan));
        SG_CUDA_TRY(cudaGetLastError());
        uint32_t nan_count = 0;
        SG_CUDA_TRY(cudaMemcpyAsync(&nan_count, base + o_nan, 4, cudaMemcpyDeviceToHost, st));
        SG_CUDA_TRY(cudaStreamSynchronize(st));
        if (nan_count) return fail(h, SGFIM_EINVAL, "the stream holds NaN values");
        // chains per warp: one while there are fewer chains than schedulers, then
        // as many as it takes to keep the warp count at about one per scheduler
        const uint64_t chains = (uint64_t)S * m;
        const uint64_t sched = (uint64_t)h->n_sm * 4;
        uint32_t lanes = (flags >> 8) & 63u;
        if (lanes == 0) lanes = (uint32_t)std::min<uint64_t>(32, std::max<uint64_t>(1, (chains + sched - 1) / sched));
        if (lanes > 32) return fail(h, SGFIM_EINVAL, "more than 32 chains per warp");
        const uint64_t warps = (chains + lanes - 1) / lanes;
        p2_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, st>>>(d_rows.as<double>(), S, m,
                                                              reinterpret_cast<const double *>(base + o_q), window,
                                                              stride, n_win, lanes, (flags & SGFIM_TX_P2_FULL) ? 1u : 0u,
                                                              d_est.as<double>());
        SG_CUDA_TRY(cudaGetLastError());
        if (anomaly) {
            d_anom.reserve(n_rows * 4, st);
            SG_CUDA_TRY(cudaMemcpyAsync(d_anom.ptr, anomaly, n_rows * 4, cudaMemcpyHostToDevice, st));
        }
        const uint64_t nt = n_win * S;
        online_bin_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(
            d_rows.as<double>(), S, window, stride, n_win, d_est.as<double>(), n_bins,
            anomaly ? d_anom.as<int32_t>() : nullptr, reinterpret_cast<double *>(base + o_edges),
            reinterpret_cast<uint32_t *>(base + o_items), reinterpret_cast<int32_t *>(base + o_lab));
        SG_CUDA_TRY(cudaGetLastError());
        h->launches += 3;
        SG_CUDA_TRY(cudaMemcpyAsync(items_out, base + o_items, nt * 4, cudaMemcpyDeviceToHost, st));
        SG_CUDA_TRY(cudaMemcpyAsync(labels_out, base + o_lab, n_win * 4, cudaMemcpyDeviceToHost, st));
        if (edges_out)
            SG_CUDA_TRY(cudaMemcpyAsync(edges_out, base + o_edges, nt * (n_bins + 1) * 8, cudaMemcpyDeviceToHost, st));
        SG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (flags & SGFIM_TX_LOAD) {
        std::vector<uint64_t> rp(n_win + 1);
        for (uint64_t w = 0; w <= n_win; ++w) rp[w] = w * S;
        return sgfim_load_csr(h, rp.data(), items_out, n_win);
    }
    return SGFIM_OK;
    API_GUARD_END(h)
}

extern "C" int sgfim_transactionize(sgfim_handle *h, const double *values, uint64_t n_rows, uint32_t n_sensors,
                                    const int32_t *anomaly, uint32_t window, uint32_t stride, uint32_t n_bins,
                                    uint32_t flags, double *edges_out, uint32_t *n_edges_out, uint32_t *items_out,
                                    int32_t *labels_out, uint64_t *n_windows_out) {
    if (!h) return SGFIM_EINVAL;
    if (!values && n_rows) return fail(h, SGFIM_EINVAL, "null values");
    if (n_sensors == 0 || n_bins < 1 || window < 1 || stride < 1)
        return fail(h, SGFIM_EINVAL, "n_sensors, n_bins, window and stride must be >= 1");
    if (window > kMaxWindow) return fail(h, SGFIM_EINVAL, "window longer than 256 rows");
    if (n_rows == 0) return fail(h, SGFIM_EINVAL, "empty stream");
    if ((uint64_t)n_sensors * n_bins > 0xffffffffull) return fail(h, SGFIM_EINVAL, "too many items");
    const uint64_t n_win = n_rows >= window ? (n_rows - window) / stride + 1 : 0;
    if (n_windows_out) *n_windows_out = n_win;
    if (!edges_out || !n_edges_out || (n_win && (!items_out || !labels_out)))
        return fail(h, SGFIM_EINVAL, "null output");
    API_GUARD_BEGIN
    SG_CUDA_TRY(cudaSetDevice(h->device));
    cudaStream_t st = h->stream;
    const uint32_t S = n_sensors, nq = n_bins + 1;
    // quantile positions exactly as numpy computes them
    std::vector<double> q(nq), gamma(nq);
    const double step = 1.0 / (double)n_bins;
    for (uint32_t i = 0; i < nq; ++i) q[i] = (double)i * step + 0.0;
    q[nq - 1] = 1.0;
    std::vector<uint64_t> need;   // order statistics
    std::vector<uint32_t> lo_pos(nq), hi_pos(nq);
    std::vector<uint64_t> lo_rank(nq), hi_rank(nq);
    const double nm1 = (double)(n_rows - 1);
    for (uint32_t i = 0; i < nq; ++i) {
        volatile double h_ = nm1 * q[i];   // one rounding, as numpy's (n - 1) * quantiles
        const double hv = h_;
        double prev = std::floor(hv);
        uint64_t lo, hi;
        if (hv >= nm1) {
            lo = hi = n_rows - 1;
            prev = -1.0;
        } else {
            lo = (uint64_t)prev;
            hi = lo + 1;
        }
        volatile double g_ = hv - prev;
        gamma[i] = g_;
        lo_rank[i] = lo;
        hi_rank[i] = hi;
        need.push_back(lo);
        need.push_back(hi);
    }
    std::sort(need.begin(), need.end());
    need.erase(std::unique(need.begin(), need.end()), need.end());
    for (uint32_t i = 0; i < nq; ++i) {
        lo_pos[i] = (uint32_t)(std::lower_bound(need.begin(), need.end(), lo_rank[i]) - need.begin());
        hi_pos[i] = (uint32_t)(std::lower_bound(need.begin(), need.end(), hi_rank[i]) - need.begin());
    }
    const uint32_t R = (uint32_t)need.size();
    std::vector<uint64_t> ranks((size_t)S * R);
    for (uint32_t s = 0; s < S; ++s)
        for (uint32_t r = 0; r < R; ++r) ranks[(size_t)s * R + r] = need[r];

    DevBuf d_rows, d_cols, d_small, d_anom, d_items;
    struct Free {
        DevBuf *b[5];
        ~Free() {
            for (DevBuf *x : b) x->release();
        }
    } guard{{&d_rows, &d_cols, &d_small, &d_anom, &d_items}};
    const size_t mat = (size_t)n_rows * S * 8;
    d_rows.reserve(mat, st);
    d_cols.reserve(mat, st);
    // small buffers: nan count | ranks | stats | lo | hi | gamma | edges | n_edges | labels
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t o_nan = carve(4), o_rank = carve(ranks.size() * 8), o_stat = carve(ranks.size() * 8),
                 o_lo = carve(nq * 4), o_hi = carve(nq * 4), o_g = carve(nq * 8), o_edge = carve((size_t)S * nq * 8),
                 o_ne = carve((size_t)S * 4), o_lab = carve(std::max<uint64_t>(n_win, 1) * 4);
    d_small.reserve(off, st);
    char *base = d_small.as<char>();
    SG_CUDA_TRY(cudaMemcpyAsync(d_rows.ptr, values, mat, cudaMemcpyHostToDevice, st));
    SG_CUDA_TRY(cudaMemsetAsync(base + o_nan, 0, 4, st));
    SG_CUDA_TRY(cudaMemcpyAsync(base + o_rank, ranks.data(), ranks.size() * 8, cudaMemcpyHostToDevice, st));
    SG_CUDA_TRY(cudaMemcpyAsync(base + o_lo, lo_pos.data(), nq * 4, cudaMemcpyHostToDevice, st));
    SG_CUDA_TRY(cudaMemcpyAsync(base + o_hi, hi_pos.data(), nq * 4, cudaMemcpyHostToDevice, st));
    SG_CUDA_TRY(cudaMemcpyAsync(base + o_g, gamma.data(), nq * 8, cudaMemcpyHostToDevice, st));
    const uint64_t total = n_rows * S;
    to_columns_kernel<<<(unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)h->n_sm * 32), 256, 0, st>>>(
        d_rows.as<double>(), n_rows, S, d_cols.as<double>(), reinterpret_cast<uint32_t *>(base + o_nan));
    SG_CUDA_TRY(cudaGetLastError());
    kth_kernel<<<dim3(R, S), 512, 0, st>>>(d_cols.as<double>(), n_rows, reinterpret_cast<const uint64_t *>(base + o_rank),
                                           R, reinterpret_cast<double *>(base + o_stat));
    SG_CUDA_TRY(cudaGetLastError());
    quantile_kernel<<<(S * nq + 127) / 128, 128, 0, st>>>(
        reinterpret_cast<const double *>(base + o_stat), R, reinterpret_cast<const uint32_t *>(base + o_lo),
        reinterpret_cast<const uint32_t *>(base + o_hi), reinterpret_cast<const double *>(base + o_g), nq, S,
        reinterpret_cast<double *>(base + o_edge));
    SG_CUDA_TRY(cudaGetLastError());
    h->launches += 3;
    uint32_t nan_count = 0;
    std::vector<double> raw((size_t)S * nq);
    SG_CUDA_TRY(cudaMemcpyAsync(&nan_count, base + o_nan, 4, cudaMemcpyDeviceToHost, st));
    SG_CUDA_TRY(cudaMemcpyAsync(raw.data(), base + o_edge, raw.size() * 8, cudaMemcpyDeviceToHost, st));
    SG_CUDA_TRY(cudaStreamSynchronize(st));
    if (nan_count) return fail(h, SGFIM_EINVAL, "the stream holds NaN values");
    // np.unique of each sensor's quantiles (already ascending), constant column rule
    std::vector<double> edges((size_t)S * nq, 0.0);
    std::vector<uint32_t> n_edges(S);
    for (uint32_t s = 0; s < S; ++s) {
        std::vector<double> e(raw.begin() + (size_t)s * nq, raw.begin() + (size_t)(s + 1) * nq);
        std::stable_sort(e.begin(), e.end());
        std::vector<double> u;
        for (double x : e)
            if (u.empty() || !(x == u.back())) u.push_back(x);
        if (u.size() < 2) u = {u[0] - 0.5, u[0] + 0.5};
        n_edges[s] = (uint32_t)u.size();
        std::copy(u.begin(), u.end(), edges.begin() + (size_t)s * nq);
    }
    memcpy(edges_out, edges.data(), edges.size() * 8);
    memcpy(n_edges_out, n_edges.data(), (size_t)S * 4);
    if (n_win) {
        SG_CUDA_TRY(cudaMemcpyAsync(base + o_edge, edges.data(), edges.size() * 8, cudaMemcpyHostToDevice, st));
        SG_CUDA_TRY(cudaMemcpyAsync(base + o_ne, n_edges.data(), (size_t)S * 4, cudaMemcpyHostToDevice, st));
        if (anomaly) {
            d_anom.reserve(n_rows * 4, st);
            SG_CUDA_TRY(cudaMemcpyAsync(d_anom.ptr, anomaly, n_rows * 4, cudaMemcpyHostToDevice, st));
        }
        d_items.reserve(n_win * S * 4, st);
        const uint64_t nt = n_win * S;
        window_bin_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(
            d_cols.as<double>(), n_rows, S, window, stride, n_win, reinterpret_cast<const double *>(base + o_edge),
            reinterpret_cast<const uint32_t *>(base + o_ne), nq, n_bins, anomaly ? d_anom.as<int32_t>() : nullptr,
            d_items.as<uint32_t>(), reinterpret_cast<int32_t *>(base + o_lab));
        SG_CUDA_TRY(cudaGetLastError());
        h->launches += 1;
        SG_CUDA_TRY(cudaMemcpyAsync(items_out, d_items.ptr, nt * 4, cudaMemcpyDeviceToHost, st));
        SG_CUDA_TRY(cudaMemcpyAsync(labels_out, base + o_lab, n_win * 4, cudaMemcpyDeviceToHost, st));
        SG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (flags & SGFIM_TX_LOAD) {
        std::vector<uint64_t> rp(n_win + 1);
        for (uint64_t w = 0; w <= n_win; ++w) rp[w] = w * S;
        return sgfim_load_csr(h, rp.data(), items_out, n_win);
    }
    return SGFIM_OK;
    API_GUARD_END(h)
}
