// noalloc.cu -- batched supports without any device allocation.
//
// Some callers of this library may not allocate device memory at all: a host
// application that owns the GPU's memory through its own pool and forbids
// foreign cudaMalloc/cudaFree (serving processes that plan every byte of HBM
// at start-up), or a latency-critical loop where cudaMalloc's implicit device
// synchronisation and unpredictable cost are not acceptable.
// sgfim_support_batch_device needs a handle (sgfim_open allocates) and grows a
// scratch buffer on demand; this entry point instead runs the same kernels
// with their scratch in a fixed file-scope device array, so nothing is
// allocated by the call.
//
// Costs of that choice: every GPU on which the library is loaded keeps the
// array (kNoAllocScratchBytes, about 25 MB) until the process exits; inputs
// larger than SGFIM_NOALLOC_MAX_CAND candidates are rejected; and all calls
// share the one array, so calls that overlap on the GPU race.
//
// Device errors (a bounded wait that ran out) land in a second file-scope
// word that stays set until sgfim_noalloc_status reads and clears it.
#include <mutex>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"

namespace {

constexpr uint64_t kMaxCand = SGFIM_NOALLOC_MAX_CAND;
// The support kernels' scratch layout for the largest accepted input.
constexpr size_t kNoAllocScratchBytes = sg::support_scratch_bytes_for(kMaxCand);

__device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];
// [sg::kCtlCode] error code, [sg::kCtlWaitUs] wait bound (0 = default); zero at load
__device__ __align__(256) uint32_t g_dev_err[64];

struct DeviceSlot {
    bool ready = false;
    void *scratch = nullptr;   // device address of g_scratch on this device
    uint32_t *err = nullptr;   // device address of g_dev_err on this device
    int n_sm = 0;
};
constexpr int kMaxDevices = 64;
DeviceSlot g_slots[kMaxDevices];
std::mutex g_mu;

// Once per device, with that device current: resolve the device addresses of
// the file-scope arrays.  In host code their names are only host-side
// stand-ins, never valid device pointers.
int setup_device(int dev, DeviceSlot **out) {
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceSlot &s = g_slots[dev];
    if (!s.ready) {
        void *p = nullptr, *e = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess) return SGFIM_EDEVICE;
        if (cudaGetSymbolAddress(&e, g_dev_err) != cudaSuccess) return SGFIM_EDEVICE;
        int n_sm = 0;
        if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SGFIM_EDEVICE;
        s.scratch = p;
        s.err = static_cast<uint32_t *>(e);
        s.n_sm = n_sm;
        s.ready = true;
    }
    *out = &s;
    return SGFIM_OK;
}

}  // namespace

extern "C" int sgfim_support_batch_noalloc(const uint64_t *bitmaps, uint32_t d, uint64_t n_words,
                                           uint64_t row_stride, const uint64_t *cand_ptr,
                                           const uint32_t *cand_items, uint64_t n_cand, uint32_t *out,
                                           void *stream) {
    if (n_cand > kMaxCand) return SGFIM_ECAPACITY;
    if ((n_cand && (!cand_ptr || !out)) || (d && !bitmaps)) return SGFIM_EINVAL;
    if (row_stride & 1) return SGFIM_EINVAL;
    const uint64_t n_even = (n_words + 1) & ~1ull;
    if (n_even > row_stride) return SGFIM_EINVAL;
    if (n_cand == 0) return SGFIM_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SGFIM_EDEVICE;
    DeviceSlot *slot = nullptr;
    int rc = setup_device(dev, &slot);
    if (rc != SGFIM_OK) return rc;
    try {
        CUtensorMap map;
        const bool map_ok = sg::encode_bitmap_map(&map, bitmaps, d, n_even, row_stride);
        sg::SupportScratch sc{slot->scratch, kNoAllocScratchBytes};
        sg::SupportPlan plan;
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (cudaStream_t)0;
        // The only non-zero return is a scratch area smaller than the layout of
        // n_cand candidates, which the size check above already rules out.
        if (sg::support_batch_device(bitmaps, d, n_even, row_stride, n_words * 64, cand_ptr, cand_items, n_cand, out,
                                     sc, plan, map_ok ? &map : nullptr, slot->err, st, slot->n_sm, nullptr) != 0)
            return SGFIM_ECAPACITY;
        return SGFIM_OK;
    } catch (const sg::CudaError &) {
        return SGFIM_EDEVICE;
    }
}

extern "C" int sgfim_noalloc_status(void *stream) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SGFIM_EDEVICE;
    DeviceSlot *slot = nullptr;
    int rc = setup_device(dev, &slot);
    if (rc != SGFIM_OK) return rc;
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (cudaStream_t)0;
    uint32_t code = 0;
    // a copy into pageable host memory returns once it has completed
    if (cudaMemcpyAsync(&code, slot->err + sg::kCtlCode, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return SGFIM_EDEVICE;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SGFIM_EDEVICE;
    if (code == DEVERR_NONE) return SGFIM_OK;
    if (cudaMemsetAsync(slot->err + sg::kCtlCode, 0, 4, st) != cudaSuccess) return SGFIM_EDEVICE;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SGFIM_EDEVICE;
    return SGFIM_EDEVICE;
}
