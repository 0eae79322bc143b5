// common.cuh -- shared declarations of the sgfim engine (host + device).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

// ------------------------------------------------------------------ errors
// Device-side error codes written to the engine's error word.  A kernel that
// gives up (bounded wait ran out, index out of range) records the first code
// and the host turns it into SGFIM_EDEVICE.
enum : uint32_t {
    DEVERR_NONE = 0,
    DEVERR_MBAR_TIMEOUT = 1,   // an mbarrier wait hit its iteration limit
    DEVERR_BAD_ITEM = 2,       // a row index >= d reached a counting kernel
    DEVERR_OVERFLOW = 3,       // an output buffer would overflow
};

#include "errors.h"

namespace sg {

constexpr int kWarp = 32;

// Device control words.  Every kernel that can wait receives `err`, a pointer
// to a small device block: err[kCtlCode] holds the first error code, and
// err[kCtlWaitUs] the bound of every mbarrier wait in microseconds of
// %globaltimer (0 = kWaitLimitUsDefault).  A wait that runs out records
// DEVERR_MBAR_TIMEOUT and the kernel leaves; the host reads and clears the
// code after the launch.
constexpr int kCtlCode = 0;
constexpr int kCtlWaitUs = 1;
constexpr uint32_t kWaitLimitUsDefault = 4000000;  // 4 s

// ------------------------------------------------------------------ device helpers
__device__ __forceinline__ uint32_t popc64(uint64_t x) { return (uint32_t)__popcll(x); }

__device__ __forceinline__ void set_device_error(uint32_t *err, uint32_t code) {
    if (err) atomicCAS(err, 0u, code);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One poll of the mbarrier phase; true once the phase with `parity` completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: polls until the phase completes or err[kCtlWaitUs]
// microseconds (kWaitLimitUsDefault when 0 or err is null) have passed on the
// global timer, then records DEVERR_MBAR_TIMEOUT and returns false.  The
// clock is only read once the first poll has failed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err) {
    if (mbar_try_wait(bar, parity)) return true;
    uint32_t us = err ? *reinterpret_cast<volatile uint32_t *>(err + kCtlWaitUs) : 0u;
    if (us == 0) us = kWaitLimitUsDefault;
    const uint64_t t0 = global_ns(), limit = (uint64_t)us * 1000ull;
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit) break;
    }
    set_device_error(err, DEVERR_MBAR_TIMEOUT);
    return false;
}

// 2-D tiled TMA load (global -> this CTA's shared memory), completion on bar.
__device__ __forceinline__ void tma_load_2d(void *smem_dst, const CUtensorMap *map, int32_t x, int32_t y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// 1-D bulk copy global -> shared (both 16-byte aligned, size multiple of 16).
__device__ __forceinline__ void bulk_load_1d(void *smem_dst, const void *gsrc, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(gsrc)), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ uint4 ld_nc_v4(const void *p) {
    uint4 r;
    asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}

__device__ __forceinline__ uint32_t popc4(uint4 v) {
    return __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
}

__device__ __forceinline__ uint4 and4(uint4 a, uint4 b) {
    return make_uint4(a.x & b.x, a.y & b.y, a.z & b.z, a.w & b.w);
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace sg
