// Device helpers: shared-memory addresses, mbarrier + bulk-copy (TMA) PTX, and
// the fixed-point -> fraction conversion used by both projectors.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "tomo_internal.h"

namespace tomo {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Retires an mbarrier whose phases have all completed, so that its shared memory can be
// initialised again (a persistent CTA's next work item).
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// One bulk (non-tensor) TMA copy global -> shared, completing on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase: returns false after `max_tries` failed polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
    for (uint32_t i = 0; i < max_tries; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Fraction in [0,1) from the low 32 bits of a 32.32 fixed-point position
// (top 23 bits placed in the mantissa of a float in [1,2)).
__device__ __forceinline__ float fix_frac(uint32_t lo) {
    return __uint_as_float((lo >> 9) | 0x3F800000u) - 1.0f;
}

// 1 + fraction in [1,2) from the low 32 bits of a 32.32 fixed-point position; used with
// (v - d, d) pairs: v + f d == fma(1 + f, d, v - d).
__device__ __forceinline__ float fix_one_plus_frac(uint32_t lo) { return __uint_as_float((lo >> 9) | 0x3F800000u); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace tomo
