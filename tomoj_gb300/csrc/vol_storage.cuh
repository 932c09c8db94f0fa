// Reduced-precision volume storage shared by the projectors and the volume
// kernels: 16-bit loads/stores (BF16 or FP16 bit patterns) and the slab-scale
// policy.  A reduced volume holds value / vscale[r] for volume row r (one XZ
// slab), vscale a power of two so that scaling never rounds.
#pragma once
#include <cstdint>
#include <cstring>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "tomo_internal.h"

namespace tomo {

constexpr float kF16Max = 65504.0f;

// Stored 16-bit pattern -> float (no scale).
template <int VT>
__device__ __forceinline__ float vol_load16(uint16_t b) {
    if (VT == kVolBF16) return __uint_as_float((uint32_t)b << 16);
    return __half2float(__ushort_as_half(b));
}

// float (already divided by the slab scale) -> stored 16-bit pattern, round to nearest even.
template <int VT>
__device__ __forceinline__ uint16_t vol_store16(float v) {
    if (VT == kVolBF16) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
    return __half_as_ushort(__float2half_rn(v));
}

__device__ __forceinline__ float vol_load16_rt(int vt, uint16_t b) {
    return vt == kVolBF16 ? vol_load16<kVolBF16>(b) : vol_load16<kVolF16>(b);
}

// Slab scale for a row whose largest |value| is m: the power of two that puts m in
// [2^4, 2^5), leaving FP16 a factor 2^11 of growth before its 65504 limit and keeping
// values down to m * 2^-18 normal.  Rows of zeros, subnormal or non-finite maxima keep 1.
__host__ __device__ inline float slab_scale_for(float m) {
    uint32_t b;
#ifdef __CUDA_ARCH__
    b = __float_as_uint(m);
#else
    std::memcpy(&b, &m, 4);
#endif
    const int be = (int)((b >> 23) & 0xFFu);
    if ((b & 0x80000000u) || be == 0 || be == 0xFF) return 1.0f;
    int se = be - 4;
    if (se < 1) se = 1;
    const uint32_t sb = (uint32_t)se << 23;
    float s;
#ifdef __CUDA_ARCH__
    s = __uint_as_float(sb);
#else
    std::memcpy(&s, &sb, 4);
#endif
    return s;
}

// A row is re-scaled after a backprojection when max / scale leaves [1, 2^10).
__host__ __device__ inline bool slab_needs_rescale(float m, float scale) {
    if (!(m > 0.0f) || !(m < 3.0e38f)) return false;
    const float q = m / scale;
    return q < 1.0f || q >= 1024.0f;
}

}  // namespace tomo
