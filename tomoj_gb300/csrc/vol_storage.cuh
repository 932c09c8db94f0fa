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

// Lower bound of every row's scale, given the volume's largest |value| M: 2^-11 of the
// scale of M.  A row whose own values are tiny (a background row, a row that a TV step
// flattened) then keeps room up to about M before FP16 overflows, so the next
// backprojection can raise it to the level of the rest of the volume; its values stay
// normal down to about M * 2^-29.  A volume of zeros (M = 0) keeps 1.
__host__ __device__ inline float slab_scale_floor(float M) {
    if (!(M > 0.0f) || !(M < 3.0e38f)) return 1.0f;
    return slab_scale_for(M) * (1.0f / 2048.0f);
}

// Scale of a row whose largest |value| is m in a volume whose largest is M.
__host__ __device__ inline float slab_scale_target(float m, float M) {
    const float a = slab_scale_for(m), b = slab_scale_floor(M);
    return a > b ? a : b;
}

// A row is re-scaled when max / scale reaches 2^10 (FP16 room running out), or when it
// fell below 1 or the row's scale is under the floor and the target differs (precision,
// headroom).  A zero maximum (a row of zeros, or a row the backprojection did not reach)
// and a non-finite one leave the row as it is.
__host__ __device__ inline bool slab_needs_rescale(float m, float scale, float M) {
    if (!(m > 0.0f) || !(m < 3.0e38f)) return false;
    const float fl = slab_scale_floor(M);
    const float q = m / scale;
    if (q >= 1024.0f) return true;
    return (q < 1.0f || scale < fl) && slab_scale_target(m, M) != scale;
}

}  // namespace tomo
