// Reduced-precision (BF16 / FP16) volume storage: packing with per-slab scales,
// unpacking, re-scaling after backprojection, fill and non-finite scan.
//
// The reference keeps its volume as float32 ImageStack slices
// (TomoReconstruction2.java:100-108).  Reduced storage is an engine option with no
// counterpart there: a volume row r (one XZ slab, the unit both projectors work
// on) holds value / vscale[r] in 16 bits, vscale[r] a power of two chosen from the
// row's largest magnitude, and every arithmetic step stays FP32.
#include <cmath>

#include "tomo_internal.h"
#include "vol_storage.cuh"

namespace tomo {
namespace {

constexpr int kThreads = 256;
constexpr int kRowZ = 16;  // planes per CTA in the row-max pass

__device__ __forceinline__ float block_max(float v, float* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

// grid (rows, ceil(D / kRowZ)): max |value| of row rr over planes [z0, z0 + kRowZ).
__global__ void rowmax_kernel(const float* __restrict__ src, int rows, int y0, int W, int D,
                              unsigned* __restrict__ vmax) {
    __shared__ float red[kThreads / 32];
    const int rr = blockIdx.x;
    const int z0 = blockIdx.y * kRowZ, z1 = min(D, z0 + kRowZ);
    float m = 0.0f;
    for (int z = z0; z < z1; z++) {
        const float* row = src + ((size_t)z * rows + rr) * W;
        for (int x = threadIdx.x; x < W; x += kThreads) m = fmaxf(m, fabsf(row[x]));  // fmaxf drops NaN
    }
    m = block_max(m, red);
    if (threadIdx.x == 0 && m > 0.0f) atomicMax(vmax + y0 + rr, __float_as_uint(m));
}

template <int VT>
__global__ void pack_kernel(const float* __restrict__ src, int rows, int y0, int W, int H, int D,
                            uint16_t* __restrict__ vol, float* __restrict__ vscale, const unsigned* __restrict__ vmax,
                            int* status, bool floor) {
    const size_t n = (size_t)D * rows * W;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        const int x = (int)(e % W);
        const size_t zr = e / W;
        const int rr = (int)(zr % rows);
        const int z = (int)(zr / rows);
        const int r = y0 + rr;
        const float m = __uint_as_float(vmax[r]);
        const float s = floor ? slab_scale_target(m, __uint_as_float(vmax[H])) : slab_scale_for(m);
        if (z == 0 && x == 0) vscale[r] = s;
        float v = src[e] / s;  // power of two: exact
        if (VT == kVolF16 && fabsf(v) > kF16Max && isfinite(v)) {
            atomicOr(status, (int)kStatusRange);
            v = copysignf(kF16Max, v);
        }
        vol[((size_t)z * H + r) * W + x] = vol_store16<VT>(v);
    }
}

template <int VT>
__global__ void unpack_kernel(const uint16_t* __restrict__ vol, const float* __restrict__ vscale, int rows, int y0,
                              int W, int H, int D, float* __restrict__ dst) {
    const size_t n = (size_t)D * rows * W;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        const int x = (int)(e % W);
        const size_t zr = e / W;
        const int rr = (int)(zr % rows);
        const int z = (int)(zr / rows);
        const int r = y0 + rr;
        dst[e] = vol_load16<VT>(vol[((size_t)z * H + r) * W + x]) * vscale[r];
    }
}

// One CTA per volume row: re-scales the row when its max left the band.
template <int VT>
__device__ __forceinline__ void rescale_row(uint16_t* __restrict__ vol, float* __restrict__ vscale,
                                            const unsigned* __restrict__ vmax, int W, int H, int D, int* status,
                                            int r) {
    const float m = __uint_as_float(vmax[r]), M = __uint_as_float(vmax[H]);
    const float s = vscale[r];
    if (!slab_needs_rescale(m, s, M)) return;
    const float ns = slab_scale_target(m, M);
    const float f = s / ns;  // ratio of powers of two: exact
    for (int z = 0; z < D; z++) {
        uint16_t* row = vol + ((size_t)z * H + r) * W;
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            float v = vol_load16<VT>(row[x]) * f;
            if (VT == kVolF16 && fabsf(v) > kF16Max && isfinite(v)) {
                atomicOr(status, (int)kStatusRange);
                v = copysignf(kF16Max, v);
            }
            row[x] = vol_store16<VT>(v);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) vscale[r] = ns;
}

template <int VT>
__global__ void rescale_kernel(uint16_t* __restrict__ vol, float* __restrict__ vscale,
                               const unsigned* __restrict__ vmax, int W, int H, int D, int* status) {
    rescale_row<VT>(vol, vscale, vmax, W, H, D, status, blockIdx.x);
}

// Batched forms over many volumes (a batch's 16-bit members): CTA y works on volume
// jobs[y]; the same per-volume passes, one launch each for all of them.
__global__ void vmax_total_batch_kernel(const VolJob* __restrict__ jobs) {
    __shared__ float red[kThreads / 32];
    const VolJob j = jobs[blockIdx.x];
    float m = 0.0f;
    for (int r = threadIdx.x; r < j.H; r += kThreads) m = fmaxf(m, __uint_as_float(j.vmax[r]));
    m = block_max(m, red);
    if (threadIdx.x == 0) j.vmax[j.H] = __float_as_uint(m);
}

__global__ void rescale_batch_kernel(const VolJob* __restrict__ jobs) {
    const VolJob j = jobs[blockIdx.y];
    if ((int)blockIdx.x >= j.H) return;
    uint16_t* v = static_cast<uint16_t*>(j.vol);
    if (j.vtype == kVolBF16) rescale_row<kVolBF16>(v, j.vscale, j.vmax, j.W, j.H, j.D, j.status, blockIdx.x);
    else rescale_row<kVolF16>(v, j.vscale, j.vmax, j.W, j.H, j.D, j.status, blockIdx.x);
}

__global__ void vmax_zero_batch_kernel(const VolJob* __restrict__ jobs) {
    const VolJob j = jobs[blockIdx.x];
    for (int r = threadIdx.x; r < j.H; r += kThreads) j.vmax[r] = 0u;
}

template <int VT>
__global__ void fill16_kernel(uint16_t* __restrict__ vol, size_t n, float stored, float* __restrict__ vscale,
                              unsigned* __restrict__ vmax, int H, float scale, float mag) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint16_t b = vol_store16<VT>(stored);
    for (size_t e = i0; e < n; e += stride) vol[e] = b;
    for (size_t r = i0; r < (size_t)H; r += stride) vscale[r] = scale;
    // row maxima and the volume's maximum (entry H) of the filled volume
    for (size_t r = i0; r <= (size_t)H; r += stride) vmax[r] = __float_as_uint(mag);
}

// One CTA: the volume's largest |value| (entry H) from the row maxima [0, H).
__global__ void vmax_total_kernel(unsigned* __restrict__ vmax, int H) {
    __shared__ float red[kThreads / 32];
    float m = 0.0f;
    for (int r = threadIdx.x; r < H; r += kThreads) m = fmaxf(m, __uint_as_float(vmax[r]));
    m = block_max(m, red);
    if (threadIdx.x == 0) vmax[H] = __float_as_uint(m);
}

template <int VT>
__global__ void scan16_kernel(const uint16_t* __restrict__ vol, size_t n, int* flags) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const uint16_t em = VT == kVolBF16 ? 0x7F80 : 0x7C00;  // exponent field
    bool bad = false;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) bad |= (vol[e] & em) == em;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, 1);
}

int grid_for(size_t n) {
    const size_t g = (n + kThreads - 1) / kThreads;
    const size_t cap = (size_t)device_sms() * 64;
    return (int)(g < cap ? (g == 0 ? 1 : g) : cap);
}

}  // namespace

cudaError_t launch_vol_rowmax(const float* src, int rows, int y0, int W, int H, int D, unsigned* vmax,
                              cudaStream_t s) {
    (void)H;
    if (rows <= 0) return cudaSuccess;
    rowmax_kernel<<<dim3(rows, (D + kRowZ - 1) / kRowZ), kThreads, 0, s>>>(src, rows, y0, W, D, vmax);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_vol_pack(const float* src, int rows, int y0, int W, int H, int D, int vtype, void* vol,
                            float* vscale, unsigned* vmax, bool floor, int* status, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    if (floor) {
        vmax_total_kernel<<<1, kThreads, 0, s>>>(vmax, H);
        count_launch();
    }
    const int g = grid_for((size_t)D * rows * W);
    uint16_t* v = static_cast<uint16_t*>(vol);
    if (vtype == kVolBF16)
        pack_kernel<kVolBF16><<<g, kThreads, 0, s>>>(src, rows, y0, W, H, D, v, vscale, vmax, status, floor);
    else if (vtype == kVolF16)
        pack_kernel<kVolF16><<<g, kThreads, 0, s>>>(src, rows, y0, W, H, D, v, vscale, vmax, status, floor);
    else
        return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_vol_unpack(const void* vol, int vtype, const float* vscale, int rows, int y0, int W, int H,
                              int D, float* dst, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    const int g = grid_for((size_t)D * rows * W);
    const uint16_t* v = static_cast<const uint16_t*>(vol);
    if (vtype == kVolBF16)
        unpack_kernel<kVolBF16><<<g, kThreads, 0, s>>>(v, vscale, rows, y0, W, H, D, dst);
    else if (vtype == kVolF16)
        unpack_kernel<kVolF16><<<g, kThreads, 0, s>>>(v, vscale, rows, y0, W, H, D, dst);
    else
        return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_vol_rescale(void* vol, int vtype, float* vscale, unsigned* vmax, int W, int H, int D,
                               int* status, cudaStream_t s) {
    uint16_t* v = static_cast<uint16_t*>(vol);
    vmax_total_kernel<<<1, kThreads, 0, s>>>(vmax, H);
    count_launch();
    if (vtype == kVolBF16)
        rescale_kernel<kVolBF16><<<H, kThreads, 0, s>>>(v, vscale, vmax, W, H, D, status);
    else if (vtype == kVolF16)
        rescale_kernel<kVolF16><<<H, kThreads, 0, s>>>(v, vscale, vmax, W, H, D, status);
    else
        return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_vol_hooks_batch(const VolJob* jobs, int n_jobs, int max_H, bool before, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    vmax_total_batch_kernel<<<n_jobs, kThreads, 0, s>>>(jobs);
    rescale_batch_kernel<<<dim3(max_H, n_jobs), kThreads, 0, s>>>(jobs);
    count_launch(2);
    if (before) {
        vmax_zero_batch_kernel<<<n_jobs, kThreads, 0, s>>>(jobs);
        count_launch();
    }
    return cudaGetLastError();
}

cudaError_t launch_vol_fill(void* vol, int vtype, float* vscale, unsigned* vmax, size_t nvox, int H, float value,
                            cudaStream_t s) {
    const float mag = std::isfinite(value) ? std::fabs(value) : 0.0f;
    const float scale = slab_scale_for(mag);
    const float stored = value / scale;
    uint16_t* v = static_cast<uint16_t*>(vol);
    const int g = grid_for(nvox > (size_t)H + 1 ? nvox : (size_t)H + 1);
    if (vtype == kVolBF16)
        fill16_kernel<kVolBF16><<<g, kThreads, 0, s>>>(v, nvox, stored, vscale, vmax, H, scale, mag);
    else if (vtype == kVolF16)
        fill16_kernel<kVolF16><<<g, kThreads, 0, s>>>(v, nvox, stored, vscale, vmax, H, scale, mag);
    else
        return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scan_nonfinite_vol(const void* vol, int vtype, size_t n, int* flags, cudaStream_t s) {
    if (vtype == kVolF32) return launch_scan_nonfinite(static_cast<const float*>(vol), n, flags, s);
    const uint16_t* v = static_cast<const uint16_t*>(vol);
    const int g = grid_for(n);
    if (vtype == kVolBF16)
        scan16_kernel<kVolBF16><<<g, kThreads, 0, s>>>(v, n, flags);
    else
        scan16_kernel<kVolF16><<<g, kThreads, 0, s>>>(v, n, flags);
    count_launch();
    return cudaGetLastError();
}

}  // namespace tomo
