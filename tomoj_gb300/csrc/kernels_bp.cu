// Voxel-driven backprojection fused with the relaxation update (separable geometry).
//
// Reference: VoxelProjector3D.backproject / backProjectPartial
// (TomoJ_Base/.../projectors/VoxelProjector3D.java:155-308) with ImageJ's
// bilinear getInterpolatedValue.  The reference adds one tilt at a time to the
// float volume (planez[i+jj] += value, then NaN/Inf -> 0 and optional
// positivity); here every voxel is loaded once, all tilts of the update are
// added to it in the same order with the same float rounding and checks, and it
// is stored once.  The SIRT/OS-SART relaxation factor is already folded into the
// difference images by the forward kernel (VoxelProjector3D.difference).
//
// CTA tile: 64 x-columns x 64 z-planes of one volume row.  Thread (tx, tzg)
// owns the 16 voxels z = z0 + 16*tzg + k of column x0 + tx.  Per chunk of 32
// tilts the CTA stages, for each tilt, the segment of the image row the tile
// projects onto as (v - slope, slope) pairs read with 128-bit loads, plus each
// column's exact z-interval of voxels that fall inside the projection.
#include <cmath>

#include "device_util.cuh"
#include "tomo_internal.h"
#include "vol_storage.cuh"

namespace tomo {
namespace {

#ifndef TOMO_BP_MIN_BLOCKS
#define TOMO_BP_MIN_BLOCKS 4
#endif
constexpr int kBpThreads = 256;
#ifndef TOMO_BP_NC
#define TOMO_BP_NC 1
#endif
constexpr int kNC = TOMO_BP_NC;                  // columns per thread
constexpr int kBpCtaThreads = kBpThreads / kNC;  // threads per CTA
constexpr int kTX = 64;
constexpr int kTZ = 64;
constexpr int kKZ = 16;      // voxels per thread along z
// Image-row segment a tile projects onto: 63 * scale * (|cos| + |sin|) + 3 pairs per
// tilt.  SEG = 96 covers scale 1; SEG = 192 (with half as many tilts per chunk, to stay
// within static shared memory) covers scale up to 2.1.
template <int SEG>
struct BpSeg {
    static constexpr int kTC = SEG <= 96 ? 32 : 16;  // tilts staged per chunk
    static constexpr int kSeg = SEG;
    static constexpr int kRawSeg = SEG + 8;           // floats staged per tilt (kSeg + 1 up to float4, + slack)
};

template <int SEG>
struct BpShared {
    static constexpr int kTC = BpSeg<SEG>::kTC, kSeg = BpSeg<SEG>::kSeg, kRawSeg = BpSeg<SEG>::kRawSeg;
    float2 seg[kTC * kSeg];  // tilt t's pairs at [t * kSeg, (t + 1) * kSeg)
    float raw[kTC][kRawSeg];
    int seg_start[kTC];
    int raw_start[kTC];
    long long C[kTC], S[kTC];
    long long AZ[kTC][4];  // position of (x0, z0 + 16 g) with the segment base, per tilt and z-group g
    int zint[kTC][kTX];
};

template <bool SANITIZE, bool POS>
__device__ __forceinline__ void bp_add(float& vox, float val) {
    if (SANITIZE) {
        if (!isnan(val)) {
            float v = vox + val;
            if (isnan(v) || isinf(v)) v = 0.0f;
            if (POS && v < 0.0f) v = 0.0f;
            vox = v;
        }
    } else {
        float v = vox + val;
        if (POS && v < 0.0f) v = 0.0f;
        vox = v;
    }
}

// Reduced-precision storage: Kahan-compensated FP32 sum (comp carries the
// running rounding error); the reference's per-add NaN/Inf and positivity rules
// act on the compensated sum and reset the compensation.
template <bool SANITIZE, bool POS>
__device__ __forceinline__ void bp_add_kahan(float& vox, float& comp, float val) {
    if (SANITIZE && isnan(val)) return;
    const float y = val - comp;
    float t = vox + y;
    comp = (t - vox) - y;
    if (SANITIZE && (isnan(t) || isinf(t))) {
        t = 0.0f;
        comp = 0.0f;
    }
    if (POS && t < 0.0f) {
        t = 0.0f;
        comp = 0.0f;
    }
    vox = t;
}

template <bool SANITIZE, bool POS, int VT>
__device__ __forceinline__ void bp_acc(float& vox, float& comp, float val) {
    if (VT == kVolF32)
        bp_add<SANITIZE, POS>(vox, val);
    else
        bp_add_kahan<SANITIZE, POS>(vox, comp, val);
}

// One CTA's work: tile (x0, z0) of volume row r of problem `a`.  The CTA has
// kBpThreads / kNC threads; thread (tx, tzg) owns the 16 voxels z = z0 + 16*tzg + k of
// the kNC columns x0 + tx + c * kCX (kCX = kTX / kNC), so the per-tilt position setup
// and interval test are shared by kNC * 16 voxel-updates.
template <bool SANITIZE, bool POS, int VT, int SEG>
__device__ __forceinline__ void bp_body(const BpLaunch& a, const int x0, const int z0, const int r) {
    constexpr int kTC = BpSeg<SEG>::kTC, kSeg = BpSeg<SEG>::kSeg, kRawSeg = BpSeg<SEG>::kRawSeg;
    constexpr int kThr = kBpCtaThreads, kCX = kTX / kNC;
    static_assert(kThr / kCX == 4 && 4 * kKZ == kTZ, "four z-groups of 16 voxels per tile");
    __shared__ __align__(16) BpShared<SEG> sh;
    const int tid = threadIdx.x;
    const int tx = tid % kCX;
    const int tzg = tid / kCX;
    const int W = a.W, H = a.H, D = a.D, w = a.w, h = a.h;
    const int jp = a.bprow ? a.bprow[r] : r + a.row_off;  // projection row seen by this volume row
    if (jp < 0 || jp >= h) return;  // no tilt reaches this row (yy outside [0,h))
    // fractional rows: blend projection rows jp and jp + 1 with weight byf (ImageJ's bilinear
    // weight along y); at jp = h - 1 ImageJ blends the row with itself
    const float byf = a.bpyf ? a.bpyf[r] : 0.0f;
    const bool blend = byf != 0.0f && jp < h - 1;
    const int zs = z0 + tzg * kKZ;

    // voxel k of a thread sits k * H * W elements after its first; tomo_create keeps
    // 16 * H * W below 2^32, so the offsets are 32-bit products of a uniform value
    const unsigned plane = (unsigned)H * (unsigned)W;
    const float vsc = (VT == kVolF32) ? 1.0f : a.vscale[r];
    // Reduced storage without the per-add NaN/Inf/positivity rules: the tilts of a staged
    // chunk are summed in `part` (plain FP32, at most 32 terms) and each chunk's sum is
    // added to the voxel with Kahan compensation, the compensation terms parked in shared
    // memory between chunks (read and written once per chunk).  With the per-add rules
    // every add is compensated (bp_add_kahan).
    constexpr bool CHUNK_KAHAN = (VT != kVolF32) && !SANITIZE && !POS;
    __shared__ float comp_sh[CHUNK_KAHAN ? kNC * kKZ * kThr : 1];
    float vox[kNC][kKZ], comp[kNC][kKZ], part[kNC][kKZ];
    int nk[kNC];
#pragma unroll
    for (int c = 0; c < kNC; c++) {
        const int x = x0 + tx + c * kCX;
        nk[c] = (x < W) ? min(kKZ, D - zs) : 0;
        const size_t v0 = ((size_t)zs * H + r) * W + x;  // voxel (x, r, zs); voxel k is at v0 + k * plane
        if (VT == kVolF32) {
            const float* vb = static_cast<const float*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < kKZ; k++) vox[c][k] = (k < nk[c]) ? vb[k * plane] : 0.0f;
        } else {
            const uint16_t* vb = static_cast<const uint16_t*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < kKZ; k++) vox[c][k] = (k < nk[c]) ? vol_load16<VT>(vb[k * plane]) * vsc : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < kKZ; k++) {
            comp[c][k] = 0.0f;
            part[c][k] = 0.0f;
            if (CHUNK_KAHAN) comp_sh[(c * kKZ + k) * kThr + tid] = 0.0f;
        }
    }

    const int xa = x0, xb = min(x0 + kTX - 1, W - 1);
    const int za = z0, zb = min(z0 + kTZ - 1, D - 1);
    const bool vec4 = ((w & 3) == 0) && ((reinterpret_cast<uintptr_t>(a.img) & 15) == 0);

    for (int c0 = 0; c0 < a.T; c0 += kTC) {
        const int tc = min(kTC, a.T - c0);
        // --- per-tilt setup: fixed-point coefficients and segment start --------------
        if (tid < tc) {
            const int tilt = a.tilts[c0 + tid];
            const BpTilt b = a.btilt[tilt];
            sh.C[tid] = b.C;
            sh.S[tid] = b.S;
            const long long p00 = b.K + (long long)xa * b.C + (long long)za * b.S;
            const long long p10 = b.K + (long long)xb * b.C + (long long)za * b.S;
            const long long p01 = b.K + (long long)xa * b.C + (long long)zb * b.S;
            const long long p11 = b.K + (long long)xb * b.C + (long long)zb * b.S;
            const long long mn = min(min(p00, p10), min(p01, p11));
            const int s = (int)(mn >> 32);
            sh.seg_start[tid] = s;
            sh.raw_start[tid] = s & ~3;
            // the tilt's segment base rides in the high word, so (X >> 32) is the flat pair index
            const long long base = (long long)(tid * kSeg - s) << 32;
#pragma unroll
            for (int g = 0; g < 4; g++) sh.AZ[tid][g] = p00 + (long long)(g * kKZ) * b.S + base;
        }
        for (int t = tzg; t < tc; t += kThr / kCX)
#pragma unroll
            for (int c = 0; c < kNC; c++) {
                const int xc = x0 + tx + c * kCX;
                sh.zint[t][tx + c * kCX] = (xc < W) ? a.zint[(size_t)a.tilts[c0 + t] * W + xc] : 0;
            }
        __syncthreads();
        // --- stage image segments: 128-bit loads of the row, then (value, slope) pairs --
        // one warp per tilt, each lane loading 4 floats at a time
        for (int t = tid >> 5; t < tc; t += kThr / 32)
          for (int v = tid & 31; v < kRawSeg / 4; v += 32) {
            const float* row = a.img + ((size_t)(c0 + t) * h + jp) * w;
            const int k0 = sh.raw_start[t] + 4 * v;
            auto load4 = [&](const float* rw) {
                float4 q;
                if (vec4 && k0 >= 0 && k0 + 3 < w) {
                    q = *reinterpret_cast<const float4*>(rw + k0);
                } else {
                    q.x = rw[min(max(k0 + 0, 0), w - 1)];
                    q.y = rw[min(max(k0 + 1, 0), w - 1)];
                    q.z = rw[min(max(k0 + 2, 0), w - 1)];
                    q.w = rw[min(max(k0 + 3, 0), w - 1)];
                }
                return q;
            };
            float4 q = load4(row);
            if (blend) {
                const float4 q1 = load4(row + w);
                q.x = __fadd_rn(q.x, __fmul_rn(byf, __fsub_rn(q1.x, q.x)));
                q.y = __fadd_rn(q.y, __fmul_rn(byf, __fsub_rn(q1.y, q.y)));
                q.z = __fadd_rn(q.z, __fmul_rn(byf, __fsub_rn(q1.z, q.z)));
                q.w = __fadd_rn(q.w, __fmul_rn(byf, __fsub_rn(q1.w, q.w)));
            }
            *reinterpret_cast<float4*>(&sh.raw[t][4 * v]) = q;
        }
        __syncthreads();
        for (int e = tid; e < tc * kSeg; e += kThr) {
            const int t = e / kSeg, m = e - t * kSeg;
            const int k = sh.seg_start[t] + m;       // image column of this pair
            const int o = k - sh.raw_start[t];        // offset in the staged floats
            const float* row = a.img + ((size_t)(c0 + t) * h + jp) * w;
            float v0, d = 0.0f;
            int k0, k1;
            if (k >= 0 && k < w - 1) {
                v0 = sh.raw[t][o];
                d = sh.raw[t][o + 1] - v0;
                k0 = k;
                k1 = k + 1;
            } else {
                // ImageJ edge value: the last column is its own right neighbour; k < 0 only
                // arises from fixed-point rounding of positions just above 0.
                k0 = k1 = (k < 0) ? 0 : w - 1;
                v0 = row[k0];
                if (blend) v0 = __fadd_rn(v0, __fmul_rn(byf, __fsub_rn(row[w + k0], v0)));
            }
            if (SANITIZE && !blend) {
                // getInterpolatedValue blends in the next row with weight 0, so a
                // non-finite neighbour there still turns the sample into NaN.
                const float* up = (jp < h - 1) ? row + w : row;
                if (!isfinite(up[k0]) || !isfinite(up[k1])) v0 = __int_as_float(0x7fc00000);
            }
            sh.seg[t * kSeg + m] = make_float2(v0 - d, d);  // sample = fma(1 + f, d, v0 - d)
        }
        __syncthreads();
        // --- accumulate the chunk's tilts in update order ----------------------------------
        for (int t = 0; t < tc; t++) {
            const long long S = sh.S[t];
            const long long Xc0 = sh.AZ[t][tzg] + (long long)(unsigned)tx * sh.C[t];
#pragma unroll
            for (int c = 0; c < kNC; c++) {
                long long X = Xc0 + (long long)(c * kCX) * sh.C[t];
                const int zi = sh.zint[t][tx + c * kCX];
                const int kl = (zi & 0xFFFF) - zs;
                const int cnt = (int)((uint32_t)zi >> 16);
                const bool full = nk[c] > 0 && kl <= 0 && kl + cnt >= kKZ;
                if (__all_sync(0xffffffffu, full)) {
                    // two independent position chains (even / odd z)
                    long long X1 = X + S;
                    const long long S2 = 2 * S;
#pragma unroll
                    for (int k = 0; k < kKZ; k += 2) {
                        const float2 p0 = sh.seg[(int)(X >> 32)];
                        const float2 p1 = sh.seg[(int)(X1 >> 32)];
                        const float s0 = fmaf(fix_one_plus_frac((uint32_t)X), p0.y, p0.x);
                        const float s1 = fmaf(fix_one_plus_frac((uint32_t)X1), p1.y, p1.x);
                        if (CHUNK_KAHAN) {
                            part[c][k] += s0;
                            part[c][k + 1] += s1;
                        } else {
                            bp_acc<SANITIZE, POS, VT>(vox[c][k], comp[c][k], s0);
                            bp_acc<SANITIZE, POS, VT>(vox[c][k + 1], comp[c][k + 1], s1);
                        }
                        X += S2;
                        X1 += S2;
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < kKZ; k++) {
                        if ((unsigned)(k - kl) < (unsigned)cnt) {
                            const float2 p = sh.seg[(int)(X >> 32)];
                            const float sv = fmaf(fix_one_plus_frac((uint32_t)X), p.y, p.x);
                            if (CHUNK_KAHAN) part[c][k] += sv;
                            else bp_acc<SANITIZE, POS, VT>(vox[c][k], comp[c][k], sv);
                        }
                        X += S;
                    }
                }
            }
        }
        if (CHUNK_KAHAN) {
#pragma unroll
            for (int c = 0; c < kNC; c++)
#pragma unroll
                for (int k = 0; k < kKZ; k++) {
                    float cp = comp_sh[(c * kKZ + k) * kThr + tid];
                    const float y = part[c][k] - cp;
                    const float t = vox[c][k] + y;
                    cp = (t - vox[c][k]) - y;
                    vox[c][k] = t;
                    comp_sh[(c * kKZ + k) * kThr + tid] = cp;
                    part[c][k] = 0.0f;
                }
        }
        __syncthreads();
    }

#pragma unroll
    for (int c = 0; c < kNC; c++) {
        const size_t v0 = ((size_t)zs * H + r) * W + x0 + tx + c * kCX;
        if (VT == kVolF32) {
            float* vb = static_cast<float*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < kKZ; k++)
                if (k < nk[c]) vb[k * plane] = vox[c][k];
        } else {
            // store value / scale (exact: power of two) and feed the row maximum for re-scaling
            uint16_t* vb = static_cast<uint16_t*>(a.vol) + v0;
            const float inv = 1.0f / vsc;
            float m = 0.0f;
            bool range = false;
#pragma unroll
            for (int k = 0; k < kKZ; k++) {
                if (k < nk[c]) {
                    const float v = vox[c][k] - (CHUNK_KAHAN ? comp_sh[(c * kKZ + k) * kThr + tid] : comp[c][k]);
                    m = fmaxf(m, fabsf(v));
                    float q = v * inv;
                    if (VT == kVolF16 && fabsf(q) > kF16Max && isfinite(q)) {
                        range = true;  // reported through the status word; the slab saturates
                        q = copysignf(kF16Max, q);
                    }
                    vb[k * plane] = vol_store16<VT>(q);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((tid & 31) == 0 && m > 0.0f) atomicMax(a.vmax + r, __float_as_uint(m));
            if (range) atomicOr(a.status, (int)kStatusRange);
        }
    }
}

// Reduced storage carries a compensation register per voxel: fewer CTAs per SM.
template <int VT>
struct BpOcc {
#ifndef TOMO_BP_MIN_BLOCKS_16
#define TOMO_BP_MIN_BLOCKS_16 3
#endif
    static constexpr int value =
        kNC == 1 ? (VT == kVolF32 ? TOMO_BP_MIN_BLOCKS : TOMO_BP_MIN_BLOCKS_16) : (VT == kVolF32 ? 4 : 3);
};

template <bool SANITIZE, bool POS, int VT, int SEG>
__global__ void __launch_bounds__(kBpCtaThreads, BpOcc<VT>::value) bp_separable_kernel(const __grid_constant__ BpLaunch a) {
    bp_body<SANITIZE, POS, VT, SEG>(a, blockIdx.x * kTX, blockIdx.y * kTZ, a.y0 + blockIdx.z);
}

// Batched form: CTA b works on item {problem, x tile, z tile, row} of many problems.
template <bool SANITIZE, bool POS, int VT>
__global__ void __launch_bounds__(kBpCtaThreads, BpOcc<VT>::value)
    bp_kernel_batch(const BpLaunch* __restrict__ descs, const int4* __restrict__ items) {
    const int4 it = items[blockIdx.x];
    bp_body<SANITIZE, POS, VT, 96>(descs[it.x], it.y * kTX, it.z * kTZ, it.w);
}

template <int VT>
void bp_batch_vt(bool sanitize, bool positivity, const BpLaunch* descs, const int4* items, int n, cudaStream_t s) {
    if (sanitize) {
        if (positivity) bp_kernel_batch<true, true, VT><<<n, kBpCtaThreads, 0, s>>>(descs, items);
        else bp_kernel_batch<true, false, VT><<<n, kBpCtaThreads, 0, s>>>(descs, items);
    } else {
        if (positivity) bp_kernel_batch<false, true, VT><<<n, kBpCtaThreads, 0, s>>>(descs, items);
        else bp_kernel_batch<false, false, VT><<<n, kBpCtaThreads, 0, s>>>(descs, items);
    }
}

template <int VT, int SEG>
void bp_separable_vt(const BpLaunch& a, dim3 grid, cudaStream_t s) {
    if (a.sanitize) {
        if (a.positivity) bp_separable_kernel<true, true, VT, SEG><<<grid, kBpCtaThreads, 0, s>>>(a);
        else bp_separable_kernel<true, false, VT, SEG><<<grid, kBpCtaThreads, 0, s>>>(a);
    } else {
        if (a.positivity) bp_separable_kernel<false, true, VT, SEG><<<grid, kBpCtaThreads, 0, s>>>(a);
        else bp_separable_kernel<false, false, VT, SEG><<<grid, kBpCtaThreads, 0, s>>>(a);
    }
}

}  // namespace

int bp_tile_x() { return kTX; }
int bp_tile_z() { return kTZ; }
int bp_segment_pairs(bool wide) { return wide ? 192 : 96; }

cudaError_t launch_bp_batch(bool sanitize, bool positivity, int vtype, const BpLaunch* descs, const int4* items,
                            int n_items, cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    if (vtype == kVolF32) bp_batch_vt<kVolF32>(sanitize, positivity, descs, items, n_items, s);
    else if (vtype == kVolBF16) bp_batch_vt<kVolBF16>(sanitize, positivity, descs, items, n_items, s);
    else if (vtype == kVolF16) bp_batch_vt<kVolF16>(sanitize, positivity, descs, items, n_items, s);
    else return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bp_separable(const BpLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.y1 <= a.y0) return cudaSuccess;
    dim3 grid((a.W + kTX - 1) / kTX, (a.D + kTZ - 1) / kTZ, a.y1 - a.y0);
    if (a.wide_seg) {
        if (a.vtype != kVolF32) return cudaErrorInvalidValue;
        bp_separable_vt<kVolF32, 192>(a, grid, s);
    } else if (a.vtype == kVolF32) bp_separable_vt<kVolF32, 96>(a, grid, s);
    else if (a.vtype == kVolBF16) bp_separable_vt<kVolBF16, 96>(a, grid, s);
    else if (a.vtype == kVolF16) bp_separable_vt<kVolF16, 96>(a, grid, s);
    else return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

}  // namespace tomo
