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

// ---------------------------------------------------------------------------------------
// Two volume rows per thread.  With a vertical tilt axis and whole-row centre offsets the
// rows r and r + 1 see the same image-column position at every (x, z) of a tilt, so the
// position, interpolation weight and z-interval test of a (voxel column, tilt) serve both
// rows.  The two rows' image segments are interleaved per pair slot as
// (v0 - d0, v1 - d1, d0, d1): one 128-bit shared load feeds a packed FP32x2 FMA (the two
// samples) and a packed add into the two voxels.  Each lane of the packed operations
// rounds as the scalar fmaf / add of the one-row kernel, so the result is bitwise the same.
//
// Tile: 64 x-columns x 4*KZ z-planes x 2 rows; thread (tx, tzg) owns KZ voxels along z of
// column x0 + tx in both rows.  16 tilts are staged per chunk.  16-bit volumes take the
// per-chunk Kahan form only (no per-add NaN / positivity rules: those go to the one-row
// kernel).
template <int KZ>
struct Bp2 {
    static constexpr int kTC = 16;
    static constexpr int kSeg = 96;
    static constexpr int kRawSeg = kSeg + 8;
    static constexpr int kTZ2 = 4 * KZ;
    static constexpr size_t seg_off = 0;                                                 // float4 [kTC][kSeg]
    static constexpr size_t raw_off = seg_off + sizeof(float4) * kTC * kSeg;            // float [kTC][2][kRawSeg]
    static constexpr size_t zint_off = raw_off + sizeof(float) * kTC * 2 * kRawSeg;     // int [kTC][kTX]
    static constexpr size_t az_off = zint_off + sizeof(int) * kTC * kTX;                 // long long [kTC][4]
    static constexpr size_t cs_off = az_off + sizeof(long long) * kTC * 4;               // long long C[kTC], S[kTC]
    static constexpr size_t st_off = cs_off + sizeof(long long) * 2 * kTC;               // int seg / raw start
    static constexpr size_t comp_off = (st_off + sizeof(int) * 2 * kTC + 15) & ~(size_t)15;  // float [2][KZ][256]
    static constexpr size_t bytes(bool kahan) {
        return comp_off + (kahan ? sizeof(float) * 2 * KZ * kBpThreads : 0);
    }
};

// Voxels per thread along z: 16 for FP32 volumes (80 registers, three CTAs per SM); 8 for
// 16-bit volumes, whose per-chunk partial sums double the voxel registers.
template <int VT>
struct Bp2Occ {
    static constexpr int value = 3;
    static constexpr int kz = VT == kVolF32 ? 16 : 8;
};

template <bool SANITIZE, bool POS, int VT, int KZ>
__device__ __forceinline__ void bp2_body(const BpLaunch& a, const int x0, const int z0, const int r0) {
    using L = Bp2<KZ>;
    constexpr int kTC = L::kTC, kSeg = L::kSeg, kRawSeg = L::kRawSeg;
    constexpr bool CHUNK_KAHAN = VT != kVolF32;
    static_assert(VT == kVolF32 || (!SANITIZE && !POS), "16-bit rows with per-add rules use the one-row kernel");
    extern __shared__ __align__(16) unsigned char bsm[];
    float4* seg = reinterpret_cast<float4*>(bsm + L::seg_off);
    float(*raw)[2][kRawSeg] = reinterpret_cast<float(*)[2][kRawSeg]>(bsm + L::raw_off);
    int(*zint)[kTX] = reinterpret_cast<int(*)[kTX]>(bsm + L::zint_off);
    long long(*AZ)[4] = reinterpret_cast<long long(*)[4]>(bsm + L::az_off);
    long long* sC = reinterpret_cast<long long*>(bsm + L::cs_off);
    long long* sS = sC + kTC;
    int* seg_start = reinterpret_cast<int*>(bsm + L::st_off);
    int* raw_start = seg_start + kTC;
    float* comp_sh = reinterpret_cast<float*>(bsm + L::comp_off);

    const int tid = threadIdx.x;
    const int tx = tid % kTX;
    const int tzg = tid / kTX;
    const int W = a.W, H = a.H, D = a.D, w = a.w, h = a.h;
    // rows r0 and r0 + 1 of [y0, y1); a row whose projection row is outside [0, h) is left as it is
    int jp[2];
    bool rin[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int r = r0 + q;
        jp[q] = r + a.row_off;
        rin[q] = r < a.y1 && jp[q] >= 0 && jp[q] < h;
    }
    if (!rin[0] && !rin[1]) return;
    const int zs = z0 + tzg * KZ;
    const int x = x0 + tx;
    const int nk = (x < W) ? min(KZ, D - zs) : 0;
    const unsigned plane = (unsigned)H * (unsigned)W;
    float vsc[2] = {1.0f, 1.0f};
    if (VT != kVolF32) {
        vsc[0] = rin[0] ? a.vscale[r0] : 1.0f;
        vsc[1] = rin[1] ? a.vscale[r0 + 1] : 1.0f;
    }
    float2 vx[KZ], pt[KZ];
    {
        const size_t v0 = ((size_t)zs * H + r0) * W + x;  // voxel (x, r0, zs); row r0 + 1 is W further
        if (VT == kVolF32) {
            const float* vb = static_cast<const float*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < KZ; k++) {
                vx[k].x = (k < nk && rin[0]) ? vb[k * plane] : 0.0f;
                vx[k].y = (k < nk && rin[1]) ? vb[k * plane + W] : 0.0f;
            }
        } else {
            const uint16_t* vb = static_cast<const uint16_t*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < KZ; k++) {
                vx[k].x = (k < nk && rin[0]) ? vol_load16<VT>(vb[k * plane]) * vsc[0] : 0.0f;
                vx[k].y = (k < nk && rin[1]) ? vol_load16<VT>(vb[k * plane + W]) * vsc[1] : 0.0f;
            }
        }
#pragma unroll
        for (int k = 0; k < KZ; k++) {
            pt[k] = make_float2(0.0f, 0.0f);
            if (CHUNK_KAHAN) {
                comp_sh[(0 * KZ + k) * kBpThreads + tid] = 0.0f;
                comp_sh[(1 * KZ + k) * kBpThreads + tid] = 0.0f;
            }
        }
    }

    const int xa = x0, xb = min(x0 + kTX - 1, W - 1);
    const int za = z0, zb = min(z0 + L::kTZ2 - 1, D - 1);
    const bool vec4 = ((w & 3) == 0) && ((reinterpret_cast<uintptr_t>(a.img) & 15) == 0);

    for (int c0 = 0; c0 < a.T; c0 += kTC) {
        const int tc = min(kTC, a.T - c0);
        if (tid < tc) {
            const int tilt = a.tilts[c0 + tid];
            const BpTilt b = a.btilt[tilt];
            sC[tid] = b.C;
            sS[tid] = b.S;
            const long long p00 = b.K + (long long)xa * b.C + (long long)za * b.S;
            const long long p10 = b.K + (long long)xb * b.C + (long long)za * b.S;
            const long long p01 = b.K + (long long)xa * b.C + (long long)zb * b.S;
            const long long p11 = b.K + (long long)xb * b.C + (long long)zb * b.S;
            const long long mn = min(min(p00, p10), min(p01, p11));
            const int s = (int)(mn >> 32);
            seg_start[tid] = s;
            raw_start[tid] = s & ~3;
            const long long base = (long long)(tid * kSeg - s) << 32;
#pragma unroll
            for (int g = 0; g < 4; g++) AZ[tid][g] = p00 + (long long)(g * KZ) * b.S + base;
        }
        for (int t = tzg; t < tc; t += kBpThreads / kTX)
            zint[t][tx] = (x < W) ? a.zint[(size_t)a.tilts[c0 + t] * W + x] : 0;
        __syncthreads();
        // stage both rows' image segments: one warp per (tilt, row), 128-bit loads
        for (int tq = tid >> 5; tq < 2 * tc; tq += kBpThreads / 32) {
            const int t = tq >> 1, q = tq & 1;
            if (!(q ? rin[1] : rin[0])) continue;
            const float* row = a.img + ((size_t)(c0 + t) * h + (q ? jp[1] : jp[0])) * w;
            for (int v = tid & 31; v < kRawSeg / 4; v += 32) {
                const int k0 = raw_start[t] + 4 * v;
                float4 f;
                if (vec4 && k0 >= 0 && k0 + 3 < w) {
                    f = *reinterpret_cast<const float4*>(row + k0);
                } else {
                    f.x = row[min(max(k0 + 0, 0), w - 1)];
                    f.y = row[min(max(k0 + 1, 0), w - 1)];
                    f.z = row[min(max(k0 + 2, 0), w - 1)];
                    f.w = row[min(max(k0 + 3, 0), w - 1)];
                }
                *reinterpret_cast<float4*>(&raw[t][q][4 * v]) = f;
            }
        }
        __syncthreads();
        for (int e = tid; e < tc * kSeg; e += kBpThreads) {
            const int t = e / kSeg, m = e - t * kSeg;
            const int k = seg_start[t] + m;
            const int o = k - raw_start[t];
            float vd[2], dd[2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float v0 = 0.0f, d = 0.0f;
                if (rin[q]) {
                    const float* row = a.img + ((size_t)(c0 + t) * h + jp[q]) * w;
                    int k0, k1;
                    if (k >= 0 && k < w - 1) {
                        v0 = raw[t][q][o];
                        d = raw[t][q][o + 1] - v0;
                        k0 = k;
                        k1 = k + 1;
                    } else {
                        k0 = k1 = (k < 0) ? 0 : w - 1;
                        v0 = row[k0];
                    }
                    if (SANITIZE) {
                        const float* up = (jp[q] < h - 1) ? row + w : row;
                        if (!isfinite(up[k0]) || !isfinite(up[k1])) v0 = __int_as_float(0x7fc00000);
                    }
                }
                vd[q] = v0 - d;
                dd[q] = d;
            }
            seg[t * kSeg + m] = make_float4(vd[0], vd[1], dd[0], dd[1]);
        }
        __syncthreads();
        for (int t = 0; t < tc; t++) {
            const long long S = sS[t];
            long long X = AZ[t][tzg] + (long long)(unsigned)tx * sC[t];
            const int zi = zint[t][tx];
            const int kl = (zi & 0xFFFF) - zs;
            const int cnt = (int)((uint32_t)zi >> 16);
            const bool full = nk > 0 && kl <= 0 && kl + cnt >= KZ;
            auto add = [&](int k, float2 sv) {
                if (CHUNK_KAHAN) {
                    pt[k] = __fadd2_rn(pt[k], sv);
                } else if (!SANITIZE && !POS) {
                    vx[k] = __fadd2_rn(vx[k], sv);
                } else {
                    float cdummy = 0.0f;
                    bp_acc<SANITIZE, POS, kVolF32>(vx[k].x, cdummy, sv.x);
                    bp_acc<SANITIZE, POS, kVolF32>(vx[k].y, cdummy, sv.y);
                }
            };
            if (__all_sync(0xffffffffu, full)) {
                long long X1 = X + S;
                const long long S2 = 2 * S;
#pragma unroll
                for (int k = 0; k < KZ; k += 2) {
                    const float4 p0 = seg[(int)(X >> 32)];
                    const float4 p1 = seg[(int)(X1 >> 32)];
                    const float f0 = fix_one_plus_frac((uint32_t)X), f1 = fix_one_plus_frac((uint32_t)X1);
                    add(k, __ffma2_rn(make_float2(f0, f0), make_float2(p0.z, p0.w), make_float2(p0.x, p0.y)));
                    add(k + 1, __ffma2_rn(make_float2(f1, f1), make_float2(p1.z, p1.w), make_float2(p1.x, p1.y)));
                    X += S2;
                    X1 += S2;
                }
            } else {
#pragma unroll
                for (int k = 0; k < KZ; k++) {
                    if ((unsigned)(k - kl) < (unsigned)cnt) {
                        const float4 p = seg[(int)(X >> 32)];
                        const float f = fix_one_plus_frac((uint32_t)X);
                        add(k, __ffma2_rn(make_float2(f, f), make_float2(p.z, p.w), make_float2(p.x, p.y)));
                    }
                    X += S;
                }
            }
        }
        if (CHUNK_KAHAN) {
#pragma unroll
            for (int k = 0; k < KZ; k++) {
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    float& vq = q ? vx[k].y : vx[k].x;
                    const float part = q ? pt[k].y : pt[k].x;
                    float cp = comp_sh[(q * KZ + k) * kBpThreads + tid];
                    const float y = part - cp;
                    const float tt = vq + y;
                    cp = (tt - vq) - y;
                    vq = tt;
                    comp_sh[(q * KZ + k) * kBpThreads + tid] = cp;
                }
                pt[k] = make_float2(0.0f, 0.0f);
            }
        }
        __syncthreads();
    }

#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (!rin[q]) continue;
        const size_t v0 = ((size_t)zs * H + r0 + q) * W + x;
        if (VT == kVolF32) {
            float* vb = static_cast<float*>(a.vol) + v0;
#pragma unroll
            for (int k = 0; k < KZ; k++)
                if (k < nk) vb[k * plane] = q ? vx[k].y : vx[k].x;
        } else {
            uint16_t* vb = static_cast<uint16_t*>(a.vol) + v0;
            const float inv = 1.0f / vsc[q];
            float m = 0.0f;
            bool range = false;
#pragma unroll
            for (int k = 0; k < KZ; k++) {
                if (k < nk) {
                    const float v = (q ? vx[k].y : vx[k].x) - comp_sh[(q * KZ + k) * kBpThreads + tid];
                    m = fmaxf(m, fabsf(v));
                    float qv = v * inv;
                    if (VT == kVolF16 && fabsf(qv) > kF16Max && isfinite(qv)) {
                        range = true;
                        qv = copysignf(kF16Max, qv);
                    }
                    vb[k * plane] = vol_store16<VT>(qv);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((tid & 31) == 0 && m > 0.0f) atomicMax(a.vmax + r0 + q, __float_as_uint(m));
            if (range) atomicOr(a.status, (int)kStatusRange);
        }
    }
}

template <bool SANITIZE, bool POS, int VT>
__global__ void __launch_bounds__(kBpThreads, Bp2Occ<VT>::value) bp2_kernel(const __grid_constant__ BpLaunch a) {
    constexpr int KZ = Bp2Occ<VT>::kz;
    bp2_body<SANITIZE, POS, VT, KZ>(a, blockIdx.x * kTX, blockIdx.y * Bp2<KZ>::kTZ2, a.y0 + 2 * blockIdx.z);
}

// Batched form: CTA b works on item {problem, x tile, z tile, first row of the pair}.
template <bool SANITIZE, bool POS, int VT>
__global__ void __launch_bounds__(kBpThreads, Bp2Occ<VT>::value)
    bp2_kernel_batch(const BpLaunch* __restrict__ descs, const int4* __restrict__ items) {
    const int4 it = items[blockIdx.x];
    constexpr int KZ = Bp2Occ<VT>::kz;
    bp2_body<SANITIZE, POS, VT, KZ>(descs[it.x], it.y * kTX, it.z * Bp2<KZ>::kTZ2, it.w);
}

// Persistent batched forms: a resident grid whose CTAs take items in list order through
// an atomic cursor until the list runs out (the host orders it by decreasing work).
template <bool SANITIZE, bool POS, int VT>
__global__ void __launch_bounds__(kBpThreads, Bp2Occ<VT>::value)
    bp2_kernel_persist(const BpLaunch* __restrict__ descs, const int4* __restrict__ items, int n_items,
                       int* __restrict__ cursor) {
    constexpr int KZ = Bp2Occ<VT>::kz;
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(cursor, 1);
        __syncthreads();
        const int i = s_item;
        __syncthreads();  // every thread has the index before thread 0 fetches the next
        if (i >= n_items) return;
        const int4 it = items[i];
        bp2_body<SANITIZE, POS, VT, KZ>(descs[it.x], it.y * kTX, it.z * Bp2<KZ>::kTZ2, it.w);
        __syncthreads();  // shared memory is free for the next item
    }
}

template <bool SANITIZE, bool POS, int VT>
__global__ void __launch_bounds__(kBpCtaThreads, BpOcc<VT>::value)
    bp_kernel_persist(const BpLaunch* __restrict__ descs, const int4* __restrict__ items, int n_items,
                      int* __restrict__ cursor) {
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(cursor, 1);
        __syncthreads();
        const int i = s_item;
        __syncthreads();  // every thread has the index before thread 0 fetches the next
        if (i >= n_items) return;
        const int4 it = items[i];
        bp_body<SANITIZE, POS, VT, 96>(descs[it.x], it.y * kTX, it.z * kTZ, it.w);
        __syncthreads();
    }
}

template <bool SANITIZE, bool POS, int VT>
cudaError_t bp2_attr_one() {
    const int m = (int)Bp2<Bp2Occ<VT>::kz>::bytes(VT != kVolF32);
    cudaError_t e = cudaFuncSetAttribute(bp2_kernel<SANITIZE, POS, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(bp2_kernel_persist<SANITIZE, POS, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(bp2_kernel_batch<SANITIZE, POS, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

// FP32 volumes: every rule combination; 16-bit volumes: the plain form only.
template <int VT>
void bp2_vt(bool sanitize, bool positivity, const BpLaunch& a, dim3 grid, cudaStream_t s) {
    const size_t sm = Bp2<Bp2Occ<VT>::kz>::bytes(VT != kVolF32);
    if constexpr (VT == kVolF32) {
        if (sanitize) {
            if (positivity) bp2_kernel<true, true, VT><<<grid, kBpThreads, sm, s>>>(a);
            else bp2_kernel<true, false, VT><<<grid, kBpThreads, sm, s>>>(a);
        } else {
            if (positivity) bp2_kernel<false, true, VT><<<grid, kBpThreads, sm, s>>>(a);
            else bp2_kernel<false, false, VT><<<grid, kBpThreads, sm, s>>>(a);
        }
    } else {
        (void)sanitize;
        (void)positivity;
        bp2_kernel<false, false, VT><<<grid, kBpThreads, sm, s>>>(a);
    }
}

template <int VT>
void bp2_batch_vt(bool sanitize, bool positivity, const BpLaunch* descs, const int4* items, int n, cudaStream_t s) {
    const size_t sm = Bp2<Bp2Occ<VT>::kz>::bytes(VT != kVolF32);
    if constexpr (VT == kVolF32) {
        if (sanitize) {
            if (positivity) bp2_kernel_batch<true, true, VT><<<n, kBpThreads, sm, s>>>(descs, items);
            else bp2_kernel_batch<true, false, VT><<<n, kBpThreads, sm, s>>>(descs, items);
        } else {
            if (positivity) bp2_kernel_batch<false, true, VT><<<n, kBpThreads, sm, s>>>(descs, items);
            else bp2_kernel_batch<false, false, VT><<<n, kBpThreads, sm, s>>>(descs, items);
        }
    } else {
        (void)sanitize;
        (void)positivity;
        bp2_kernel_batch<false, false, VT><<<n, kBpThreads, sm, s>>>(descs, items);
    }
}

template <int VT>
void bp2_persist_vt(bool sanitize, bool positivity, const BpLaunch* descs, const int4* items, int n, int* cursor,
                    int grid, cudaStream_t s) {
    const size_t sm = Bp2<Bp2Occ<VT>::kz>::bytes(VT != kVolF32);
    if constexpr (VT == kVolF32) {
        if (sanitize) {
            if (positivity) bp2_kernel_persist<true, true, VT><<<grid, kBpThreads, sm, s>>>(descs, items, n, cursor);
            else bp2_kernel_persist<true, false, VT><<<grid, kBpThreads, sm, s>>>(descs, items, n, cursor);
        } else {
            if (positivity) bp2_kernel_persist<false, true, VT><<<grid, kBpThreads, sm, s>>>(descs, items, n, cursor);
            else bp2_kernel_persist<false, false, VT><<<grid, kBpThreads, sm, s>>>(descs, items, n, cursor);
        }
    } else {
        (void)sanitize;
        (void)positivity;
        bp2_kernel_persist<false, false, VT><<<grid, kBpThreads, sm, s>>>(descs, items, n, cursor);
    }
}

template <int VT>
void bp_persist_vt(bool sanitize, bool positivity, const BpLaunch* descs, const int4* items, int n, int* cursor,
                   int grid, cudaStream_t s) {
    if (sanitize) {
        if (positivity) bp_kernel_persist<true, true, VT><<<grid, kBpCtaThreads, 0, s>>>(descs, items, n, cursor);
        else bp_kernel_persist<true, false, VT><<<grid, kBpCtaThreads, 0, s>>>(descs, items, n, cursor);
    } else {
        if (positivity) bp_kernel_persist<false, true, VT><<<grid, kBpCtaThreads, 0, s>>>(descs, items, n, cursor);
        else bp_kernel_persist<false, false, VT><<<grid, kBpCtaThreads, 0, s>>>(descs, items, n, cursor);
    }
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

// FP32 volumes only: the 16-bit form's per-chunk partial sums cost more than the pairing
// saves (measured: 89.9 against 85.7 ms per 2048 x 512 x 2048 x 121-tilt backprojection).
bool bp_row_pairs(int vtype, bool sanitize, bool positivity) {
    (void)sanitize;
    (void)positivity;
    return vtype == kVolF32;
}
int bp_pair_tile_z(int vtype) { return 4 * (vtype == kVolF32 ? Bp2Occ<kVolF32>::kz : Bp2Occ<kVolF16>::kz); }

cudaError_t bp_init_attributes() {
    cudaError_t e;
    if ((e = bp2_attr_one<false, false, kVolF32>()) != cudaSuccess) return e;
    if ((e = bp2_attr_one<false, true, kVolF32>()) != cudaSuccess) return e;
    if ((e = bp2_attr_one<true, false, kVolF32>()) != cudaSuccess) return e;
    if ((e = bp2_attr_one<true, true, kVolF32>()) != cudaSuccess) return e;
    if ((e = bp2_attr_one<false, false, kVolBF16>()) != cudaSuccess) return e;
    return bp2_attr_one<false, false, kVolF16>();
}

cudaError_t launch_bp_batch(bool sanitize, bool positivity, int vtype, bool pairs, const BpLaunch* descs,
                            const int4* items, int n_items, cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    if (pairs) {
        if (!bp_row_pairs(vtype, sanitize, positivity)) return cudaErrorInvalidValue;
        if (vtype == kVolF32) bp2_batch_vt<kVolF32>(sanitize, positivity, descs, items, n_items, s);
        else if (vtype == kVolBF16) bp2_batch_vt<kVolBF16>(sanitize, positivity, descs, items, n_items, s);
        else if (vtype == kVolF16) bp2_batch_vt<kVolF16>(sanitize, positivity, descs, items, n_items, s);
        else return cudaErrorInvalidValue;
        count_launch();
        return cudaGetLastError();
    }
    if (vtype == kVolF32) bp_batch_vt<kVolF32>(sanitize, positivity, descs, items, n_items, s);
    else if (vtype == kVolBF16) bp_batch_vt<kVolBF16>(sanitize, positivity, descs, items, n_items, s);
    else if (vtype == kVolF16) bp_batch_vt<kVolF16>(sanitize, positivity, descs, items, n_items, s);
    else return cudaErrorInvalidValue;
    count_launch();
    return cudaGetLastError();
}

int bp_persist_ctas_per_sm(int vtype, bool pairs) {
    if (pairs) return vtype == kVolF32 ? Bp2Occ<kVolF32>::value : Bp2Occ<kVolF16>::value;
    return vtype == kVolF32 ? BpOcc<kVolF32>::value : BpOcc<kVolF16>::value;
}

cudaError_t launch_bp_persist(bool sanitize, bool positivity, int vtype, bool pairs, const BpLaunch* descs,
                              const int4* items, int n_items, int* cursor, int grid, cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    if (pairs) {
        if (!bp_row_pairs(vtype, sanitize, positivity)) return cudaErrorInvalidValue;
        if (vtype == kVolF32) bp2_persist_vt<kVolF32>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else if (vtype == kVolBF16) bp2_persist_vt<kVolBF16>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else if (vtype == kVolF16) bp2_persist_vt<kVolF16>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else return cudaErrorInvalidValue;
    } else {
        if (vtype == kVolF32) bp_persist_vt<kVolF32>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else if (vtype == kVolBF16) bp_persist_vt<kVolBF16>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else if (vtype == kVolF16) bp_persist_vt<kVolF16>(sanitize, positivity, descs, items, n_items, cursor, grid, s);
        else return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bp_separable(const BpLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.y1 <= a.y0) return cudaSuccess;
    const int tz2 = bp_pair_tile_z(a.vtype);
    dim3 g2((a.W + kTX - 1) / kTX, (a.D + tz2 - 1) / tz2, (a.y1 - a.y0 + 1) / 2);
    // row pairs halve the CTAs: below two waves of resident CTAs the one-row kernel's
    // fuller grid is faster (256 x 64 x 256: 0.093 against 0.126 ms)
    const long long ctas2 = (long long)g2.x * g2.y * g2.z;
    const bool big = ctas2 >= 2LL * Bp2Occ<kVolF32>::value * (a.sms > 0 ? a.sms : 148);
    if (!a.bprow && !a.wide_seg && bp_row_pairs(a.vtype, a.sanitize, a.positivity) &&
        (a.rows_mode == 2 || (a.rows_mode == 0 && big))) {
        if (a.vtype == kVolF32) bp2_vt<kVolF32>(a.sanitize, a.positivity, a, g2, s);
        else if (a.vtype == kVolBF16) bp2_vt<kVolBF16>(false, false, a, g2, s);
        else if (a.vtype == kVolF16) bp2_vt<kVolF16>(false, false, a, g2, s);
        else return cudaErrorInvalidValue;
        count_launch();
        return cudaGetLastError();
    }
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
