// Forward projection fused with the residual (separable geometry).
//
// Reference: VoxelProjector3D.projectJosephPartial + difference
// (TomoJ_Base/.../projectors/VoxelProjector3D.java:671-821, 414-433) and the
// sampler TomoReconstruction2.getPixel(double,double,int) (TomoReconstruction2.java:154-190).
//
// One CTA owns one projection row j (= volume row r = j - row_off) for a group
// of TG tilts.  It walks the row's XZ plane in chunks of ZC planes: one thread
// stages each chunk with bulk TMA copies (one per plane row, completing on an
// mbarrier), all threads turn it into (v - d, d) pairs so that a bilinear
// sample is one 64-bit shared load and one FMA, and every thread advances its
// 16 rays (TG tilts x QP detector columns) through the chunk.  A ray position is
// 32.32 fixed point whose per-plane step also carries the pair-row pitch, so its
// integer part is directly the shared-memory pair index.  Ray sums accumulate in
// FP32 along z (two interleaved sub-chains per chunk), matching the reference's
// float ray_sum to rounding.  The epilogue writes proj/norm and, when the
// aligned measurement is given, diff = (float)(((e - th) / norm) * factor) and
// the per-row FP64 sum of squared differences.
//
// This header is compiled once per detector-column count per thread (QP) by the
// fp_kernel_q*.cu translation units.
#pragma once
#include <cmath>
#include <type_traits>

#include <cuda_fp16.h>

#include "device_util.cuh"
#include "tomo_internal.h"
#include "vol_storage.cuh"

namespace tomo {
namespace fpk {

constexpr uint32_t kWaitTries = 1u << 24;

struct Smem {
    int PW;
    size_t raw_off, pair_off, red_off, step_off, total;
};

// Shared memory: mbarrier | raw chunk [rows][ZC][W] | pairs [ZC][W+4] | reduction scratch | steps.
// PK (pair kind) 0: FP32 rows and float2 pairs; 1: 16-bit rows and half2 pairs.
__host__ __device__ inline Smem layout(int ZC, int W, int tgmax, int rows = 1, int PK = 0) {
    Smem L;
    L.PW = W + 4;
    size_t o = 16;
    L.raw_off = o;
    o += (size_t)rows * ZC * W * (PK ? sizeof(uint16_t) : sizeof(float));
    o = (o + 15) & ~(size_t)15;
    L.pair_off = o;
    o += (size_t)ZC * L.PW * (PK ? sizeof(uint32_t) : sizeof(float2));
    o = (o + 15) & ~(size_t)15;
    L.red_off = o;
    o += (kFpMaxThreads / 32) * sizeof(double);
    L.step_off = o;
    o += (size_t)tgmax * sizeof(long long);
    L.total = o;
    return L;
}

// Pairs of a plane row: slot k+2 holds the sample at floor(x) = k for k in [-2, W+1]
// as (v_k - d_k, d_k), d_k = v_{k+1} - v_k, so that a bilinear sample with fraction f is
// fma(1 + f, d_k, v_k - d_k).  d = 0 where the reference returns the raw floor voxel
// (last column, last row, last plane) and outside [0, W-1].
//
// A chunk's rows are converted together: the block is laid out as NT / q rows x
// q groups (q groups per row), so a 512-wide row of 128 float4 groups keeps all 256
// threads busy instead of half of them.

// Group m of an FP32 row: pairs 4m .. 4m+3 (W % 4 == 0).
__device__ __forceinline__ void pairs4_f32(const float* __restrict__ src, float2* __restrict__ dst, int W, int m,
                                           bool flat) {
    const float4 v = *reinterpret_cast<const float4*>(src + 4 * m);
    const float nx = (4 * m + 4 < W) ? src[4 * m + 4] : v.w;
    float d0 = v.y - v.x, d1 = v.z - v.y, d2 = v.w - v.z, d3 = nx - v.w;
    if (flat) d0 = d1 = d2 = d3 = 0.0f;
    float4* o = reinterpret_cast<float4*>(dst + 4 * m + 2);
    o[0] = make_float4(v.x - d0, d0, v.y - d1, d1);
    o[1] = make_float4(v.z - d2, d2, v.w - d3, d3);
}

// Pair k of an FP32 row (any W).
__device__ __forceinline__ void pair1_f32(const float* __restrict__ src, float2* __restrict__ dst, int W, int k,
                                          bool flat) {
    const float v = src[k];
    float d = (k + 1 < W) ? src[k + 1] - v : 0.0f;
    if (flat) d = 0.0f;
    dst[k + 2] = make_float2(v - d, d);
}

// The same from a row stored in 16 bits (reduced-precision volume; the slab scale is
// applied to the finished ray sum).
template <int VT>
__device__ __forceinline__ void pairs4_16(const uint16_t* __restrict__ src, float2* __restrict__ dst, int W, int m,
                                          bool flat) {
    const uint2 u = *reinterpret_cast<const uint2*>(src + 4 * m);
    const float vx = vol_load16<VT>((uint16_t)(u.x & 0xFFFFu)), vy = vol_load16<VT>((uint16_t)(u.x >> 16));
    const float vz = vol_load16<VT>((uint16_t)(u.y & 0xFFFFu)), vw = vol_load16<VT>((uint16_t)(u.y >> 16));
    const float nx = (4 * m + 4 < W) ? vol_load16<VT>(src[4 * m + 4]) : vw;
    float d0 = vy - vx, d1 = vz - vy, d2 = vw - vz, d3 = nx - vw;
    if (flat) d0 = d1 = d2 = d3 = 0.0f;
    float4* o = reinterpret_cast<float4*>(dst + 4 * m + 2);
    o[0] = make_float4(vx - d0, d0, vy - d1, d1);
    o[1] = make_float4(vz - d2, d2, vw - d3, d3);
}

template <int VT>
__device__ __forceinline__ void pair1_16(const uint16_t* __restrict__ src, float2* __restrict__ dst, int W, int k,
                                         bool flat) {
    const float v = vol_load16<VT>(src[k]);
    float d = (k + 1 < W) ? vol_load16<VT>(src[k + 1]) - v : 0.0f;
    if (flat) d = 0.0f;
    dst[k + 2] = make_float2(v - d, d);
}

// Half2 pairs of a 16-bit row (PK 1): the pair of slot k is (v_k - d_k, d_k) computed in
// FP32 from the stored values and rounded once to FP16 (both in units of the row's slab
// scale, whose maximum is in [16, 32), so the FP16 range is never left): a sample is one
// 32-bit shared load, two conversions and one FMA, and the gathers move half the bytes.
__device__ __forceinline__ uint32_t hpair(float v, float d) {
    const __half2 h = __floats2half2_rn(v - d, d);
    return *reinterpret_cast<const uint32_t*>(&h);
}

template <int VT>
__device__ __forceinline__ void hpairs4_16(const uint16_t* __restrict__ src, uint32_t* __restrict__ dst, int W, int m,
                                           bool flat) {
    const uint2 u = *reinterpret_cast<const uint2*>(src + 4 * m);
    const float vx = vol_load16<VT>((uint16_t)(u.x & 0xFFFFu)), vy = vol_load16<VT>((uint16_t)(u.x >> 16));
    const float vz = vol_load16<VT>((uint16_t)(u.y & 0xFFFFu)), vw = vol_load16<VT>((uint16_t)(u.y >> 16));
    const float nx = (4 * m + 4 < W) ? vol_load16<VT>(src[4 * m + 4]) : vw;
    float d0 = vy - vx, d1 = vz - vy, d2 = vw - vz, d3 = nx - vw;
    if (flat) d0 = d1 = d2 = d3 = 0.0f;
    // slot 4m + 2 is 8-byte aligned (W + 4 words per row, rows start 16-byte aligned)
    uint2* o = reinterpret_cast<uint2*>(dst + 4 * m + 2);
    o[0] = make_uint2(hpair(vx, d0), hpair(vy, d1));
    o[1] = make_uint2(hpair(vz, d2), hpair(vw, d3));
}

template <int VT>
__device__ __forceinline__ void hpair1_16(const uint16_t* __restrict__ src, uint32_t* __restrict__ dst, int W, int k,
                                          bool flat) {
    const float v = vol_load16<VT>(src[k]);
    float d = (k + 1 < W) ? vol_load16<VT>(src[k + 1]) - v : 0.0f;
    if (flat) d = 0.0f;
    dst[k + 2] = hpair(v, d);
}

// Pair k of a row blended between volume rows r (src0) and r + 1 (src1) with weight
// yf: b = v0 + yf (v1 - v0), then pairs of b.  The reference returns the raw voxel of
// row r (unblended) at the last column, so that slot keeps v0; on the last plane
// (`flat`) every sample is the raw voxel of row r.
__device__ __forceinline__ void pair1_blend(const float* __restrict__ src0, const float* __restrict__ src1, float yf,
                                            float2* __restrict__ dst, int W, int k, bool flat) {
    const float v0 = src0[k];
    float2 pr = make_float2(v0, 0.0f);
    if (!flat && k + 1 < W) {
        const float b = __fadd_rn(v0, __fmul_rn(yf, __fsub_rn(src1[k], v0)));
        const float v0n = src0[k + 1];
        const float bn = __fadd_rn(v0n, __fmul_rn(yf, __fsub_rn(src1[k + 1], v0n)));
        const float d = __fsub_rn(bn, b);
        pr = make_float2(__fsub_rn(b, d), d);
    }
    dst[k + 2] = pr;
}

// Calls fn(zz, m) for every row zz < zc and group m < q, spreading rows over the block.
template <int NT, class Fn>
__device__ __forceinline__ void for_chunk_groups(int zc, int q, Fn fn) {
    const int tid = threadIdx.x;
    if (q <= NT) {
        const int R = NT / q;
        const int r0 = tid / q, m = tid - r0 * q;
        if (r0 < R)
            for (int zz = r0; zz < zc; zz += R) fn(zz, m);
    } else {
        for (int zz = 0; zz < zc; zz++)
            for (int m = tid; m < q; m += NT) fn(zz, m);
    }
}

// All pairs of a staged chunk of zc plane rows.  raw: rows [zc][W] as stored (FP32 or
// 16-bit), raw1: row r + 1 of every plane (blended form); zflat: the chunk row of the
// volume's last plane, or -1.
template <int NT>
__device__ __forceinline__ void build_pairs_chunk(const void* raw, const float* raw1, float2* __restrict__ pairs, int W,
                                                  int PW, int zc, int vt, bool blend, float yf, bool last_row,
                                                  int zflat) {
    const float* r32 = static_cast<const float*>(raw);
    const uint16_t* r16 = static_cast<const uint16_t*>(raw);
    auto flat = [&](int zz) { return last_row || zz == zflat; };
    if (blend) {
        for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
            pair1_blend(r32 + (size_t)zz * W, raw1 + (size_t)zz * W, yf, pairs + (size_t)zz * PW, W, k, flat(zz));
        });
    } else if (vt == kVolF32) {
        if ((W & 3) == 0)
            for_chunk_groups<NT>(zc, W >> 2, [&](int zz, int m) {
                pairs4_f32(r32 + (size_t)zz * W, pairs + (size_t)zz * PW, W, m, flat(zz));
            });
        else
            for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
                pair1_f32(r32 + (size_t)zz * W, pairs + (size_t)zz * PW, W, k, flat(zz));
            });
    } else if (vt == kVolBF16) {
        if ((W & 3) == 0)
            for_chunk_groups<NT>(zc, W >> 2, [&](int zz, int m) {
                pairs4_16<kVolBF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, m, flat(zz));
            });
        else
            for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
                pair1_16<kVolBF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, k, flat(zz));
            });
    } else {
        if ((W & 3) == 0)
            for_chunk_groups<NT>(zc, W >> 2, [&](int zz, int m) {
                pairs4_16<kVolF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, m, flat(zz));
            });
        else
            for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
                pair1_16<kVolF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, k, flat(zz));
            });
    }
    // slots -2, -1, W, W+1 of every row: the edge values with slope 0.  In the blended
    // form x in [-ACCURACY, 0) samples column 0 with weight 0 (the blended value) and
    // slots past the row are never sampled (x < W).
    for (int e = threadIdx.x; e < zc * 4; e += NT) {
        const int zz = e >> 2, t = e & 3;
        const int col = (t < 2) ? 0 : W - 1;
        const size_t o = (size_t)zz * W + col;
        float v;
        if (vt == kVolF32)
            v = r32[o];
        else if (vt == kVolBF16)
            v = vol_load16<kVolBF16>(r16[o]);
        else
            v = vol_load16<kVolF16>(r16[o]);
        if (blend && t < 2 && !flat(zz)) v = __fadd_rn(v, __fmul_rn(yf, __fsub_rn(raw1[o], v)));
        const int k = (t < 2) ? t - 2 : W + t - 2;  // -2, -1, W, W+1
        pairs[(size_t)zz * PW + k + 2] = make_float2(v, 0.0f);
    }
}

// All half2 pairs of a staged chunk of zc 16-bit plane rows (PK 1).
template <int NT>
__device__ __forceinline__ void build_hpairs_chunk(const uint16_t* r16, uint32_t* __restrict__ pairs, int W, int PW,
                                                   int zc, int vt, bool last_row, int zflat) {
    auto flat = [&](int zz) { return last_row || zz == zflat; };
    if (vt == kVolBF16) {
        if ((W & 3) == 0)
            for_chunk_groups<NT>(zc, W >> 2, [&](int zz, int m) {
                hpairs4_16<kVolBF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, m, flat(zz));
            });
        else
            for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
                hpair1_16<kVolBF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, k, flat(zz));
            });
    } else {
        if ((W & 3) == 0)
            for_chunk_groups<NT>(zc, W >> 2, [&](int zz, int m) {
                hpairs4_16<kVolF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, m, flat(zz));
            });
        else
            for_chunk_groups<NT>(zc, W, [&](int zz, int k) {
                hpair1_16<kVolF16>(r16 + (size_t)zz * W, pairs + (size_t)zz * PW, W, k, flat(zz));
            });
    }
    for (int e = threadIdx.x; e < zc * 4; e += NT) {
        const int zz = e >> 2, t = e & 3;
        const int col = (t < 2) ? 0 : W - 1;
        const float v = vol_load16_rt(vt, r16[(size_t)zz * W + col]);
        const int k = (t < 2) ? t - 2 : W + t - 2;  // -2, -1, W, W+1
        pairs[(size_t)zz * PW + k + 2] = hpair(v, 0.0f);
    }
}

__device__ __forceinline__ float sample(const float2* __restrict__ P, long long x) {
    const float2 p = P[(int)(x >> 32)];
    return fmaf(fix_one_plus_frac((uint32_t)x), p.y, p.x);
}

__device__ __forceinline__ float sample(const __half2* __restrict__ P, long long x) {
    const float2 p = __half22float2(P[(int)(x >> 32)]);
    return fmaf(fix_one_plus_frac((uint32_t)x), p.y, p.x);
}

// Detector column of ray slot (t, q) of thread tid: warps own blocks of 32 consecutive
// columns (contiguous shared-memory reads).
template <int NT, int QP>
__device__ __forceinline__ int ray_column(int t, int q, int tid) {
    (void)t;
    return tid + q * NT;
}

// Partial chunk of one ray (it enters or leaves the volume inside the chunk):
// branch-free, the load is predicated and an out-of-range sample adds fma(F, 0, 0) = 0.
// Kept out of line: it is rare, and inlining it for every ray slot bloats the
// instruction footprint of the sampling loop.
struct PartialOut {
    long long x;
    float s;
};
__device__ __forceinline__ float2 pair_at(const float2* __restrict__ P, long long x) { return P[(int)(x >> 32)]; }
__device__ __forceinline__ float2 pair_at(const __half2* __restrict__ P, long long x) {
    return __half22float2(P[(int)(x >> 32)]);
}

template <class PT>
static __device__ __noinline__ PartialOut partial_chunk(const PT* __restrict__ P, long long x, long long step, int lo,
                                                        int cnt, int zc) {
    float s = 0.0f;
    for (int zz = 0; zz < zc; zz++) {
        const bool in = (unsigned)(zz - lo) < (unsigned)cnt;
        float2 p = make_float2(0.0f, 0.0f);
        if (in) p = pair_at(P, x);
        s += fmaf(fix_one_plus_frac((uint32_t)x), p.y, p.x);
        x += step;
    }
    return PartialOut{x, s};
}

// Full chunk of one ray (all ZC planes inside): two interleaved sub-chains (even / odd
// planes).  Returns the position after ZC steps and the chunk's sum.
template <int ZC, class PT>
__device__ __forceinline__ PartialOut full_chunk_inl(const PT* __restrict__ P, long long x, long long step) {
    const long long s2 = 2 * step;
    long long x0 = x, x1 = x + step;
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (int zz = 0; zz < ZC; zz += 2) {
        a0 += sample(P, x0);
        a1 += sample(P, x1);
        x0 += s2;
        x1 += s2;
    }
    return PartialOut{x0, a0 + a1};
}

// One CTA's work: projection row j, tilts [g0, g0 + tilts_per_cta) of problem `a`,
// depth part zp of a.zparts.
// BLEND: the fractional-row form (row maps, two staged rows per plane).  A separate
// instantiation, so that the whole-row kernels compile without any of it.
// PK: pair kind (0: FP32 volume, float2 pairs; 1: 16-bit volume, half2 pairs).
// Returns false when a bounded wait ran out (the CTA recorded it and has nothing in
// flight); with `retire` the chunk mbarrier is invalidated at the end so that a persistent
// CTA can initialise it again for its next work item.
template <int NT, int QP, int ZC, bool BLEND, int PK>
__device__ __forceinline__ bool fp_body(const FpLaunch& a, const int g0, const int j, const int use_tma,
                                        const int zp, const bool retire = false) {
    static_assert(!(BLEND && PK), "the fractional-row form is FP32 only");
    using PairT = typename std::conditional<PK == 1, __half2, float2>::type;
    constexpr int TGMAX = kFpRays / QP > 0 ? kFpRays / QP : 1;
    constexpr int NR = TGMAX * QP;
    extern __shared__ __align__(16) unsigned char smem[];
    const Smem L = layout(ZC, a.W, TGMAX, BLEND ? 2 : 1, PK);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    float* raw = reinterpret_cast<float*>(smem + L.raw_off);
    PairT* pairs = reinterpret_cast<PairT*>(smem + L.pair_off);
    double* red = reinterpret_cast<double*>(smem + L.red_off);
    long long* s_step = reinterpret_cast<long long*>(smem + L.step_off);

    const int tid = threadIdx.x;
    const int W = a.W, H = a.H, D = a.D, w = a.w, h = a.h;
    const int PW = L.PW;
    const int TG = min(a.tilts_per_cta, a.T - g0);
    const int r = BLEND ? a.rowmap[j] : j - a.row_off;
    const bool row_in = (r >= 0 && r < H);
    const float yf = BLEND ? a.rowyf[j] : 0.0f;
    // blend rows r and r + 1 (the raw floor voxel rule makes the last row unblended)
    const bool blend = BLEND && yf != 0.0f && r < H - 1;
    // chunks [c_begin, c_end) of the plane stack belong to this depth part
    const int P = a.zparts > 1 ? a.zparts : 1;
    const int nch_all = (D + ZC - 1) / ZC;
    const int cpp = (nch_all + P - 1) / P;
    const int c_begin = min(nch_all, zp * cpp);
    const int c_end = min(nch_all, c_begin + cpp);

    // ray k = t * QP + q: tilt g0 + t, detector column ray_column(t, q, tid)
    long long X[NR];
    float acc[NR];
    int zab[NR];
#pragma unroll
    for (int k = 0; k < NR; k++) {
        const int t = k / QP, q = k % QP;
        const int i = ray_column<NT, QP>(t, q, tid);
        acc[k] = 0.0f;
        X[k] = 0;
        zab[k] = 0;
        if (t < TG) {
            const int tilt = a.tilts[g0 + t];
            if (tid == 0 && q == 0) s_step[t] = a.ftilt[tilt].step;
            if (i < w && row_in) {
                const FpRay ray = a.rays[(size_t)tilt * w + i];
                X[k] = ray.X0 + (long long)(c_begin * ZC) * a.ftilt[tilt].step;
                zab[k] = ray.zab;
            }
        } else if (tid == 0 && q == 0) {
            s_step[t] = 0;
        }
    }

    if (row_in && c_begin < c_end) {
        const bool last_row = (r == H - 1);
        const long long pitch = (long long)PW << 32;  // one pair row in position units
        const int vt = a.vtype;
        const uint32_t rowb = (uint32_t)(W * vol_elem_bytes(vt));  // bytes of one plane row
        const unsigned char* volb = static_cast<const unsigned char*>(a.vol);
        unsigned char* rawb = reinterpret_cast<unsigned char*>(raw);
        float* raw1 = BLEND ? raw + (size_t)ZC * W : nullptr;  // row r + 1 of every plane (blended rows)
        auto stage = [&](int c) {  // chunk c -> raw
            const int z0 = c * ZC, zn = min(ZC, D - z0);
            if (use_tma) {
                if (tid == 0) {
                    fence_proxy_async();
                    mbar_arrive_expect_tx(bar, (uint32_t)zn * rowb * (BLEND && blend ? 2u : 1u));
                    // test hook: the first chunk's copies are held back (its wait runs out)
                    const int issue = (a.hold_first_copy && c == c_begin) ? 0 : zn;
                    for (int zz = 0; zz < issue; zz++) {
                        tma_load_1d(rawb + (size_t)zz * rowb, volb + ((size_t)(z0 + zz) * H + r) * rowb, rowb, bar);
                        if (BLEND && blend)
                            tma_load_1d(raw1 + (size_t)zz * W, volb + ((size_t)(z0 + zz) * H + r + 1) * rowb, rowb,
                                        bar);
                    }
                }
            } else if (vt == kVolF32) {
                for (int zz = 0; zz < zn; zz++) {
                    const float* src = reinterpret_cast<const float*>(volb + ((size_t)(z0 + zz) * H + r) * rowb);
                    for (int k = tid; k < W; k += NT) raw[(size_t)zz * W + k] = src[k];
                    if (BLEND && blend) {
                        const float* s1 = src + (size_t)W;
                        for (int k = tid; k < W; k += NT) raw1[(size_t)zz * W + k] = s1[k];
                    }
                }
            } else {
                uint16_t* raw16 = reinterpret_cast<uint16_t*>(raw);
                for (int zz = 0; zz < zn; zz++) {
                    const uint16_t* src = reinterpret_cast<const uint16_t*>(volb + ((size_t)(z0 + zz) * H + r) * rowb);
                    for (int k = tid; k < W; k += NT) raw16[(size_t)zz * W + k] = src[k];
                }
            }
        };
        if (use_tma && tid == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        stage(c_begin);
        for (int c = c_begin; c < c_end; c++) {
            const int z0 = c * ZC;
            const int zc = min(ZC, D - z0);
            const uint32_t parity = (uint32_t)((c - c_begin) & 1);
            if (use_tma) {
                const bool held = a.hold_first_copy && c == c_begin;  // nothing was issued for it
                const bool ok = mbar_wait_bounded(bar, parity, held ? kHoldWaitTries : kWaitTries);
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) atomicOr(a.status, kStatusTimeout);
                    // let any copy still in flight land before the CTA's shared memory is released
                    if (!held) mbar_wait_bounded(bar, parity, kWaitTries);
                    return false;
                }
            } else {
                __syncthreads();
            }
            if (PK == 1)
                build_hpairs_chunk<NT>(reinterpret_cast<const uint16_t*>(raw), reinterpret_cast<uint32_t*>(pairs), W, PW,
                                   zc, vt, last_row, D - 1 - z0 < zc ? D - 1 - z0 : -1);
            else
                build_pairs_chunk<NT>(raw, raw1, reinterpret_cast<float2*>(pairs), W, PW, zc, vt, BLEND && blend, yf,
                                  last_row, D - 1 - z0 < zc ? D - 1 - z0 : -1);
            __syncthreads();
            if (c + 1 < c_end && use_tma) stage(c + 1);
            const PairT* P = pairs + 2;
            // ray slot k over this chunk: full (unrolled chains), none (skip) or partial
            auto one = [&](int k) {
                const long long st = s_step[k / QP];
                const int za = zab[k] & 0xFFFF;
                const int cnt = (int)((uint32_t)zab[k] >> 16);
                const bool full = (za <= z0) && (za + cnt >= z0 + zc);
                const bool none = (cnt == 0) || (za + cnt <= z0) || (za >= z0 + zc);
                if (__all_sync(0xffffffffu, full) && zc == ZC) {
                    if (ZC >= 2) {
                        const PartialOut fo = full_chunk_inl<ZC>(P, X[k], st + pitch);
                        X[k] = fo.x - (long long)ZC * pitch;
                        acc[k] += fo.s;
                    } else {
                        acc[k] += sample(P, X[k]);
                        X[k] += st;
                    }
                } else if (__all_sync(0xffffffffu, none)) {
                    X[k] += (long long)zc * st;
                } else {
                    const PartialOut po = partial_chunk(P, X[k], st + pitch, za - z0, cnt, zc);
                    X[k] = po.x - (long long)zc * pitch;
                    acc[k] += po.s;
                }
            };
#pragma unroll
            for (int k = 0; k < NR; k++) {
                if (k / QP >= TG) break;  // uniform: tilt slot past the batch
                one(k);
            }
            __syncthreads();
            if (c + 1 < c_end && !use_tma) stage(c + 1);
        }
        if (retire && use_tma && tid == 0) mbar_inval(bar);  // every phase has completed
    }

    // Depth split: publish this part's sums; the last part to arrive adds all parts in
    // order (deterministic) and runs the epilogue.
    if (P > 1) {
        __shared__ int s_last;
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const int t = k / QP, q = k % QP;
            const int i = ray_column<NT, QP>(t, q, tid);
            if (t < TG && i < w) a.part[(((size_t)zp * a.T + g0 + t) * h + j) * w + i] = acc[k];
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            unsigned* tk = a.tickets + (size_t)(g0 / a.tilts_per_cta) * h + j;
            const unsigned ticket = atomicAdd(tk, 1u);
            s_last = (ticket == (unsigned)(P - 1));
            if (s_last) *tk = 0u;  // every part has arrived: ready for the next launch
        }
        __syncthreads();
        if (!s_last) return true;
        __threadfence();
#pragma unroll
        for (int k = 0; k < NR; k++) {
            const int t = k / QP, q = k % QP;
            const int i = ray_column<NT, QP>(t, q, tid);
            float sum = 0.0f;
            if (t < TG && i < w)
                for (int pp = 0; pp < P; pp++) sum += __ldcg(a.part + (((size_t)pp * a.T + g0 + t) * h + j) * w + i);
            acc[k] = sum;
        }
    }

    // Epilogue: projection, norm, residual.
    const int lane = tid & 31, warp = tid >> 5;
    // reduced storage: ray sums are in units of the row's slab scale (a power of two)
    const double vsc = (a.vscale != nullptr && row_in) ? (double)a.vscale[r] : 1.0;
#pragma unroll
    for (int t = 0; t < TGMAX; t++) {
        if (t >= TG) break;
        const int tilt = a.tilts[g0 + t];
        const double ninc = a.ftilt[tilt].ninc;
        double e2 = 0.0;
#pragma unroll
        for (int q = 0; q < QP; q++) {
            const int i = ray_column<NT, QP>(t, q, tid);
            if (i >= w) continue;
            const int cnt = (int)((uint32_t)zab[t * QP + q] >> 16);
            float th, nrm;
            if (cnt == 0) {
                th = __int_as_float(0x7fc00000);
                nrm = 0.0f;
            } else {
                th = (a.vscale != nullptr) ? __double2float_rn((double)acc[t * QP + q] * vsc * ninc)
                                           : __double2float_rn((double)acc[t * QP + q] * ninc);
                nrm = a.rays[(size_t)tilt * w + i].norm;
            }
            const size_t o = ((size_t)(g0 + t) * h + j) * w + i;
            a.proj[o] = th;
            a.norm[o] = nrm;
            if (a.meas != nullptr) {
                const float e = a.meas[((size_t)tilt * h + j) * w + i];
                float d = 0.0f;
                if (!isnan(e) && !isnan(th)) {
                    const float qv = __fdiv_rn(__fsub_rn(e, th), nrm);
                    const double v = (double)qv * a.factor;
                    d = __double2float_rn(v);
                    e2 += v * v;
                }
                a.diff[o] = d;
            }
        }
        if (a.meas != nullptr) {
            e2 = warp_sum(e2);
            if (lane == 0) red[warp] = e2;
            __syncthreads();
            if (tid == 0) {
                double sum = 0.0;
                for (int k = 0; k < NT / 32; k++) sum += red[k];
                a.errpart[(size_t)(g0 + t) * h + j] = sum;
            }
            __syncthreads();
        }
    }
    return true;
}

template <int NT, int QP, int ZC, bool BLEND, int PK>
__global__ void __launch_bounds__(NT, fp_ctas_per_sm(NT)) fp_kernel(const __grid_constant__ FpLaunch a, int use_tma) {
    fp_body<NT, QP, ZC, BLEND, PK>(a, blockIdx.x * a.tilts_per_cta, a.j0 + blockIdx.y, use_tma, blockIdx.z);
}

// Batched form: CTA b works on item {problem, first tilt, row, use_tma} of many problems
// (all of pair kind PK: FP32 and 16-bit volumes go to separate launches).
template <int NT, int QP, int ZC, int PK>
__global__ void __launch_bounds__(NT, fp_ctas_per_sm(NT))
    fp_kernel_batch(const FpLaunch* __restrict__ descs, const int4* __restrict__ items) {
    const int4 it = items[blockIdx.x];
    fp_body<NT, QP, ZC, false, PK>(descs[it.x], it.y, it.z, it.w, 0);
}

// Persistent batched form: a resident grid whose CTAs take work items {problem, first
// tilt, row, flags} in list order through an atomic cursor until the list runs out, so a
// forward phase of a batch is one launch per block size and chunk depth whatever the
// members' widths and storage types: the item's flags select the body (bit 0 bulk
// copies, bits 1-3 log2 of the detector columns per thread QP, bit 4 16-bit pairs).  The
// host orders the list by decreasing work, so the last items to start are the shortest.
// A bounded wait that runs out ends the CTA (recorded in the problem's status word).
template <int NT>
struct FpPersistQP;
template <>
struct FpPersistQP<256> {
    static constexpr int lo = 0, hi = 1;  // QP 1, 2
};
template <>
struct FpPersistQP<512> {
    static constexpr int lo = 1, hi = 3;  // QP 2, 4, 8
};

// One work item as a call of its own: each body keeps the register allocation and
// instruction schedule it has as a kernel (inlined into the item loop it ran slower).
template <int NT, int QP, int ZC, int PK>
__device__ __noinline__ bool fp_item_call(const FpLaunch* a, int g0, int j, int use_tma) {
    return fp_body<NT, QP, ZC, false, PK>(*a, g0, j, use_tma, 0, true);
}

template <int NT, int ZC, int LQ>
__device__ __forceinline__ bool fp_persist_item(const FpLaunch* a, int g0, int j, int use_tma, int lq, int pk) {
    if constexpr (LQ > FpPersistQP<NT>::hi) {
        return true;
    } else {
        if (lq == LQ)
            return pk ? fp_item_call<NT, 1 << LQ, ZC, 1>(a, g0, j, use_tma)
                      : fp_item_call<NT, 1 << LQ, ZC, 0>(a, g0, j, use_tma);
        return fp_persist_item<NT, ZC, LQ + 1>(a, g0, j, use_tma, lq, pk);
    }
}

template <int NT, int ZC>
__global__ void __launch_bounds__(NT, fp_ctas_per_sm(NT))
    fp_kernel_persist(const FpLaunch* __restrict__ descs, const int4* __restrict__ items, int n_items,
                      int* __restrict__ cursor) {
    __shared__ int s_item;
    int next = 0;  // thread 0: the item after the current one, fetched while it runs
    if (threadIdx.x == 0) next = atomicAdd(cursor, 1);
    for (;;) {
        if (threadIdx.x == 0) s_item = next;
        __syncthreads();
        const int i = s_item;
        if (i >= n_items) return;
        if (threadIdx.x == 0) next = atomicAdd(cursor, 1);
        const int4 it = items[i];
        const int f = it.w;
        if (!fp_persist_item<NT, ZC, FpPersistQP<NT>::lo>(descs + it.x, it.y, it.z, f & 1, (f >> 1) & 7, (f >> 4) & 1))
            return;
        __syncthreads();  // shared memory (and s_item) are free for the next item
    }
}

template <int NT, int ZC>
cudaError_t persist_attr() {
    return cudaFuncSetAttribute(fp_kernel_persist<NT, ZC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fp_smem_budget(NT));
}

template <int NT, int ZC>
void persist_launch(const FpLaunch* descs, const int4* items, int n_items, int* cursor, int grid, size_t smem,
                    cudaStream_t s) {
    fp_kernel_persist<NT, ZC><<<grid, NT, smem, s>>>(descs, items, n_items, cursor);
}

template <int NT, int QP, int ZC>
cudaError_t set_attr_one() {
    const int m = (int)fp_smem_budget(NT);
    cudaError_t e = cudaFuncSetAttribute(fp_kernel<NT, QP, ZC, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fp_kernel<NT, QP, ZC, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fp_kernel<NT, QP, ZC, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fp_kernel_batch<NT, QP, ZC, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fp_kernel_batch<NT, QP, ZC, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

template <int NT, int QP>
cudaError_t set_attr_qp() {
    cudaError_t e;
    if ((e = set_attr_one<NT, QP, 16>()) != cudaSuccess) return e;
    if ((e = set_attr_one<NT, QP, 8>()) != cudaSuccess) return e;
    if ((e = set_attr_one<NT, QP, 4>()) != cudaSuccess) return e;
    if ((e = set_attr_one<NT, QP, 2>()) != cudaSuccess) return e;
    return set_attr_one<NT, QP, 1>();
}

template <int NT, int QP, int ZC>
void launch_zc(const FpLaunch& a, dim3 grid, size_t smem, int use_tma, cudaStream_t s) {
    if (a.two_rows) fp_kernel<NT, QP, ZC, true, 0><<<grid, NT, smem, s>>>(a, use_tma);
    else if (a.vtype != kVolF32) fp_kernel<NT, QP, ZC, false, 1><<<grid, NT, smem, s>>>(a, use_tma);
    else fp_kernel<NT, QP, ZC, false, 0><<<grid, NT, smem, s>>>(a, use_tma);
}

template <int NT, int QP>
cudaError_t launch_qp(const FpLaunch& a, cudaStream_t s) {
    const int rows = a.two_rows ? 2 : 1;
    const int PK = a.vtype != kVolF32 ? 1 : 0;
    if (PK && a.two_rows) return cudaErrorInvalidValue;
    const int ZC = fp_choose_zc(a.W, rows, a.vtype, NT);
    const Smem L = layout(ZC, a.W, kFpRays / QP > 0 ? kFpRays / QP : 1, rows, PK);
    if (L.total > fp_smem_budget(NT)) return cudaErrorInvalidValue;
    const int use_tma = fp_use_tma(a.W, a.vtype, a.vol);
    dim3 grid((a.T + a.tilts_per_cta - 1) / a.tilts_per_cta, a.j1 - a.j0, a.zparts > 1 ? a.zparts : 1);
    switch (ZC) {
        case 16: launch_zc<NT, QP, 16>(a, grid, L.total, use_tma, s); break;
        case 8: launch_zc<NT, QP, 8>(a, grid, L.total, use_tma, s); break;
        case 4: launch_zc<NT, QP, 4>(a, grid, L.total, use_tma, s); break;
        case 2: launch_zc<NT, QP, 2>(a, grid, L.total, use_tma, s); break;
        default: launch_zc<NT, QP, 1>(a, grid, L.total, use_tma, s); break;
    }
    count_launch();
    return cudaGetLastError();
}

template <int NT, int QP, int PK>
void launch_batch_pk(const FpLaunch* descs, const int4* items, int n_items, int ZC, size_t smem, cudaStream_t s) {
    switch (ZC) {
        case 16: fp_kernel_batch<NT, QP, 16, PK><<<n_items, NT, smem, s>>>(descs, items); break;
        case 8: fp_kernel_batch<NT, QP, 8, PK><<<n_items, NT, smem, s>>>(descs, items); break;
        case 4: fp_kernel_batch<NT, QP, 4, PK><<<n_items, NT, smem, s>>>(descs, items); break;
        case 2: fp_kernel_batch<NT, QP, 2, PK><<<n_items, NT, smem, s>>>(descs, items); break;
        default: fp_kernel_batch<NT, QP, 1, PK><<<n_items, NT, smem, s>>>(descs, items); break;
    }
}

template <int NT, int QP>
cudaError_t launch_batch_qp(const FpLaunch* descs, const int4* items, int n_items, int ZC, size_t smem, int pk,
                            cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    if (smem > fp_smem_budget(NT)) return cudaErrorInvalidValue;
    if (pk) launch_batch_pk<NT, QP, 1>(descs, items, n_items, ZC, smem, s);
    else launch_batch_pk<NT, QP, 0>(descs, items, n_items, ZC, smem, s);
    count_launch();
    return cudaGetLastError();
}

}  // namespace fpk
}  // namespace tomo

// One translation unit per (threads, QP) pair defines these entry points.
#define TOMO_FP_INSTANTIATE(NT, QP)                                                                        \
    namespace tomo {                                                                                       \
    cudaError_t fp_launch_t##NT##_q##QP(const FpLaunch& a, cudaStream_t s) {                               \
        return fpk::launch_qp<NT, QP>(a, s);                                                               \
    }                                                                                                      \
    cudaError_t fp_attr_t##NT##_q##QP() { return fpk::set_attr_qp<NT, QP>(); }                            \
    cudaError_t fp_batch_t##NT##_q##QP(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, \
                                       cudaStream_t s) {                                                   \
        return fpk::launch_batch_qp<NT, QP>(d, it, n, zc, smem, pk, s);                                    \
    }                                                                                                      \
    }
