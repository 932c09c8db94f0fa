// Forward projection fused with the residual (separable geometry).
//
// Reference: VoxelProjector3D.projectJosephPartial + difference
// (TomoJ_Base/.../projectors/VoxelProjector3D.java:671-821, 414-433) and the
// sampler TomoReconstruction2.getPixel(double,double,int) (TomoReconstruction2.java:154-190).
//
// One CTA owns one projection row j (= volume row r = j - row_off) for a group
// of TG tilts.  It walks the row's XZ plane in z-chunks of ZC planes: a single
// thread stages each chunk with bulk TMA copies (one per plane row, completing
// on an mbarrier), all threads turn it into (value, slope) pairs so a bilinear
// sample is one 64-bit shared load + one FMA, and every thread advances its
// rays (TG tilts x QP detector columns) through the chunk in 32.32 fixed point.
// Ray sums accumulate in FP32 in z order, like the reference's float ray_sum.
// The epilogue writes proj/norm and, when the aligned measurement is given,
// diff = (float)(((e - th) / norm) * factor) and the per-row FP64 sum of
// squared differences.
#include <cmath>

#include "device_util.cuh"
#include "tomo_internal.h"

namespace tomo {
namespace {

constexpr int kFpThreads = 256;
constexpr uint32_t kWaitTries = 1u << 24;
constexpr size_t kFpMaxSmem = 112 * 1024;  // two CTAs per SM


struct FpSmem {
    int ZC, W, PW;
    size_t raw_off, pair_off, red_off, step_off, total;
};

__host__ __device__ inline FpSmem fp_smem_layout(int ZC, int W, bool tma, int tgmax) {
    FpSmem L;
    L.ZC = ZC;
    L.W = W;
    L.PW = W + 2;
    size_t o = 16;  // mbarrier
    L.raw_off = o;
    if (tma) o += (size_t)ZC * W * sizeof(float);
    o = (o + 15) & ~(size_t)15;
    L.pair_off = o;
    o += (size_t)ZC * L.PW * sizeof(float2);
    o = (o + 15) & ~(size_t)15;
    L.red_off = o;
    o += (kFpThreads / 32) * sizeof(double);
    L.step_off = o;
    o += (size_t)tgmax * sizeof(long long);
    L.total = o;
    return L;
}

template <int QP, int TGMAX, bool USE_TMA>
__global__ void __launch_bounds__(kFpThreads, 2) fp_separable_kernel(FpLaunch a, int ZC) {
    extern __shared__ __align__(16) unsigned char smem[];
    const FpSmem L = fp_smem_layout(ZC, a.W, USE_TMA, TGMAX);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    float* raw = reinterpret_cast<float*>(smem + L.raw_off);
    float2* pairs = reinterpret_cast<float2*>(smem + L.pair_off);
    double* red = reinterpret_cast<double*>(smem + L.red_off);
    long long* s_step = reinterpret_cast<long long*>(smem + L.step_off);

    const int tid = threadIdx.x;
    const int W = a.W, H = a.H, D = a.D, w = a.w, h = a.h;
    const int PW = L.PW;
    const int j = a.j0 + blockIdx.y;
    const int g0 = blockIdx.x * a.tilts_per_cta;
    const int TG = min(a.tilts_per_cta, a.T - g0);
    const int r = j - a.row_off;
    const bool row_in = (r >= 0 && r < H);

    long long X[TGMAX][QP];
    float acc[TGMAX][QP];
    int zab[TGMAX][QP];
#pragma unroll
    for (int t = 0; t < TGMAX; t++) {
        int tilt = (t < TG) ? a.tilts[g0 + t] : 0;
        if (tid == 0 && t < TG) s_step[t] = a.ftilt[tilt].step;
#pragma unroll
        for (int q = 0; q < QP; q++) {
            const int i = tid + q * kFpThreads;
            acc[t][q] = 0.0f;
            X[t][q] = 0;
            zab[t][q] = 0;
            if (t < TG && i < w && row_in) {
                const FpRay ray = a.rays[(size_t)tilt * w + i];
                X[t][q] = ray.X0;
                zab[t][q] = ray.zab;
            }
        }
    }

    if (row_in) {
        const int nchunks = (D + ZC - 1) / ZC;
        const bool last_row = (r == H - 1);
        if (USE_TMA) {
            if (tid == 0) {
                mbar_init(bar, 1);
                fence_mbar_init();
            }
            __syncthreads();
            if (tid == 0) {
                const int zc = min(ZC, D);
                mbar_arrive_expect_tx(bar, (uint32_t)(zc * W * sizeof(float)));
                for (int zz = 0; zz < zc; zz++)
                    tma_load_1d(raw + (size_t)zz * W, a.vol + ((size_t)zz * H + r) * W, W * sizeof(float), bar);
            }
        } else {
            __syncthreads();
        }
        for (int c = 0; c < nchunks; c++) {
            const int z0 = c * ZC;
            const int zc = min(ZC, D - z0);
            if (USE_TMA) {
                const bool ok = mbar_wait_bounded(bar, (uint32_t)(c & 1), kWaitTries);
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) atomicOr(a.status, kStatusTimeout);
                    // let any copy still in flight land before the CTA's shared memory is released
                    mbar_wait_bounded(bar, (uint32_t)(c & 1), kWaitTries);
                    return;
                }
            }
            // (value, slope) pairs; index k+1 holds the sample at floor(x) = k, k in [-1, W]
            // (k = -1 and k = W absorb fixed-point rounding at the volume borders).
            for (int zz = 0; zz < zc; zz++) {
                const bool flat = last_row || (z0 + zz == D - 1);  // raw floor voxel on the last row / plane
                const float* src = USE_TMA ? raw + (size_t)zz * W : a.vol + ((size_t)(z0 + zz) * H + r) * W;
                float2* dst = pairs + (size_t)zz * PW;
                for (int k = tid - 1; k <= W; k += kFpThreads) {
                    float v0, d = 0.0f;
                    if (k < 0) {
                        v0 = src[0];
                    } else if (k >= W - 1) {
                        v0 = src[W - 1];
                    } else {
                        v0 = src[k];
                        if (!flat) d = src[k + 1] - v0;
                    }
                    dst[k + 1] = make_float2(v0, d);
                }
            }
            __syncthreads();
            if (USE_TMA && tid == 0 && c + 1 < nchunks) {
                fence_proxy_async();
                const int zn = min(ZC, D - (z0 + ZC));
                mbar_arrive_expect_tx(bar, (uint32_t)(zn * W * sizeof(float)));
                for (int zz = 0; zz < zn; zz++)
                    tma_load_1d(raw + (size_t)zz * W, a.vol + ((size_t)(z0 + ZC + zz) * H + r) * W,
                                W * sizeof(float), bar);
            }
#pragma unroll
            for (int t = 0; t < TGMAX; t++) {
                if (t >= TG) break;
                const long long step = s_step[t];
#pragma unroll
                for (int q = 0; q < QP; q++) {
                    const int za = zab[t][q] & 0xFFFF;
                    const int cnt = (int)((uint32_t)zab[t][q] >> 16);
                    const bool full = (za <= z0) && (za + cnt >= z0 + zc);
                    const bool none = (cnt == 0) || (za + cnt <= z0) || (za >= z0 + zc);
                    long long x = X[t][q];
                    float s = acc[t][q];
                    if (__all_sync(0xffffffffu, full) && zc == ZC) {
#pragma unroll 4
                        for (int zz = 0; zz < ZC; zz++) {
                            const float2 p = pairs[zz * PW + (int)(x >> 32) + 1];
                            s += fmaf(fix_frac((uint32_t)x), p.y, p.x);
                            x += step;
                        }
                    } else if (__all_sync(0xffffffffu, none)) {
                        x += (long long)zc * step;
                    } else {
                        for (int zz = 0; zz < zc; zz++) {
                            if ((unsigned)(z0 + zz - za) < (unsigned)cnt) {
                                const float2 p = pairs[zz * PW + (int)(x >> 32) + 1];
                                s += fmaf(fix_frac((uint32_t)x), p.y, p.x);
                            }
                            x += step;
                        }
                    }
                    X[t][q] = x;
                    acc[t][q] = s;
                }
            }
            __syncthreads();
        }
    }

    // Epilogue: projection, norm, residual.
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int t = 0; t < TGMAX; t++) {
        if (t >= TG) break;
        const int tilt = a.tilts[g0 + t];
        const double ninc = a.ftilt[tilt].ninc;
        double e2 = 0.0;
#pragma unroll
        for (int q = 0; q < QP; q++) {
            const int i = tid + q * kFpThreads;
            if (i >= w) continue;
            const int cnt = (int)((uint32_t)zab[t][q] >> 16);
            float th, nrm;
            if (cnt == 0) {
                th = __int_as_float(0x7fc00000);
                nrm = 0.0f;
            } else {
                th = __double2float_rn((double)acc[t][q] * ninc);
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
                for (int k = 0; k < kFpThreads / 32; k++) sum += red[k];
                a.errpart[(size_t)(g0 + t) * h + j] = sum;
            }
            __syncthreads();
        }
    }
}

template <int QP, int TGMAX>
cudaError_t set_attr() {
    cudaError_t e = cudaFuncSetAttribute(fp_separable_kernel<QP, TGMAX, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFpMaxSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fp_separable_kernel<QP, TGMAX, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kFpMaxSmem);
}

template <int QP, int TGMAX>
cudaError_t launch_qp(const FpLaunch& a, cudaStream_t s, bool tma) {
    const int ZC = max(1, min(a.D, 8192 / max(a.W, 1)));
    const FpSmem L = fp_smem_layout(ZC, a.W, tma, TGMAX);
    dim3 grid((a.T + a.tilts_per_cta - 1) / a.tilts_per_cta, a.j1 - a.j0);
    if (L.total > kFpMaxSmem) return cudaErrorInvalidValue;
    if (tma)
        fp_separable_kernel<QP, TGMAX, true><<<grid, kFpThreads, L.total, s>>>(a, ZC);
    else
        fp_separable_kernel<QP, TGMAX, false><<<grid, kFpThreads, L.total, s>>>(a, ZC);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

// Raises the dynamic shared-memory limit of every forward-projector variant once,
// outside any stream capture.
cudaError_t fp_init_attributes() {
    cudaError_t e;
    if ((e = set_attr<1, 16>()) != cudaSuccess) return e;
    if ((e = set_attr<2, 8>()) != cudaSuccess) return e;
    if ((e = set_attr<4, 4>()) != cudaSuccess) return e;
    if ((e = set_attr<8, 2>()) != cudaSuccess) return e;
    return set_attr<16, 1>();
}

int fp_max_tilts_per_cta(int w) {
    const int qp = (w + kFpThreads - 1) / kFpThreads;
    if (qp <= 1) return 16;
    if (qp <= 2) return 8;
    if (qp <= 4) return 4;
    if (qp <= 8) return 2;
    if (qp <= 16) return 1;
    return 0;
}

cudaError_t launch_fp_separable(const FpLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.j1 <= a.j0) return cudaSuccess;
    const bool tma = (a.W % 4 == 0) && ((reinterpret_cast<uintptr_t>(a.vol) & 15) == 0);
    const int qp = (a.w + kFpThreads - 1) / kFpThreads;
    if (qp <= 1) return launch_qp<1, 16>(a, s, tma);
    if (qp <= 2) return launch_qp<2, 8>(a, s, tma);
    if (qp <= 4) return launch_qp<4, 4>(a, s, tma);
    if (qp <= 8) return launch_qp<8, 2>(a, s, tma);
    if (qp <= 16) return launch_qp<16, 1>(a, s, tma);
    return cudaErrorInvalidValue;
}

}  // namespace tomo
