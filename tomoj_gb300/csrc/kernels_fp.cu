// Forward-projection dispatch: picks the kernel instantiation for the number of
// detector columns each thread owns (QP = ceil(w / threads)); the kernel itself is in
// fp_kernel.cuh and is compiled once per (threads, QP) pair (fp_kernel_q*.cu).
#include "tomo_internal.h"

namespace tomo {

cudaError_t fp_launch_t256_q1(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_t256_q2(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_t512_q2(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_t512_q4(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_t512_q8(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_attr_t256_q1();
cudaError_t fp_attr_t256_q2();
cudaError_t fp_attr_t512_q2();
cudaError_t fp_attr_t512_q4();
cudaError_t fp_attr_t512_q8();
cudaError_t fp_batch_t256_q1(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, cudaStream_t s);
cudaError_t fp_batch_t256_q2(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, cudaStream_t s);
cudaError_t fp_batch_t512_q2(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, cudaStream_t s);
cudaError_t fp_batch_t512_q4(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, cudaStream_t s);
cudaError_t fp_batch_t512_q8(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, int pk, cudaStream_t s);
cudaError_t fp_persist_attr_t256();
cudaError_t fp_persist_attr_t512();
cudaError_t fp_persist_t256(int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor, int grid,
                            size_t smem, cudaStream_t s);
cudaError_t fp_persist_t512(int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor, int grid,
                            size_t smem, cudaStream_t s);

// Raises the dynamic shared-memory limit of every forward-projector variant once,
// outside any stream capture.
cudaError_t fp_init_attributes() {
    cudaError_t e;
    if ((e = fp_attr_t256_q1()) != cudaSuccess) return e;
    if ((e = fp_attr_t256_q2()) != cudaSuccess) return e;
    if ((e = fp_attr_t512_q2()) != cudaSuccess) return e;
    if ((e = fp_attr_t512_q4()) != cudaSuccess) return e;
    if ((e = fp_persist_attr_t256()) != cudaSuccess) return e;
    if ((e = fp_persist_attr_t512()) != cudaSuccess) return e;
    return fp_attr_t512_q8();
}

bool fp_persist_supported(int nt, int zc) { return (nt == 256 && zc == 16) || (nt == 512 && (zc == 16 || zc == 8)); }

cudaError_t launch_fp_persist(int nt, int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor,
                              int grid, size_t smem, cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    if (!fp_persist_supported(nt, zc) || smem > fp_smem_budget(nt) || grid <= 0) return cudaErrorInvalidValue;
    const cudaError_t e = nt == 256 ? fp_persist_t256(zc, descs, items, n_items, cursor, grid, smem, s)
                                    : fp_persist_t512(zc, descs, items, n_items, cursor, grid, smem, s);
    if (e != cudaSuccess) return e;
    count_launch();
    return cudaGetLastError();
}

int fp_threads(int w) { return w <= 512 ? 256 : 512; }

int fp_qp(int w) {
    const int nt = fp_threads(w);
    const int qp = (w + nt - 1) / nt;
    return qp <= 1 ? 1 : qp <= 2 ? 2 : qp <= 4 ? 4 : qp <= 8 ? 8 : 0;
}

int fp_max_tilts_per_cta(int w) {
    const int qp = fp_qp(w);
    if (qp == 0) return 0;
    return kFpRays / qp > 0 ? kFpRays / qp : 1;
}

// Shared-memory bytes of a CTA for width W and planes per chunk ZC (matches fpk::layout):
// FP32 volumes stage 4-byte voxels and build 8-byte pairs, 16-bit volumes 2-byte voxels
// and 4-byte pairs.
size_t fp_smem_bytes(int ZC, int W, int qp, int rows, int vtype) {
    const bool h = vtype != kVolF32;
    size_t o = 16 + (size_t)rows * ZC * W * (h ? 2 : 4);
    o = (o + 15) & ~(size_t)15;
    o += (size_t)ZC * (W + 4) * (h ? 4 : 8);
    o = (o + 15) & ~(size_t)15;
    o += (kFpMaxThreads / 32) * sizeof(double) + (size_t)(kFpRays / qp > 0 ? kFpRays / qp : 1) * sizeof(long long);
    return o;
}

int fp_choose_zc(int W, int rows, int vtype, int nt) {
    for (int zc = 16; zc > 1; zc >>= 1)
        if (fp_smem_bytes(zc, W, 1, rows, vtype) <= fp_smem_budget(nt)) return zc;
    return 1;
}

#ifndef TOMO_FP_MAX_ZPARTS
#define TOMO_FP_MAX_ZPARTS 8
#endif

int fp_zparts(int ctas, int D, int zc, int sms, int ctas_per_sm) {
    const int slots = ctas_per_sm * sms;  // resident forward-projector CTAs
    if (ctas <= 0 || ctas >= slots) return 1;
    const int nch = (D + zc - 1) / zc;
    // A CTA's time is about (chunks + 1) chunk-times (the +1 is its set-up, first
    // bulk copy and partial-sum exchange), independent of what else runs on its SM:
    // minimise waves x (chunks per part + 1).
    int best = 1;
    long long best_cost = (long long)nch + 1;
    for (int P = 2; P <= TOMO_FP_MAX_ZPARTS && P <= nch; P++) {
        const int cpp = (nch + P - 1) / P;
        const long long waves = ((long long)ctas * P + slots - 1) / slots;
        const long long cost = waves * (cpp + 1);
        if (cost < best_cost) {
            best_cost = cost;
            best = P;
        }
    }
    return best;
}

cudaError_t launch_fp_batch(int qp, int nt, const FpLaunch* descs, const int4* items, int n_items, int zc,
                            size_t smem, int pk, cudaStream_t s) {
    if (nt == 256) {
        if (qp == 1) return fp_batch_t256_q1(descs, items, n_items, zc, smem, pk, s);
        if (qp == 2) return fp_batch_t256_q2(descs, items, n_items, zc, smem, pk, s);
    } else if (nt == 512) {
        switch (qp) {
            case 2: return fp_batch_t512_q2(descs, items, n_items, zc, smem, pk, s);
            case 4: return fp_batch_t512_q4(descs, items, n_items, zc, smem, pk, s);
            case 8: return fp_batch_t512_q8(descs, items, n_items, zc, smem, pk, s);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_fp_separable(const FpLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.j1 <= a.j0) return cudaSuccess;
    const int nt = fp_threads(a.w), qp = fp_qp(a.w);
    if (nt == 256) return qp == 1 ? fp_launch_t256_q1(a, s) : fp_launch_t256_q2(a, s);
    switch (qp) {
        case 2: return fp_launch_t512_q2(a, s);
        case 4: return fp_launch_t512_q4(a, s);
        case 8: return fp_launch_t512_q8(a, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace tomo
