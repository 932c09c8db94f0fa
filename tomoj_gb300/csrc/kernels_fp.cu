// Forward-projection dispatch: picks the kernel instantiation for the number of
// detector columns each thread owns (QP = ceil(w / 256)); the kernel itself is in
// fp_kernel.cuh and is compiled once per QP (fp_kernel_q*.cu).
#include "tomo_internal.h"

namespace tomo {

cudaError_t fp_launch_q1(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_q2(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_q4(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_q8(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_launch_q16(const FpLaunch& a, cudaStream_t s);
cudaError_t fp_attr_q1();
cudaError_t fp_attr_q2();
cudaError_t fp_attr_q4();
cudaError_t fp_attr_q8();
cudaError_t fp_attr_q16();
cudaError_t fp_batch_q1(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, cudaStream_t s);
cudaError_t fp_batch_q2(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, cudaStream_t s);
cudaError_t fp_batch_q4(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, cudaStream_t s);
cudaError_t fp_batch_q8(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, cudaStream_t s);
cudaError_t fp_batch_q16(const FpLaunch* d, const int4* it, int n, int zc, size_t smem, cudaStream_t s);

namespace {
constexpr int kFpThreads = 256;
}

// Raises the dynamic shared-memory limit of every forward-projector variant once,
// outside any stream capture.
cudaError_t fp_init_attributes() {
    cudaError_t e;
    if ((e = fp_attr_q1()) != cudaSuccess) return e;
    if ((e = fp_attr_q2()) != cudaSuccess) return e;
    if ((e = fp_attr_q4()) != cudaSuccess) return e;
    if ((e = fp_attr_q8()) != cudaSuccess) return e;
    return fp_attr_q16();
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

int fp_qp(int w) {
    const int qp = (w + kFpThreads - 1) / kFpThreads;
    return qp <= 1 ? 1 : qp <= 2 ? 2 : qp <= 4 ? 4 : qp <= 8 ? 8 : qp <= 16 ? 16 : 0;
}

// Shared-memory bytes of a CTA for width W and planes per chunk ZC (matches fpk::layout).
size_t fp_smem_bytes(int ZC, int W, int qp) {
    size_t o = 16 + (size_t)ZC * W * sizeof(float);
    o = (o + 15) & ~(size_t)15;
    o += (size_t)ZC * (W + 4) * sizeof(float2);
    o = (o + 15) & ~(size_t)15;
    o += (kFpThreads / 32) * sizeof(double) + (size_t)(16 / qp) * sizeof(long long);
    return o;
}

int fp_choose_zc(int W) {
    for (int zc = 16; zc > 1; zc >>= 1)
        if (fp_smem_bytes(zc, W, 1) <= 112 * 1024) return zc;
    return 1;
}

cudaError_t launch_fp_batch(int qp, const FpLaunch* descs, const int4* items, int n_items, int zc, size_t smem,
                            cudaStream_t s) {
    switch (qp) {
        case 1: return fp_batch_q1(descs, items, n_items, zc, smem, s);
        case 2: return fp_batch_q2(descs, items, n_items, zc, smem, s);
        case 4: return fp_batch_q4(descs, items, n_items, zc, smem, s);
        case 8: return fp_batch_q8(descs, items, n_items, zc, smem, s);
        case 16: return fp_batch_q16(descs, items, n_items, zc, smem, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_fp_separable(const FpLaunch& a, cudaStream_t s) {
    if (a.T <= 0 || a.j1 <= a.j0) return cudaSuccess;
    const int qp = (a.w + kFpThreads - 1) / kFpThreads;
    if (qp <= 1) return fp_launch_q1(a, s);
    if (qp <= 2) return fp_launch_q2(a, s);
    if (qp <= 4) return fp_launch_q4(a, s);
    if (qp <= 8) return fp_launch_q8(a, s);
    if (qp <= 16) return fp_launch_q16(a, s);
    return cudaErrorInvalidValue;
}

}  // namespace tomo
