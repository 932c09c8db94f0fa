// Persistent batched forward projection for 256-thread CTAs (detector rows of up to 512
// columns): one kernel serving QP = 1 and 2 and both pair kinds (see fp_kernel.cuh).
#include "fp_kernel.cuh"

namespace tomo {

cudaError_t fp_persist_attr_t256() { return fpk::persist_attr<256, 16>(); }

cudaError_t fp_persist_t256(int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor, int grid,
                            size_t smem, cudaStream_t s) {
    if (zc != 16) return cudaErrorNotSupported;
    fpk::persist_launch<256, 16>(descs, items, n_items, cursor, grid, smem, s);
    return cudaSuccess;
}

}  // namespace tomo
