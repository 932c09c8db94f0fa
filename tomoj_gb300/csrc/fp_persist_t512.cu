// Persistent batched forward projection for 512-thread CTAs (detector rows of 513 to 4096
// columns): one kernel per chunk depth (16 or 8 planes) serving QP = 2, 4 and 8 and both
// pair kinds (see fp_kernel.cuh).
#include "fp_kernel.cuh"

namespace tomo {

cudaError_t fp_persist_attr_t512() {
    cudaError_t e = fpk::persist_attr<512, 16>();
    if (e != cudaSuccess) return e;
    return fpk::persist_attr<512, 8>();
}

cudaError_t fp_persist_t512(int zc, const FpLaunch* descs, const int4* items, int n_items, int* cursor, int grid,
                            size_t smem, cudaStream_t s) {
    if (zc == 16) fpk::persist_launch<512, 16>(descs, items, n_items, cursor, grid, smem, s);
    else if (zc == 8) fpk::persist_launch<512, 8>(descs, items, n_items, cursor, grid, smem, s);
    else return cudaErrorNotSupported;
    return cudaSuccess;
}

}  // namespace tomo
