// Forward-projection kernels for QP = 2 detector columns per thread, 256-thread CTAs
// (see fp_kernel.cuh).
#include "fp_kernel.cuh"

TOMO_FP_INSTANTIATE(256, 2)
