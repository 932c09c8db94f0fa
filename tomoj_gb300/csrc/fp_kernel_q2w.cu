// Forward-projection kernels for QP = 2 detector columns per thread, 512-thread CTAs
// (see fp_kernel.cuh; a translation unit of its own so that the two compile in parallel).
#include "fp_kernel.cuh"

TOMO_FP_INSTANTIATE(512, 2)
