// Forward-projection kernels for QP = 8 detector columns per thread (see fp_kernel.cuh).
#include "fp_kernel.cuh"

TOMO_FP_INSTANTIATE(512, 8)
