// Forward-projection kernels for QP = 1 detector columns per thread (see fp_kernel.cuh).
#include "fp_kernel.cuh"

TOMO_FP_INSTANTIATE(256, 1)
