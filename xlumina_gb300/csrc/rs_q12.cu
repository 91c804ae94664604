// RS / VRS kernels for Q = 2^12 (one translation unit of rs_kernels.cuh).
#include "rs_kernels.cuh"

XL_RS_INSTANTIATE(12)
