// RS / VRS kernels for Q = 2^9, 2^10 (one translation unit of rs_kernels.cuh).
#include "rs_kernels.cuh"

XL_RS_INSTANTIATE(9)
XL_RS_INSTANTIATE(10)
