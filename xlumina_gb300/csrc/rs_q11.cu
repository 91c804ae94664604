// RS / VRS kernels for Q = 2^11 (one translation unit of rs_kernels.cuh).
#include "rs_kernels.cuh"

XL_RS_INSTANTIATE(11)
