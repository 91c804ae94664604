// RS / VRS kernels for Q = 2^4, 2^5, 2^6, 2^7, 2^8 (one translation unit of rs_kernels.cuh).
#include "rs_kernels.cuh"

XL_RS_INSTANTIATE(4)
XL_RS_INSTANTIATE(5)
XL_RS_INSTANTIATE(6)
XL_RS_INSTANTIATE(7)
XL_RS_INSTANTIATE(8)
