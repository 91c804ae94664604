// Chirp-z kernels for Bluestein lengths 2^5, 2^6, 2^7, 2^8, 2^9 (one translation unit of czt_kernels.cuh).
#include "czt_kernels.cuh"

XL_CZT_INSTANTIATE(5)
XL_CZT_INSTANTIATE(6)
XL_CZT_INSTANTIATE(7)
XL_CZT_INSTANTIATE(8)
XL_CZT_INSTANTIATE(9)
