// Chirp-z kernels for Bluestein lengths 2^12, 2^13 (one translation unit of czt_kernels.cuh).
#include "czt_kernels.cuh"

XL_CZT_INSTANTIATE(12)
XL_CZT_INSTANTIATE(13)
