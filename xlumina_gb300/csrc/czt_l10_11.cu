// Chirp-z kernels for Bluestein lengths 2^10, 2^11 (one translation unit of czt_kernels.cuh).
#include "czt_kernels.cuh"

XL_CZT_INSTANTIATE(10)
XL_CZT_INSTANTIATE(11)
