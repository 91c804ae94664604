// Chirp-z kernels for Bluestein length 2^13 (one translation unit of czt_kernels.cuh).
#include "czt_kernels.cuh"

XL_CZT_INSTANTIATE(13)
