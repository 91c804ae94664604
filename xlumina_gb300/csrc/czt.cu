// Chirp-z (Bluestein) propagation kernels.
#include "common.cuh"
#include "internal.h"

namespace xl {

cudaError_t czt_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

}  // namespace xl
