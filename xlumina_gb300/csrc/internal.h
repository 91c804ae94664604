// Host-side helpers shared by the translation units of libxlgb.
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>

#include "xlgb.h"

namespace xl {

// Thread-local last-error string (defined in capi.cu).
void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* where);
int ensure_init();  // uploads twiddle tables to the current device once
constexpr unsigned long long kDefaultWaitLimitNs = 1000000000ull;   // bounded waits: one second
int set_wait_limit(unsigned long long ns);       // xl_set_wait_limit (current device)
int read_status(unsigned int* flag, int clear);  // xl_device_status

// The kernel variant selected for a pass at transform length 2^log2_len
// (xl_set_kernel_variant; defined in capi.cu).
int kernel_variant(int pass, int log2_len);

inline int ilog2_ceil(long long v) {
  int l = 0;
  while ((1LL << l) < v) ++l;
  return l;
}

// Allow a kernel more than 48 KB of dynamic shared memory (once per device).
template <typename K>
inline cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

#define XL_CHECK_LAUNCH(where)                                  \
  do {                                                          \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return ::xl::cuda_fail(_e, where);   \
  } while (0)

// Each translation unit with kernels holds its own copy of the device tables
// (whole-program compilation, one device module per unit).  It registers,
// from a static initialiser, the function that fills them from the host
// twiddles and, optionally, a reader of its device timeout counter.
// A unit with bounded waits also registers the setter of its status word
// pointer and wait limit.
using TableUpload = cudaError_t (*)(const float2* host_twiddles);
using TimeoutCounter = cudaError_t (*)(unsigned int* count, int reset);
using StatusSetup = cudaError_t (*)(unsigned int* status_word, unsigned long long wait_limit_ns);
bool register_device_tables(TableUpload upload, TimeoutCounter timeouts, StatusSetup status = nullptr);

}  // namespace xl
