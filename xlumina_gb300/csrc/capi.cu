// Library-wide C ABI pieces: error reporting, version, per-device set-up.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "internal.h"

namespace xl {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_fail(cudaError_t e, const char* where) {
  set_error("%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
  return XL_ECUDA;
}

static std::mutex g_init_mu;
static bool g_init_dev[256];

struct DeviceTables {
  TableUpload upload;
  TimeoutCounter timeouts;
  StatusSetup status;
};

static std::vector<DeviceTables>& registry() {
  static std::vector<DeviceTables> r;
  return r;
}

bool register_device_tables(TableUpload upload, TimeoutCounter timeouts, StatusSetup status) {
  registry().push_back({upload, timeouts, status});
  return true;
}

// The status word kernels raise when a bounded wait runs out: one word of
// mapped (zero-copy) pinned host memory for the process, so that the host
// reads it without synchronising the device.  Allocated at the first device
// set-up; null if mapped host memory is unavailable (the counters remain).
static unsigned int* g_status_host = nullptr;
static unsigned int* g_status_dev = nullptr;
static unsigned long long g_wait_limit[256];

static cudaError_t status_word() {
  if (g_status_host) return cudaSuccess;
  void* h = nullptr;
  cudaError_t e = cudaHostAlloc(&h, sizeof(unsigned int), cudaHostAllocMapped | cudaHostAllocPortable);
  if (e != cudaSuccess) return e;
  *(volatile unsigned int*)h = 0u;
  void* d = nullptr;
  if ((e = cudaHostGetDevicePointer(&d, h, 0)) != cudaSuccess) {
    cudaFreeHost(h);
    return e;
  }
  g_status_host = (unsigned int*)h;
  g_status_dev = (unsigned int*)d;
  return cudaSuccess;
}

// Point every unit's kernels at the status word and set their wait limit (current device).
static cudaError_t set_status_all(unsigned long long limit_ns) {
  for (const DeviceTables& t : registry())
    if (t.status)
      if (cudaError_t e = t.status(g_status_dev, limit_ns)) return e;
  return cudaSuccess;
}

// Twiddle tables for S = 1, 2, 4, ..., XL_MAX_FFT at offset S: e^{-2 pi i q / S},
// computed in float64 and rounded once.
static const std::vector<float2>& host_twiddles() {
  static std::vector<float2> t;
  if (t.empty()) {
    t.assign(2 * XL_MAX_FFT, make_float2(0.f, 0.f));
    for (int s = 1; s <= XL_MAX_FFT; s <<= 1)
      for (int q = 0; q < s; ++q) {
        const double a = 2.0 * M_PI * (double)q / (double)s;
        t[s + q] = make_float2((float)cos(a), (float)-sin(a));
      }
  }
  return t;
}

int ensure_init() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 256) {
    set_error("device index %d out of range", dev);
    return XL_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (g_init_dev[dev]) return XL_OK;
  const float2* h = host_twiddles().data();
  for (const DeviceTables& t : registry())
    if ((e = t.upload(h)) != cudaSuccess) return cuda_fail(e, "upload device tables");
  if ((e = status_word()) != cudaSuccess) return cuda_fail(e, "status word (mapped host memory)");
  g_wait_limit[dev] = kDefaultWaitLimitNs;
  if ((e = set_status_all(g_wait_limit[dev])) != cudaSuccess) return cuda_fail(e, "device status set-up");
  g_init_dev[dev] = true;
  return XL_OK;
}

int set_wait_limit(unsigned long long ns) {
  if (int rc = ensure_init()) return rc;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_init_mu);
  if ((e = set_status_all(ns)) != cudaSuccess) return cuda_fail(e, "xl_set_wait_limit");
  g_wait_limit[dev] = ns;
  return XL_OK;
}

int read_status(unsigned int* flag, int clear) {
  std::lock_guard<std::mutex> lk(g_init_mu);
  *flag = g_status_host ? *(volatile unsigned int*)g_status_host : 0u;
  if (clear && g_status_host) *(volatile unsigned int*)g_status_host = 0u;
  return XL_OK;
}

// ---- kernel variants per (pass, transform length) ----
// Available variants: the one-line kernel (0) everywhere; for 1024..4096-point
// RS transforms the packed two-line column pass, interleaved (1) or in
// barrier groups (2), the one-line kernel with L2 prefetch (3), the
// interleaved packed one with L2 and register prefetch (4), and the one-line
// kernel with prefetch in two barrier groups (5) or in CTAs of half the
// columns, two per SM (6), and the two groups of (5) started half a
// component apart (7), the one-line kernel persistent (8: the pass twiddle
// table loaded once per CTA); for 4096-point transforms also the radix-64
// column pass (9: two passes of 64 elements per thread, one exchange per
// transform) and the persistent one-line kernel that keeps each unit's
// spectrum values in Tensor Memory for its later components (10).  The chirp-z x transform: the stage capped for two
// CTAs per SM (0), every plane staged that fits one CTA per SM (1), no
// staging (2), as 0 with registers for two CTAs per SM (3), and at 4096
// points for three components one group transforming them one after the
// other, two CTAs per SM (4).  The chirp-z y transform: one CTA per column
// tile and entry (0), persistent (1).
static int variant_count(int pass, int log2_len) {
  if (pass < 0 || pass >= XL_NUM_PASSES || log2_len < 1 || log2_len > 13) return 0;
  if (pass == XL_PASS_RS_COLS && log2_len == 12) return 11;
  if (pass == XL_PASS_RS_COLS && log2_len >= 10 && log2_len <= 11) return 9;
  if (pass == XL_PASS_CZT_ROWS && log2_len == 12) return 5;
  if (pass == XL_PASS_CZT_ROWS && log2_len >= 5) return 4;
  if (pass == XL_PASS_CZT_COLS && log2_len >= 5) return 2;
  return 1;
}
static std::atomic<int> g_variant[XL_NUM_PASSES][14];

// Defaults that differ from variant 0, by measurement: the 4096-point chirp-z
// x transform (the 2048^2 high-NA focus) with registers for two CTAs per SM,
// 1451 against 1400 tables/s on the high-NA optimisation step; the
// persistent one-line RS column pass at 4096 points, 1.929 against 1.971 ms
// per 8 x 2048^2 VRS fields (the same at 2048 points: 5549-5564 against
// 5524-5566 4f tables/s, so variant 0 stays the default there).
// The persistent chirp-z y transform at 4096 points: 1945 against 1925
// tables/s on the high-NA step (on the 4f step's 2048- and 1024-point
// transforms it measured 0.3 % slower, so variant 0 stays there).
static const bool g_variant_defaults = [] {
  g_variant[XL_PASS_CZT_ROWS][12].store(3, std::memory_order_relaxed);
  g_variant[XL_PASS_RS_COLS][12].store(8, std::memory_order_relaxed);
  g_variant[XL_PASS_CZT_COLS][12].store(1, std::memory_order_relaxed);
  return true;
}();


int kernel_variant(int pass, int log2_len) {
  if (pass < 0 || pass >= XL_NUM_PASSES || log2_len < 0 || log2_len > 13) return 0;
  return g_variant[pass][log2_len].load(std::memory_order_relaxed);
}

}  // namespace xl

extern "C" int xl_kernel_variant_count(int pass, int log2_len) { return xl::variant_count(pass, log2_len); }

extern "C" int xl_set_kernel_variant(int pass, int log2_len, int variant) {
  const int n = xl::variant_count(pass, log2_len);
  if (n == 0 || variant < 0 || variant >= n) {
    xl::set_error("xl_set_kernel_variant: pass %d at length 2^%d has %d variant(s), got %d", pass, log2_len, n,
                  variant);
    return XL_EINVAL;
  }
  xl::g_variant[pass][log2_len].store(variant, std::memory_order_relaxed);
  return XL_OK;
}

extern "C" int xl_get_kernel_variant(int pass, int log2_len) {
  if (xl::variant_count(pass, log2_len) == 0) {
    xl::set_error("xl_get_kernel_variant: unknown pass %d or length 2^%d", pass, log2_len);
    return XL_EINVAL;
  }
  return xl::kernel_variant(pass, log2_len);
}

extern "C" const char* xl_last_error(void) { return xl::g_err; }

extern "C" int xl_version(void) { return 100; }

extern "C" size_t xl_struct_size(const char* name) {
  if (!name) return 0;
  struct Entry {
    const char* name;
    size_t size;
  };
  static const Entry sizes[] = {
      {"XlOp", sizeof(XlOp)},           {"XlProg", sizeof(XlProg)},
      {"XlRsArgs", sizeof(XlRsArgs)},   {"XlCztArgs", sizeof(XlCztArgs)},
      {"XlCztChirpArgs", sizeof(XlCztChirpArgs)},
      {"XlBsArgs", sizeof(XlBsArgs)},   {"XlNoiseArgs", sizeof(XlNoiseArgs)},
      {"XlAdamWTensor", sizeof(XlAdamWTensor)}, {"XlAdamWArgs", sizeof(XlAdamWArgs)},
  };
  for (const Entry& e : sizes)
    if (strcmp(e.name, name) == 0) return e.size;
  return 0;
}

extern "C" int xl_init(void) { return xl::ensure_init(); }

extern "C" int xl_device_status(unsigned int* flag, int clear) {
  if (!flag) {
    xl::set_error("xl_device_status: null output");
    return XL_EINVAL;
  }
  return xl::read_status(flag, clear);
}

extern "C" int xl_set_wait_limit(unsigned long long ns) { return xl::set_wait_limit(ns); }

extern "C" int xl_host_mapped(const void* host, void** dev) {
  if (!host || !dev) {
    xl::set_error("xl_host_mapped: null pointer");
    return XL_EINVAL;
  }
  *dev = nullptr;
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, host);
  if (e != cudaSuccess || at.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    xl::set_error("xl_host_mapped: not page-locked host memory");
    return XL_EINVAL;
  }
  void* d = nullptr;
  e = cudaHostGetDevicePointer(&d, const_cast<void*>(host), 0);
  if (e != cudaSuccess || !d) {
    cudaGetLastError();
    xl::set_error("xl_host_mapped: host memory not mapped for the current device");
    return XL_EINVAL;
  }
  *dev = d;
  return XL_OK;
}

extern "C" int xl_device_timeouts(unsigned int* count, int reset) {
  if (!count) {
    xl::set_error("xl_device_timeouts: null output");
    return XL_EINVAL;
  }
  unsigned int total = 0;
  for (const xl::DeviceTables& t : xl::registry()) {
    if (!t.timeouts) continue;
    unsigned int c = 0;
    cudaError_t e = t.timeouts(&c, reset);
    if (e != cudaSuccess) return xl::cuda_fail(e, "xl_device_timeouts");
    total += c;
  }
  *count = total;
  return XL_OK;
}
