// Interface between the RS / VRS host entry points (rs.cu) and the kernel
// translation units (rs_q*.cu, one or a few transform lengths each, compiled
// in parallel).
#pragma once

#include "internal.h"

namespace xl {

// Arguments of one RS / VRS launch (device pointers; see XlRsArgs in xlgb.h).
struct RsLaunch {
  int B, cin, cout, ny, nx;
  const float2* in[3];
  long long ibs;
  float2* out[3];
  long long obs;
  const double* x;
  const double* y;
  const double* z;
  const float2* spec;
  long long sstride;
  const int* sidx;
  const float2* const* specs;   // per batch entry (overrides spec / sstride / sidx when set)
  float2* work;
  XlProg pre, post;
  int adjoint;
};

// Q = 2^logq is the half transform length: the smallest power of two >= the field side.
// Q = 2^logq >= the field side, at least 32: the transfer-spectrum row pass
// takes G = 256 / T rows per CTA, which for Q = 16 (P = 32) exceeds P.
inline int rs_logq(int ny, int nx) {
  const int n = ny > nx ? ny : nx;
  const int l = ilog2_ceil(n);
  return l < 5 ? 5 : l;
}

// Transfer spectrum and propagation passes for Q = 2^LOGQ (explicitly
// instantiated for LOGQ = 4..12 in the kernel translation units).
template <int LOGQ>
int rs_spectrum(cudaStream_t st, int ny, int nx, const double* offx, const double* offy, double z,
                const double* zp, double wavelength, double scale, float2* spec, float2* work, int dz);
template <int LOGQ>
int rs_propagate(cudaStream_t st, const RsLaunch& p, int stage);

}  // namespace xl
