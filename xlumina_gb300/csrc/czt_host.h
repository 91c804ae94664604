// Interface between the chirp-z host entry points (czt.cu) and the kernel
// translation units (czt_l*.cu, a few transform lengths each, compiled in
// parallel).
#pragma once

#include "internal.h"

namespace xl {

// Arguments of one chirp-z launch (device pointers; see XlCztArgs in xlgb.h).
struct CztLaunch {
  int B, cin, cout, ny, nx, my, mx, mxp;  // input plane ny x nx, output plane my x mx (mxp: mx rounded up)
  int mode;                               // XL_CZT_SCALAR / XL_CZT_VECTOR / XL_CZT_PLAIN
  int adjoint;                            // conjugate transpose of the forward transform
  int ioff_x, ooff_x, ioff_y, ooff_y;     // where input / output lines sit in the length-L line
  int lw;                                 // log2 of the intermediate's column-tile width
  const float2* in[3];
  long long ibs;
  float2* out[3];
  long long obs;
  const double* x;
  const double* y;
  const double* xo;
  const double* yo;
  double z, inv_lambda;
  float k;
  float2 cte;
  const float2* pre_x;   // nx
  const float2* g_x;     // Lx, natural order
  const float2* post_x;  // mx (includes 1/Lx)
  const float2* pre_y;   // ny
  const float2* g_y;     // Ly, natural order
  const float2* post_y;  // my (includes 1/Ly)
  float2* work;          // B x cout x ny x mxp, column tiles of 2^lw
  XlProg pre;
  const double* zb;      // per-entry distances (NULL: z for every entry); with them the
  const float2* cteb;    // chirps are packed per entry and cteb[b] replaces cte
  const float2* fin;     // transfer function on the input plane (ny x nx), or NULL
  const float2* fout;    // and on the output plane (my x mx), or NULL
};

// Entry b's chirp vector: the shared one, or its slot in the per-entry packing.
__device__ __forceinline__ const float2* czt_entry(const float2* v, const CztLaunch& p, int b, int len) {
  return p.zb ? v + (long long)b * len : v;
}

// Column-tile width of the intermediate, set by the y transform's length 2^logl.
inline int czt_tile_w(int logl) {
  const int t = (1 << logl) / 16;
  return logl >= 13 ? 2 : ((32 / t) > 4 ? (32 / t) : 4);
}

// The x transform (rows, prologue) and the y transform (columns, epilogue)
// for Bluestein length 2^LOGL (explicitly instantiated for LOGL = 5..13 in the
// kernel translation units).
template <int LOGL>
int czt_rows_launch(cudaStream_t st, const CztLaunch& p);
template <int LOGL>
int czt_cols_launch(cudaStream_t st, const CztLaunch& p);

}  // namespace xl
