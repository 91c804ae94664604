// Chirp-z propagation (scalar CZT, vectorial VCZT, the high-NA focus): the C
// ABI entry points.  The reference (wave_optics.py:333-460) runs Bluestein's
// algorithm along y and then along x; the kernels (czt_kernels.cuh) run the x
// transform over rows with the fused prologue and the y transform over
// column tiles with the fused epilogue.
#include <math.h>

#include "czt_host.h"

namespace xl {

#define XL_CZT_DISPATCH(LL, FN, ...)          \
  switch (LL) {                               \
    case 5: return FN<5>(__VA_ARGS__);        \
    case 6: return FN<6>(__VA_ARGS__);        \
    case 7: return FN<7>(__VA_ARGS__);        \
    case 8: return FN<8>(__VA_ARGS__);        \
    case 9: return FN<9>(__VA_ARGS__);        \
    case 10: return FN<10>(__VA_ARGS__);      \
    case 11: return FN<11>(__VA_ARGS__);      \
    case 12: return FN<12>(__VA_ARGS__);      \
    case 13: return FN<13>(__VA_ARGS__);      \
    default: break;                           \
  }

static int dispatch_rows(cudaStream_t st, const CztLaunch& p, int ll) {
  XL_CZT_DISPATCH(ll, czt_rows_launch, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", ll);
  return XL_EUNSUPPORTED;
}

static int dispatch_cols(cudaStream_t st, const CztLaunch& p, int ll) {
  XL_CZT_DISPATCH(ll, czt_cols_launch, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", ll);
  return XL_EUNSUPPORTED;
}

}  // namespace xl

using namespace xl;

extern "C" size_t xl_czt_work_bytes(int batch, int comps, int ny, int mx) {
  if (batch < 1 || comps < 1 || ny < 1 || mx < 1) return 0;
  const size_t mxp = ((size_t)mx + 31) / 32 * 32;  // column tiles may round mx up (tile widths divide 32)
  return (size_t)batch * comps * ny * mxp * sizeof(float2);
}

static int czt_run(void* stream, const XlCztArgs* a, int stage) {
  if (!a) {
    set_error("xl_czt: null args");
    return XL_EINVAL;
  }
  if (a->ny < 2 || a->nx < 2 || a->my < 2 || a->mx < 2 || a->batch < 1) {
    set_error("xl_czt: bad shape batch=%d in %dx%d out %dx%d (outputs need >= 2 samples per axis)",
              a->batch, a->ny, a->nx, a->my, a->mx);
    return XL_EINVAL;
  }
  const bool ok_modes = (a->mode == XL_CZT_SCALAR && a->comps_in == 1 && a->comps_out == 1) ||
                        (a->mode == XL_CZT_VECTOR && !a->adjoint && a->comps_in == 2 && a->comps_out == 3) ||
                        (a->mode == XL_CZT_VECTOR && a->adjoint && a->comps_in == 3 && a->comps_out == 3) ||
                        (a->mode == XL_CZT_PLAIN && a->comps_in >= 1 && a->comps_in <= 3 &&
                         a->comps_out >= a->comps_in && a->comps_out <= 3);
  if (!ok_modes) {
    set_error("xl_czt: mode %d with comps %d -> %d is not supported", a->mode, a->comps_in, a->comps_out);
    return XL_EINVAL;
  }
  const int llx = a->log2_lx, lly = a->log2_ly;
  if (llx < 5 || llx > 13 || lly < 5 || lly > 13 || (1 << llx) < a->nx + a->mx ||
      (1 << lly) < a->ny + a->my) {
    set_error("xl_czt: Bluestein lengths 2^%d, 2^%d must be in 32..8192 and exceed m + M - 1",
              a->log2_lx, a->log2_ly);
    return XL_EINVAL;
  }
  if (!a->pre_x || !a->g_x || !a->post_x || !a->pre_y || !a->g_y || !a->post_y || !a->work) {
    set_error("xl_czt: null chirp vector or workspace");
    return XL_EINVAL;
  }
  if (a->mode != XL_CZT_PLAIN && (!a->x || !a->y || !a->xout || !a->yout || !(a->wavelength > 0))) {
    set_error("xl_czt: transfer functions need x, y, xout, yout and wavelength > 0");
    return XL_EINVAL;
  }
  for (int c = 0; c < a->comps_in; ++c)
    if (!a->in[c]) { set_error("xl_czt: null input plane %d", c); return XL_EINVAL; }
  const int nout = (a->adjoint && a->mode == XL_CZT_VECTOR) ? 2 : a->comps_out;
  for (int c = 0; c < nout; ++c)
    if (!a->out[c]) { set_error("xl_czt: null output plane %d", c); return XL_EINVAL; }
  if (a->pre.nops < 0 || a->pre.nops > XL_MAX_OPS || (a->adjoint && a->pre.nops)) {
    set_error("xl_czt: op program too long (or given to the adjoint)");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  CztLaunch p;
  p.B = a->batch; p.cin = a->comps_in; p.cout = a->comps_out;
  p.ny = a->ny; p.nx = a->nx; p.my = a->my; p.mx = a->mx; p.mode = a->mode;
  const int wt = czt_tile_w(lly);
  p.mxp = (a->mx + wt - 1) / wt * wt;
  p.lw = ilog2_ceil(wt);
  p.adjoint = a->adjoint ? 1 : 0;
  // forward: the input line starts at 0 and the output window at m; the adjoint swaps them
  p.ioff_x = p.adjoint ? a->mx : 0;
  p.ooff_x = p.adjoint ? 0 : a->nx;
  p.ioff_y = p.adjoint ? a->my : 0;
  p.ooff_y = p.adjoint ? 0 : a->ny;
  for (int c = 0; c < 3; ++c) {
    p.in[c] = (const float2*)a->in[c];
    p.out[c] = (float2*)a->out[c];
  }
  p.ibs = a->in_bstride; p.obs = a->out_bstride;
  p.x = a->x; p.y = a->y; p.xo = a->xout; p.yo = a->yout;
  p.z = a->z;
  p.inv_lambda = a->wavelength > 0 ? 1.0 / a->wavelength : 0.0;
  p.k = a->wavelength > 0 ? (float)(2.0 * M_PI / a->wavelength) : 0.f;
  p.cte = make_float2((float)a->cte_re, (float)(a->adjoint ? -a->cte_im : a->cte_im));
  p.pre_x = (const float2*)a->pre_x; p.g_x = (const float2*)a->g_x; p.post_x = (const float2*)a->post_x;
  p.pre_y = (const float2*)a->pre_y; p.g_y = (const float2*)a->g_y; p.post_y = (const float2*)a->post_y;
  p.work = (float2*)a->work;
  p.pre = a->pre;
  cudaStream_t st = (cudaStream_t)stream;
  if (stage < 0 || stage == 0)
    if (int rc = dispatch_rows(st, p, llx)) return rc;
  if (stage < 0 || stage == 1)
    if (int rc = dispatch_cols(st, p, lly)) return rc;
  return XL_OK;
}

extern "C" int xl_czt(void* stream, const XlCztArgs* a) { return czt_run(stream, a, -1); }

extern "C" int xl_czt_stage(void* stream, const XlCztArgs* a, int stage) {
  if (stage < 0 || stage > 1) {
    set_error("xl_czt_stage: stage must be 0 or 1 (got %d)", stage);
    return XL_EINVAL;
  }
  return czt_run(stream, a, stage);
}
