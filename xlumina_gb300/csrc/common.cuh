// Device helpers shared by the propagation kernels: twiddle tables, phase
// generation with an FP64 argument, and the per-pixel Jones-operation
// program that is fused into the first and last passes of a propagator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_core.cuh"
#include "xl_types.h"

namespace xl {

// Twiddle tables for every power-of-two size S <= 8192: g_tw[S + q] = e^{-2 pi i q / S}.
// Filled from host-computed float64 values (rounded once) at library set-up.
// `static` gives each translation unit its own copy, filled by its own set-up hook.
static __device__ float2 g_tw[2 * XL_MAX_FFT];

__device__ __forceinline__ const float2* tw_table(int logn) { return g_tw + (1 << logn); }

// e^{i 2 pi t}: the argument in turns is reduced in float64, then the
// reduced fraction goes to sincospif (argument in [-1, 1]).
__device__ __forceinline__ float2 cis_turns(double t) {
  const double f = t - rint(t);
  float s, c;
  sincospif(2.0f * (float)f, &s, &c);
  return make_float2(c, s);
}

// Rayleigh-Sommerfeld impulse response at offset (X, Y), distance z:
// exp(+-i k r) * z / (2 pi r^2) * (1/r - i k), r = sqrt(X^2 + Y^2 + z^2);
// the exponent's sign follows the sign of z.  r and k r are float64.
__device__ __forceinline__ float2 rs_kernel_value(double X, double Y, double z, double inv_lambda,
                                                  float k) {
  const double r = sqrt(X * X + Y * Y + z * z);
  const double t = r * inv_lambda;
  const float2 e = cis_turns(z > 0 ? t : -t);
  const float rf = (float)r;
  const float a = (float)z / (6.283185307179586f * rf * rf);
  return cmul(e, make_float2(a / rf, -a * k));
}

// ---- fused per-pixel Jones program ----

struct PixelCtx {
  int row, col;  // pixel position
  long long pix; // row * ld + col inside one plane of the parameter arrays
  int batch;
};

__device__ __forceinline__ float op_param(const XlOp& op, int i, const PixelCtx& px) {
  if (op.pmask & (1 << i)) {
    const float* p = (const float*)op.ptr[i];
    return __ldg(p + (long long)px.batch * op.pbstride + px.pix);
  }
  return op.sval[i];
}

// Apply one op to the pixel's (Ex, Ey, Ez) (scalar fields use e[0] only).
__device__ __forceinline__ void apply_op(const XlOp& op, float2 (&e)[3], const PixelCtx& px) {
  switch (op.kind) {
    case XL_OP_PHASE: {  // scalar SLM: field * e^{i phi}
      float s, c;
      sincosf(op_param(op, 0, px), &s, &c);
      e[0] = cmul(e[0], make_float2(c, s));
      break;
    }
    case XL_OP_SSLM: {  // diag(e^{i a}, e^{i p}); Ez unchanged
      float s, c;
      sincosf(op_param(op, 0, px), &s, &c);
      e[0] = cmul(e[0], make_float2(c, s));
      sincosf(op_param(op, 1, px), &s, &c);
      e[1] = cmul(e[1], make_float2(c, s));
      break;
    }
    case XL_OP_SSLM_AMP: {  // diag(A1 e^{i a}, A2 e^{i p}); Ez unchanged
      float s, c;
      sincosf(op_param(op, 0, px), &s, &c);
      e[0] = cscale(cmul(e[0], make_float2(c, s)), op_param(op, 2, px));
      sincosf(op_param(op, 1, px), &s, &c);
      e[1] = cscale(cmul(e[1], make_float2(c, s)), op_param(op, 3, px));
      break;
    }
    case XL_OP_LCD: {  // general retarder with delta = 0 (eta, theta); Ez unchanged
      float sh, ch, s2, c2;
      float st, ct;
      if (op.pmask & 1) sincosf(0.5f * op_param(op, 0, px), &sh, &ch);
      else { ch = op.dval[0]; sh = op.dval[1]; }   // scalar eta: cos, sin of eta/2 from the host
      if (op.pmask & 2) sincosf(op_param(op, 1, px), &st, &ct);
      else { ct = op.dval[2]; st = op.dval[3]; }   // scalar theta
      // a = ch - i sh (c^2 - s^2), b = c = -i sh 2 s c, d = ch + i sh (c^2 - s^2)
      c2 = ct * ct - st * st;
      s2 = 2.f * st * ct;
      const float2 a = make_float2(ch, -sh * c2);
      const float2 b = make_float2(0.f, -sh * s2);
      const float2 d = make_float2(ch, sh * c2);
      const float2 x = e[0], y = e[1];
      e[0] = cadd(cmul(a, x), cmul(b, y));
      e[1] = cadd(cmul(b, x), cmul(d, y));
      break;
    }
    case XL_OP_LP: {  // linear polarizer at alpha; Ez set to zero
      float s, c;
      if (op.pmask & 1) sincosf(op_param(op, 0, px), &s, &c);
      else { c = op.sval[2]; s = op.sval[3]; }   // scalar alpha: cos, sin from the host
      const float2 x = e[0], y = e[1];
      e[0] = cadd(cscale(x, c * c), cscale(y, c * s));
      e[1] = cadd(cscale(x, c * s), cscale(y, s * s));
      e[2] = make_float2(0.f, 0.f);
      break;
    }
    case XL_OP_SEPMASK: {  // separable complex mask ax[col]*ay[row] with an FP64 pupil test
      // ptr[0]: float2 colfac[nx]; ptr[1]: float2 rowfac[ny];
      // ptr[2], ptr[3]: double pupil terms (col, row); pupil = (tc + tr < 1) if present.
      const float2 fc = ((const float2*)op.ptr[0])[px.col];
      const float2 fr = ((const float2*)op.ptr[1])[px.row];
      float2 m = cmul(fc, fr);
      if (op.ptr[2]) {
        const double tc = ((const double*)op.ptr[2])[px.col];
        const double tr = ((const double*)op.ptr[3])[px.row];
        if (!(tc + tr < 1.0)) m = make_float2(0.f, 0.f);
      }
      e[0] = cmul(e[0], m);
      e[1] = cmul(e[1], m);
      if (op.sval[0] != 0.f) e[2] = make_float2(0.f, 0.f);  // vector lens drops Ez
      else e[2] = cmul(e[2], m);
      break;
    }
    case XL_OP_CMUL: {  // multiply every component by a per-pixel complex array
      const float2* p = (const float2*)op.ptr[0];
      const float2 m = p[(long long)px.batch * op.pbstride + px.pix];
      e[0] = cmul(e[0], m);
      e[1] = cmul(e[1], m);
      e[2] = cmul(e[2], m);
      break;
    }
    case XL_OP_HIGHNA: {  // optical_elements.py:528-594
      const double Xd = ((const double*)op.ptr[0])[px.col];
      const double Yd = ((const double*)op.ptr[1])[px.row];
      const double rad = op.dval[0];
      const double q = (Xd * Xd + Yd * Yd) / (rad * rad);   // (u^2 + v^2), FP64 pupil test
      const float smax = (float)op.dval[2];
      const float G = q < 1.0 ? 1.f / sqrtf(fabsf(1.f - (float)q * smax * smax)) : 0.f;
      const float X = (float)Xd, Y = (float)Yd;
      const float rho = sqrtf(X * X + Y * Y);
      const float th = rho / (float)op.dval[1];
      const float phi = atan2f(Y, X);
      float st, ct, sp, cp;
      sincosf(th, &st, &ct);
      sincosf(phi, &sp, &cp);
      const float w = sqrtf(fabsf(ct)) * G;
      const float2 ex = e[0], ey = e[1];
      const float2 ez = cadd(cscale(ex, X / rho), cscale(ey, Y / rho));  // NaN at rho = 0, as the reference
      const float2 ox = cadd(cadd(cscale(ex, ct * cp * cp + sp * sp), cscale(ey, ct * cp * sp - sp * cp)),
                             cscale(ez, -cp * st));
      const float2 oy = cadd(cadd(cscale(ex, sp * ct * cp - cp * sp), cscale(ey, ct * sp * sp + cp * cp)),
                             cscale(ez, -sp * st));
      const float2 oz = cadd(cadd(cscale(ex, st * cp), cscale(ey, st * sp)), cscale(ez, ct));
      e[0] = cscale(ox, w);
      e[1] = cscale(oy, w);
      e[2] = cscale(oz, w);
      break;
    }
    default:
      break;
  }
}

__device__ __forceinline__ void apply_prog(const XlProg& prog, float2 (&e)[3], const PixelCtx& px) {
  for (int i = 0; i < prog.nops; ++i) apply_op(prog.ops[i], e, px);
}

}  // namespace xl
