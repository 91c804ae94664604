// Device helpers shared by the propagation kernels: twiddle tables, phase
// generation with an FP64 argument, and the per-pixel Jones-operation
// program that is fused into the first and last passes of a propagator.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_core.cuh"
#include "xlgb.h"

namespace xl {

// Twiddle tables for every power-of-two size S <= 8192: g_tw[S + q] = e^{-2 pi i q / S}.
// Filled from host-computed float64 values (rounded once) at library set-up.
// `static` gives each translation unit its own copy, filled by its own set-up hook.
static __device__ float2 g_tw[2 * XL_MAX_FFT];

__device__ __forceinline__ const float2* tw_table(int logn) { return g_tw + (1 << logn); }

// ---- float-float arithmetic: a value hi + lo held in two floats, ~48
// significant bits (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2).  The RS phase
// k r needs more than float precision (k r ~ 1e6 rad at 10 cm), and GB300's
// FP64 rate is a small fraction of its FP32 rate.  The _rn intrinsics are
// never contracted into FMAs, which would break the error terms.
struct ffloat {
  float hi, lo;
};
__device__ __forceinline__ ffloat ff_split(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ ffloat ff_fast_two_sum(float a, float b) {   // needs |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ffloat ff_add(ffloat x, ffloat y) {
  const float s = __fadd_rn(x.hi, y.hi);
  const float bb = __fsub_rn(s, x.hi);
  const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
  return ff_fast_two_sum(s, __fadd_rn(e, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ ffloat ff_mul(ffloat x, ffloat y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float e = fmaf(x.hi, y.hi, -p);
  return ff_fast_two_sum(p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e)));
}
// One Newton step from the float square root: r + (x - r^2) / (2 r), the
// residual taken exactly by an FMA.
__device__ __forceinline__ ffloat ff_sqrt(ffloat x) {
  const float r = sqrtf(x.hi);
  const float d = __fadd_rn(fmaf(-r, r, x.hi), x.lo);
  return ff_fast_two_sum(r, __fdiv_rn(d, __fmul_rn(2.f, r)));
}

// Per-launch constants of the RS impulse response, split into float-float
// once per thread: z^2, 1/lambda, and float copies for the amplitude.
struct RsGeom {
  ffloat z2, invl;
  float zf, k, sgn;   // z, 2 pi / lambda, sign of z (the exponent's sign)
};
__device__ __forceinline__ RsGeom rs_geom(double z, double inv_lambda, float k) {
  RsGeom g;
  const ffloat zz = ff_split(z);
  g.z2 = ff_mul(zz, zz);
  g.invl = ff_split(inv_lambda);
  g.zf = (float)z;
  g.k = k;
  g.sgn = z > 0 ? 1.f : -1.f;
  return g;
}

// s = X^2 + Y^2 + z^2 in float-float for an offset split into float-float
// parts (z^2 + Y^2 first: it is the larger term).
__device__ __forceinline__ ffloat rs_s(const RsGeom& g, ffloat x, ffloat y) {
  return ff_add(ff_add(g.z2, ff_mul(y, y)), ff_mul(x, x));
}

// e^{+-i 2 pi r / lambda} for r = sqrt(s) (sign of z), and r as a float.
__device__ __forceinline__ float2 rs_phase(const RsGeom& g, ffloat s, float* rf) {
  const ffloat r = ff_sqrt(s);
  const ffloat t = ff_mul(r, g.invl);
  float f = __fadd_rn(__fsub_rn(t.hi, rintf(t.hi)), t.lo);
  f = __fsub_rn(f, rintf(f));
  *rf = r.hi;
  float sn, cs;
  sincospif(2.0f * g.sgn * f, &sn, &cs);
  return make_float2(cs, sn);
}

// Rayleigh-Sommerfeld impulse response at s = X^2 + Y^2 + z^2:
// exp(+-i k r) * z / (2 pi r^2) * (1/r - i k), r = sqrt(s); the exponent's
// sign follows the sign of z.  r and k r are float-float.
__device__ __forceinline__ float2 rs_value_s(const RsGeom& g, ffloat s) {
  float rf;
  const float2 e = rs_phase(g, s, &rf);
  const float a = g.zf / (6.283185307179586f * rf * rf);
  return cmul(e, make_float2(a / rf, -a * g.k));
}

// Its derivative with respect to z, from H = e^{i s k r} a(r, z),
// a = z (1/r - i k) / (2 pi r^2), s = sign(z), dr/dz = z/r:
// dH/dz = e^{i s k r} (i s k (z/r) a + da/dz),
// da/dz = ((1/r^3 - i k / r^2) + z^2 (-3/r^5 + 2 i k / r^4)) / (2 pi).
__device__ __forceinline__ float2 rs_dz_value_s(const RsGeom& g, ffloat s) {
  float rf;
  const float2 e = rs_phase(g, s, &rf);
  const float zf = g.zf, k = g.k;
  const float ir = 1.f / rf, ir2 = ir * ir, ir3 = ir2 * ir;
  const float inv2pi = 0.15915494309189533577f;
  const float2 a = make_float2(zf * ir3 * inv2pi, -zf * k * ir2 * inv2pi);
  const float z2 = zf * zf;
  const float2 da = make_float2((ir3 - 3.f * z2 * ir3 * ir2) * inv2pi, (-k * ir2 + 2.f * k * z2 * ir2 * ir2) * inv2pi);
  const float w = g.sgn * k * zf * ir;   // i s k (z / r) a
  const float2 ia = make_float2(-w * a.y, w * a.x);
  return cmul(e, cadd(ia, da));
}

// The same at an offset (X, Y) given in float64.
__device__ __forceinline__ float2 rs_kernel_value(double X, double Y, double z, double inv_lambda, float k) {
  const RsGeom g = rs_geom(z, inv_lambda, k);
  return rs_value_s(g, rs_s(g, ff_split(X), ff_split(Y)));
}

// sin and cos of a mask phase in radians (one place for every Jones op and
// its backward).  The accurate sincosf: the high-NA focus sums millions of
// pixels with heavy cancellation, and the hardware approximation's 4e-7
// absolute error per pixel shows up there above the 1e-5 parity bar.
__device__ __forceinline__ void phase_sincos(float x, float* s, float* c) { sincosf(x, s, c); }

// ---- fused per-pixel Jones program ----

struct PixelCtx;
__device__ __forceinline__ void highna_coeffs(const XlOp& op, const PixelCtx& px, float (&kc)[6]);

struct PixelCtx {
  int row, col;  // pixel position
  long long pix; // row * ld + col inside one plane of the parameter arrays
  int batch;
};

// High-NA objective lens (optical_elements.py:528-594) as a real 3x2 matrix K
// per pixel: E' = K [Ex, Ey], folding in Ez = Ex X/rho + Ey Y/rho (NaN at
// rho = 0, as the reference), the rotation RL(theta, phi), sqrt|cos theta|
// and the pupil factor G.  kc = {K00, K01, K10, K11, K20, K21}.
__device__ __forceinline__ void highna_coeffs(const XlOp& op, const PixelCtx& px, float (&kc)[6]) {
  if (op.ptr[2]) {  // precomputed coefficient planes (6 x ny x nx float32)
    const float* cp = (const float*)op.ptr[2];
    const long long plane = op.pbstride;   // ny * nx
#pragma unroll
    for (int q = 0; q < 6; ++q) kc[q] = __ldg(cp + q * plane + px.pix);
    return;
  }
  const double Xd = ((const double*)op.ptr[0])[px.col];
  const double Yd = ((const double*)op.ptr[1])[px.row];
  const double rad = op.dval[0];
  // pupil (X^2 + Y^2) / r^2 < 1, tested as X^2 + Y^2 < r^2 (equivalent for positive doubles)
  const double rho2 = Xd * Xd + Yd * Yd;
  const bool inside = rho2 < rad * rad;
  const float smax = (float)op.dval[2];
  const float q = (float)rho2 * (float)op.dval[3];   // (u^2 + v^2), dval[3] = 1 / r^2
  const float G = inside ? 1.f / sqrtf(fabsf(1.f - q * smax * smax)) : 0.f;
  const float X = (float)Xd, Y = (float)Yd;
  const float rho = sqrtf(X * X + Y * Y);
  const float th = rho / (float)op.dval[1];
  const float phi = atan2f(Y, X);
  float st, ct, sp, cp;
  sincosf(th, &st, &ct);
  sincosf(phi, &sp, &cp);
  const float w = sqrtf(fabsf(ct)) * G;
  const float ux = X / rho, uy = Y / rho;
  const float r00 = ct * cp * cp + sp * sp, r01 = ct * cp * sp - sp * cp, r02 = -cp * st;
  const float r10 = sp * ct * cp - cp * sp, r11 = ct * sp * sp + cp * cp, r12 = -sp * st;
  const float r20 = st * cp, r21 = st * sp, r22 = ct;
  kc[0] = w * (r00 + r02 * ux); kc[1] = w * (r01 + r02 * uy);
  kc[2] = w * (r10 + r12 * ux); kc[3] = w * (r11 + r12 * uy);
  kc[4] = w * (r20 + r22 * ux); kc[5] = w * (r21 + r22 * uy);
}

__device__ __forceinline__ void apply_highna(const float (&kc)[6], float2 (&e)[3]) {
  const float2 ex = e[0], ey = e[1];
  e[0] = cadd(cscale(ex, kc[0]), cscale(ey, kc[1]));
  e[1] = cadd(cscale(ex, kc[2]), cscale(ey, kc[3]));
  e[2] = cadd(cscale(ex, kc[4]), cscale(ey, kc[5]));
}

__device__ __forceinline__ void apply_highna_bwd(const float (&kc)[6], float2 (&g)[3]) {
  const float2 g0 = g[0], g1 = g[1], g2 = g[2];
  g[0] = cadd(cadd(cscale(g0, kc[0]), cscale(g1, kc[2])), cscale(g2, kc[4]));
  g[1] = cadd(cadd(cscale(g0, kc[1]), cscale(g1, kc[3])), cscale(g2, kc[5]));
  g[2] = make_float2(0.f, 0.f);
}

// The lens's Ez row alone (XL_OP_HIGHNA_EZ) and its backward: only e0
// depends on the input, gEx = K20 g0, gEy = K21 g0.
__device__ __forceinline__ void apply_highna_ez(const float (&kc)[6], float2 (&e)[3]) {
  const float2 ex = e[0], ey = e[1];
  e[0] = cadd(cscale(ex, kc[4]), cscale(ey, kc[5]));
  e[1] = make_float2(0.f, 0.f);
  e[2] = make_float2(0.f, 0.f);
}

__device__ __forceinline__ void apply_highna_ez_bwd(const float (&kc)[6], float2 (&g)[3]) {
  const float2 g0 = g[0];
  g[0] = cscale(g0, kc[4]);
  g[1] = cscale(g0, kc[5]);
  g[2] = make_float2(0.f, 0.f);
}

__device__ __forceinline__ float op_param(const XlOp& op, int i, const PixelCtx& px) {
  if (op.pmask & (1 << i)) {
    const float* p = (const float*)op.ptr[i];
    return __ldg(p + (long long)px.batch * op.pbstride + px.pix);
  }
  return op.sval[i];
}

// Per-pixel parameters read from the op's planes in global memory.
struct GlobalParams {
  __device__ __forceinline__ float operator()(const XlOp& op, int, int i, const PixelCtx& px) const {
    return op_param(op, i, px);
  }
};

// The LCD retarder (delta = 0) from cos, sin of eta/2 and of theta:
// a = ch - i sh (c^2 - s^2), b = c = -i sh 2 s c, d = ch + i sh (c^2 - s^2).
__device__ __forceinline__ void lcd_apply_trig(float ch, float sh, float ct, float st, float2 (&e)[3]) {
  const float c2 = ct * ct - st * st, s2 = 2.f * st * ct;
  const float2 a = make_float2(ch, -sh * c2);
  const float2 b = make_float2(0.f, -sh * s2);
  const float2 d = make_float2(ch, sh * c2);
  const float2 x = e[0], y = e[1];
  e[0] = cadd(cmul(a, x), cmul(b, y));
  e[1] = cadd(cmul(b, x), cmul(d, y));
}

// Op k of a program applied to one pixel's (Ex, Ey, Ez) (scalar fields use
// e[0] only), its kind a compile-time constant; its real parameters come from
// the reader pr(op, k, i, px).
template <int KIND, class PR>
__device__ __forceinline__ void apply_kind(const XlOp& op, int k, float2 (&e)[3], const PixelCtx& px,
                                           const PR& pr) {
  if constexpr (KIND == XL_OP_PHASE) {  // scalar SLM: field * e^{i phi}
    float s, c;
    phase_sincos(pr(op, k, 0, px), &s, &c);
    e[0] = cmul(e[0], make_float2(c, s));
  } else if constexpr (KIND == XL_OP_SSLM) {  // diag(e^{i a}, e^{i p}); Ez unchanged
    float s, c;
    phase_sincos(pr(op, k, 0, px), &s, &c);
    e[0] = cmul(e[0], make_float2(c, s));
    phase_sincos(pr(op, k, 1, px), &s, &c);
    e[1] = cmul(e[1], make_float2(c, s));
  } else if constexpr (KIND == XL_OP_SSLM_AMP) {  // diag(A1 e^{i a}, A2 e^{i p}); Ez unchanged
    float s, c;
    phase_sincos(pr(op, k, 0, px), &s, &c);
    e[0] = cscale(cmul(e[0], make_float2(c, s)), pr(op, k, 2, px));
    phase_sincos(pr(op, k, 1, px), &s, &c);
    e[1] = cscale(cmul(e[1], make_float2(c, s)), pr(op, k, 3, px));
  } else if constexpr (KIND == XL_OP_LCD) {  // general retarder with delta = 0 (eta, theta); Ez unchanged
    float sh, ch, st, ct;
    if (op.pmask & 1) phase_sincos(0.5f * pr(op, k, 0, px), &sh, &ch);
    else { ch = op.dval[0]; sh = op.dval[1]; }   // scalar eta: cos, sin of eta/2 from the host
    if (op.pmask & 2) phase_sincos(pr(op, k, 1, px), &st, &ct);
    else { ct = op.dval[2]; st = op.dval[3]; }   // scalar theta
    lcd_apply_trig(ch, sh, ct, st, e);
  } else if constexpr (KIND == XL_OP_LP) {  // linear polarizer at alpha; Ez set to zero
    float s, c;
    if (op.pmask & 1) phase_sincos(pr(op, k, 0, px), &s, &c);
    else { c = op.sval[2]; s = op.sval[3]; }   // scalar alpha: cos, sin from the host
    const float2 x = e[0], y = e[1];
    e[0] = cadd(cscale(x, c * c), cscale(y, c * s));
    e[1] = cadd(cscale(x, c * s), cscale(y, s * s));
    e[2] = make_float2(0.f, 0.f);
  } else if constexpr (KIND == XL_OP_SEPMASK) {  // separable complex mask ax[col]*ay[row] with an FP64 pupil test
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
  } else if constexpr (KIND == XL_OP_CMUL) {  // multiply every component by a per-pixel complex array
    const float2* p = (const float2*)op.ptr[0];
    const float2 m = p[(long long)px.batch * op.pbstride + px.pix];
    e[0] = cmul(e[0], m);
    e[1] = cmul(e[1], m);
    e[2] = cmul(e[2], m);
  } else if constexpr (KIND == XL_OP_HIGHNA) {  // optical_elements.py:528-594
    float kc[6];
    highna_coeffs(op, px, kc);
    apply_highna(kc, e);
  } else if constexpr (KIND == XL_OP_HIGHNA_EZ) {  // the lens's Ez row alone
    float kc[6];
    highna_coeffs(op, px, kc);
    apply_highna_ez(kc, e);
  }
}

// The switch over an op's kind, with BODY(K) run for the kind K.
#define XL_OP_SWITCH(kind, BODY)                          \
  switch (kind) {                                         \
    case XL_OP_PHASE: BODY(XL_OP_PHASE) break;            \
    case XL_OP_SSLM: BODY(XL_OP_SSLM) break;              \
    case XL_OP_SSLM_AMP: BODY(XL_OP_SSLM_AMP) break;      \
    case XL_OP_LCD: BODY(XL_OP_LCD) break;                \
    case XL_OP_LP: BODY(XL_OP_LP) break;                  \
    case XL_OP_SEPMASK: BODY(XL_OP_SEPMASK) break;        \
    case XL_OP_CMUL: BODY(XL_OP_CMUL) break;              \
    case XL_OP_HIGHNA: BODY(XL_OP_HIGHNA) break;          \
    case XL_OP_HIGHNA_EZ: BODY(XL_OP_HIGHNA_EZ) break;    \
    default: break;                                       \
  }

// Apply op number k of a program to one pixel.
template <class PR>
__device__ __forceinline__ void apply_op_r(const XlOp& op, int k, float2 (&e)[3], const PixelCtx& px,
                                           const PR& pr) {
#define XL_ONE_(K) apply_kind<K>(op, k, e, px, pr);
  XL_OP_SWITCH(op.kind, XL_ONE_)
#undef XL_ONE_
}

// Apply op number k to NPX pixels at once: the kind is dispatched once, and
// the pixels' loads and arithmetic are independent, so they overlap.
template <int NPX, class PR>
__device__ __forceinline__ void apply_op_vec(const XlOp& op, int k, float2 (&e)[NPX][3], const PixelCtx (&px)[NPX],
                                             const PR (&pr)[NPX]) {
#define XL_VEC_(K)                                            \
  _Pragma("unroll") for (int q = 0; q < NPX; ++q) apply_kind<K>(op, k, e[q], px[q], pr[q]);
  XL_OP_SWITCH(op.kind, XL_VEC_)
#undef XL_VEC_
}

template <int NPX, class PR>
__device__ __forceinline__ void apply_prog_vec(const XlProg& prog, float2 (&e)[NPX][3], const PixelCtx (&px)[NPX],
                                               const PR (&pr)[NPX]) {
  for (int i = 0; i < prog.nops; ++i) apply_op_vec<NPX>(prog.ops[i], i, e, px, pr);
}

// A program's op kinds as a compile-time list, for kernels specialised to
// the programs the tables run (FixedKinds<> : none, read them from the
// program).  at(k) folds to a constant once the caller's loop over k unrolls.
template <int... KS> struct FixedKinds {
  static constexpr int n = 0;
  __host__ __device__ static constexpr int at(int) { return XL_OP_NONE; }
  static bool matches(const XlProg&) { return false; }
};
template <int K0, int... KR> struct FixedKinds<K0, KR...> {
  static constexpr int n = 1 + sizeof...(KR);
  __host__ __device__ static constexpr int at(int k) { return k == 0 ? K0 : FixedKinds<KR...>::at(k - 1); }
  // the program has exactly these kinds, in this order
  static bool matches(const XlProg& p) {
    const int ks[] = {K0, KR...};
    if (p.nops != n) return false;
    for (int k = 0; k < n; ++k)
      if (p.ops[k].kind != ks[k]) return false;
    return true;
  }
};

// apply_prog_vec for a program whose kinds FK fixes (no switches): ops K..
template <class FK, int K = 0, int NPX, class PR>
__device__ __forceinline__ void apply_prog_fixed(const XlProg& prog, float2 (&e)[NPX][3],
                                                 const PixelCtx (&px)[NPX], const PR (&pr)[NPX]) {
  static_assert(FK::n > 0 && FK::n <= XL_MAX_OPS, "a fixed program");
  if constexpr (K < FK::n) {
#pragma unroll
    for (int q = 0; q < NPX; ++q) apply_kind<FK::at(K)>(prog.ops[K], K, e[q], px[q], pr[q]);
    apply_prog_fixed<FK, K + 1>(prog, e, px, pr);
  }
}

// The same for one pixel.
template <class FK, int K = 0, class PR>
__device__ __forceinline__ void apply_prog_fixed1(const XlProg& prog, float2 (&e)[3], const PixelCtx& px,
                                                  const PR& pr) {
  static_assert(FK::n > 0 && FK::n <= XL_MAX_OPS, "a fixed program");
  if constexpr (K < FK::n) {
    apply_kind<FK::at(K)>(prog.ops[K], K, e, px, pr);
    apply_prog_fixed1<FK, K + 1>(prog, e, px, pr);
  }
}

template <class PR>
__device__ __forceinline__ void apply_prog_r(const XlProg& prog, float2 (&e)[3], const PixelCtx& px, const PR& pr) {
  for (int i = 0; i < prog.nops; ++i) apply_op_r(prog.ops[i], i, e, px, pr);
}

__device__ __forceinline__ void apply_op(const XlOp& op, float2 (&e)[3], const PixelCtx& px) {
  apply_op_r(op, 0, e, px, GlobalParams{});
}

__device__ __forceinline__ void apply_prog(const XlProg& prog, float2 (&e)[3], const PixelCtx& px) {
  apply_prog_r(prog, e, px, GlobalParams{});
}

// ---- backward of one op ----
// e: the op's input (Ex, Ey, Ez); g: on entry the gradient of the op's output,
// on exit the gradient of its input (torch convention for complex tensors:
// g = 2 dL/d conj(y)).  pg[i] += dL/dp_i for the op's real parameters, where
// dL/dp = Re(sum_c g_c conj(dy_c/dp)).
__device__ __forceinline__ float re_gconj(float2 g, float2 d) { return g.x * d.x + g.y * d.y; }

// Backward of lcd_apply_trig: parameter gradients into pg[0] (eta), pg[1]
// (theta); g becomes J^H g (J symmetric: conj(J) g).
__device__ __forceinline__ void lcd_bwd_trig(float ch, float sh, float ct, float st, const float2 (&e)[3],
                                             float2 (&g)[3], float (&pg)[4]) {
  const float c2 = ct * ct - st * st, s2 = 2.f * st * ct;
  const float2 a = make_float2(ch, -sh * c2), bb = make_float2(0.f, -sh * s2), d = make_float2(ch, sh * c2);
  // derivatives of the matrix entries
  const float2 a_e = make_float2(-0.5f * sh, -0.5f * ch * c2), b_e = make_float2(0.f, -0.5f * ch * s2);
  const float2 d_e = make_float2(-0.5f * sh, 0.5f * ch * c2);
  const float2 a_t = make_float2(0.f, 2.f * sh * s2), b_t = make_float2(0.f, -2.f * sh * c2);
  const float2 d_t = make_float2(0.f, -2.f * sh * s2);
  const float2 x = e[0], y = e[1];
  pg[0] += re_gconj(g[0], cadd(cmul(a_e, x), cmul(b_e, y))) + re_gconj(g[1], cadd(cmul(b_e, x), cmul(d_e, y)));
  pg[1] += re_gconj(g[0], cadd(cmul(a_t, x), cmul(b_t, y))) + re_gconj(g[1], cadd(cmul(b_t, x), cmul(d_t, y)));
  const float2 g0 = g[0], g1 = g[1];
  g[0] = cadd(cmul(cconj(a), g0), cmul(cconj(bb), g1));
  g[1] = cadd(cmul(cconj(bb), g0), cmul(cconj(d), g1));
}

// The sines and cosines an op's forward and backward need, so that a caller
// that runs both (xl_ops_backward) evaluates them once: PHASE (c0, s0) of p0;
// sSLM (c0, s0) of p0 and (c1, s1) of p1; LCD (c0, s0) of eta/2 and (c1, s1)
// of theta; LP (c0, s0) of alpha.  Scalar parameters take the host's values.
// The kind is passed apart from the op so that a kernel specialised for a
// fixed program folds the switches below (the generic callers pass op.kind).
__device__ __forceinline__ float4 op_trig(int kind, const XlOp& op, const PixelCtx& px) {
  float4 t = make_float4(1.f, 0.f, 1.f, 0.f);   // (c0, s0, c1, s1)
  switch (kind) {
    case XL_OP_PHASE:
      phase_sincos(op_param(op, 0, px), &t.y, &t.x);
      break;
    case XL_OP_SSLM:
    case XL_OP_SSLM_AMP:
      phase_sincos(op_param(op, 0, px), &t.y, &t.x);
      phase_sincos(op_param(op, 1, px), &t.w, &t.z);
      break;
    case XL_OP_LCD:
      if (op.pmask & 1) phase_sincos(0.5f * op_param(op, 0, px), &t.y, &t.x);
      else { t.x = op.dval[0]; t.y = op.dval[1]; }
      if (op.pmask & 2) phase_sincos(op_param(op, 1, px), &t.w, &t.z);
      else { t.z = op.dval[2]; t.w = op.dval[3]; }
      break;
    case XL_OP_LP:
      if (op.pmask & 1) phase_sincos(op_param(op, 0, px), &t.y, &t.x);
      else { t.x = op.sval[2]; t.y = op.sval[3]; }
      break;
    default:
      break;
  }
  return t;
}
__device__ __forceinline__ float4 op_trig(const XlOp& op, const PixelCtx& px) { return op_trig(op.kind, op, px); }

// apply_op with the trig of op_trig (the same arithmetic as apply_op_r).
__device__ __forceinline__ void apply_op_t(int kind, const XlOp& op, const float4& t, float2 (&e)[3],
                                           const PixelCtx& px) {
  switch (kind) {
    case XL_OP_PHASE:
      e[0] = cmul(e[0], make_float2(t.x, t.y));
      break;
    case XL_OP_SSLM:
      e[0] = cmul(e[0], make_float2(t.x, t.y));
      e[1] = cmul(e[1], make_float2(t.z, t.w));
      break;
    case XL_OP_SSLM_AMP:
      e[0] = cscale(cmul(e[0], make_float2(t.x, t.y)), op_param(op, 2, px));
      e[1] = cscale(cmul(e[1], make_float2(t.z, t.w)), op_param(op, 3, px));
      break;
    case XL_OP_LCD:
      lcd_apply_trig(t.x, t.y, t.z, t.w, e);
      break;
    case XL_OP_LP: {
      const float c = t.x, s = t.y;
      const float2 x = e[0], y = e[1];
      e[0] = cadd(cscale(x, c * c), cscale(y, c * s));
      e[1] = cadd(cscale(x, c * s), cscale(y, s * s));
      e[2] = make_float2(0.f, 0.f);
      break;
    }
    default:
      apply_op(op, e, px);
      break;
  }
}
__device__ __forceinline__ void apply_op_t(const XlOp& op, const float4& t, float2 (&e)[3], const PixelCtx& px) {
  apply_op_t(op.kind, op, t, e, px);
}

__device__ __forceinline__ void apply_op_bwd_t(int kind, const XlOp& op, const float4& t, const float2 (&e)[3],
                                               float2 (&g)[3], const PixelCtx& px, float (&pg)[4]) {
  switch (kind) {
    case XL_OP_PHASE: {
      const float2 ph = make_float2(t.x, t.y);
      const float2 y = cmul(e[0], ph);
      pg[0] += re_gconj(g[0], make_float2(-y.y, y.x));   // dy/dphi = i y
      g[0] = cmulc(g[0], ph);
      break;
    }
    case XL_OP_SSLM:
    case XL_OP_SSLM_AMP: {
      const bool amp = kind == XL_OP_SSLM_AMP;
      const float2 p0 = make_float2(t.x, t.y);
      const float2 p1 = make_float2(t.z, t.w);
      const float a1 = amp ? op_param(op, 2, px) : 1.f, a2 = amp ? op_param(op, 3, px) : 1.f;
      const float2 u0 = cmul(e[0], p0), u1 = cmul(e[1], p1);   // before the amplitudes
      pg[0] += a1 * re_gconj(g[0], make_float2(-u0.y, u0.x));
      pg[1] += a2 * re_gconj(g[1], make_float2(-u1.y, u1.x));
      if (amp) {
        pg[2] += re_gconj(g[0], u0);
        pg[3] += re_gconj(g[1], u1);
      }
      g[0] = cscale(cmulc(g[0], p0), a1);
      g[1] = cscale(cmulc(g[1], p1), a2);
      break;
    }
    case XL_OP_LCD:
      lcd_bwd_trig(t.x, t.y, t.z, t.w, e, g, pg);
      break;
    case XL_OP_LP: {
      const float c = t.x, s = t.y;
      const float2 x = e[0], y = e[1];
      const float dcs = c * c - s * s, tcs = 2.f * c * s;
      pg[0] += re_gconj(g[0], cadd(cscale(x, -tcs), cscale(y, dcs))) +
               re_gconj(g[1], cadd(cscale(x, dcs), cscale(y, tcs)));
      const float2 g0 = g[0], g1 = g[1];
      g[0] = cadd(cscale(g0, c * c), cscale(g1, c * s));
      g[1] = cadd(cscale(g0, c * s), cscale(g1, s * s));
      g[2] = make_float2(0.f, 0.f);
      break;
    }
    case XL_OP_SEPMASK: {
      const float2 fc = ((const float2*)op.ptr[0])[px.col];
      const float2 fr = ((const float2*)op.ptr[1])[px.row];
      float2 m = cmul(fc, fr);
      if (op.ptr[2]) {
        const double tc = ((const double*)op.ptr[2])[px.col];
        const double tr = ((const double*)op.ptr[3])[px.row];
        if (!(tc + tr < 1.0)) m = make_float2(0.f, 0.f);
      }
      g[0] = cmulc(g[0], m);
      g[1] = cmulc(g[1], m);
      g[2] = op.sval[0] != 0.f ? make_float2(0.f, 0.f) : cmulc(g[2], m);
      break;
    }
    case XL_OP_CMUL: {
      const float2 m = ((const float2*)op.ptr[0])[(long long)px.batch * op.pbstride + px.pix];
      g[0] = cmulc(g[0], m);
      g[1] = cmulc(g[1], m);
      g[2] = cmulc(g[2], m);
      break;
    }
    case XL_OP_HIGHNA: {
      float kc[6];
      highna_coeffs(op, px, kc);
      apply_highna_bwd(kc, g);
      break;
    }
    case XL_OP_HIGHNA_EZ: {
      float kc[6];
      highna_coeffs(op, px, kc);
      apply_highna_ez_bwd(kc, g);
      break;
    }
    default:
      break;
  }
}

__device__ __forceinline__ void apply_op_bwd_t(const XlOp& op, const float4& t, const float2 (&e)[3],
                                               float2 (&g)[3], const PixelCtx& px, float (&pg)[4]) {
  apply_op_bwd_t(op.kind, op, t, e, g, px, pg);
}

__device__ __forceinline__ void apply_op_bwd(int kind, const XlOp& op, const float2 (&e)[3], float2 (&g)[3],
                                             const PixelCtx& px, float (&pg)[4]) {
  apply_op_bwd_t(kind, op, op_trig(kind, op, px), e, g, px, pg);
}
__device__ __forceinline__ void apply_op_bwd(const XlOp& op, const float2 (&e)[3], float2 (&g)[3],
                                             const PixelCtx& px, float (&pg)[4]) {
  apply_op_bwd(op.kind, op, e, g, px, pg);
}

}  // namespace xl

// ---- TMA bulk copies into shared memory, completed on an mbarrier ----
namespace xl {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Make prior generic-proxy shared-memory accesses visible to the async proxy
// (the TMA engine) before it overwrites the same buffer.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: arm the barrier for `bytes` and start a 1-D bulk copy
// global -> shared (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* mbar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Arm the barrier for `bytes` of bulk copies (one arrival, by one thread).
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
               : "memory");
}

// One bulk copy global -> shared completing on an armed barrier (16-byte
// aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes,
                                              unsigned long long* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

// Bring `bytes` (a multiple of 16, 16-byte aligned start) of global memory
// into L2 ahead of use (one thread; no registers or shared memory held).
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// ---- bounded waits and the error status they report ----
// Each translation unit has its own copies (filled at device set-up):
// a count of waits that ran out, the wait limit, and the device address of a
// word in mapped host memory that a kernel sets when one of its waits runs
// out, so that the host sees the event without synchronising.
static __device__ unsigned int g_line_timeouts;
static __device__ unsigned long long g_wait_limit_ns = 1000000000ull;
static __device__ unsigned int* g_status_word;
constexpr unsigned long long kDrainLimitNs = 1000000000ull;

// Bounded wait for phase `phase` of the barrier: gives up after `limit_ns`
// of wall time and returns false (it never spins forever).  A limit of 0
// gives up without waiting (the test setting of xl_set_wait_limit).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* mbar, unsigned phase,
                                                  unsigned long long limit_ns = kDrainLimitNs) {
  if (limit_ns == 0) return false;
  if (mbar_try_wait(mbar, phase)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(mbar, phase)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// A wait ran out: count it and raise the host-visible status word.
__device__ __forceinline__ void record_timeout() {
  atomicAdd(&g_line_timeouts, 1u);
  if (g_status_word) {
    *(volatile unsigned int*)g_status_word = 1u;
    __threadfence_system();
  }
}

}  // namespace xl
