// 4096-point transforms as two radix-64 passes: a line is transformed by 64
// threads holding 64 elements each, with one shared-memory exchange per
// transform (the radix-16 engine of fft_core.cuh needs two at this length).
//
// Four-step decomposition, n = j + 64 m and k = k1 + 64 k2:
//   pass 0, thread j:   Y[j][k1] = sum_m x[j + 64 m] w64^(m k1), then the
//                       twiddle w4096^(j k1), written to the exchange buffer;
//   pass 1, thread k1:  X[k1 + 64 k2] = sum_j Y[j][k1] w64^(j k2).
// Thread j holds v[m] = x[j + 64 m] on entry and X[j + 64 m] on exit (the
// layout of fft_core.cuh with T = 64), so loads and stores stay coalesced.
//
// Exchange slots: element L = 64 a + b of a line sits at 69 a + b (five pad
// slots per 64).  With four lines interleaved in the lanes of a warp (lane =
// 4 (j % 8) + line) and lines F64_XB slots apart, the pass-0 writes (a = j)
// and the pass-1 gathers (b = j) of every half-warp fall on 16 distinct
// 8-byte bank pairs.
//
// Every function is host+device so the CPU harness runs the pass code thread
// by thread against numpy.
#pragma once

#include "fft_core.cuh"

namespace xl {

constexpr int F64_ROW = 69;                 // slots per 64 elements (5 pad slots)
constexpr int F64_XS = 64 * F64_ROW;        // 4416 slots per line
constexpr int F64_XB = F64_XS + 4;          // line stride of four interleaved lines

// cos(2 pi r / 64), r = 0..16 (decimal expansions of the constants).
XL_HD constexpr float kcos64(int r) {
  return r == 0    ? 1.0f
         : r == 1  ? 0.99518472667219688624f
         : r == 2  ? 0.98078528040323044913f
         : r == 3  ? 0.95694033573220886494f
         : r == 4  ? 0.92387953251128675613f
         : r == 5  ? 0.88192126434835502971f
         : r == 6  ? 0.83146961230254523708f
         : r == 7  ? 0.77301045336273696081f
         : r == 8  ? 0.70710678118654752440f
         : r == 9  ? 0.63439328416364549822f
         : r == 10 ? 0.55557023301960222474f
         : r == 11 ? 0.47139673682599764856f
         : r == 12 ? 0.38268343236508977173f
         : r == 13 ? 0.29028467725446236764f
         : r == 14 ? 0.19509032201612826785f
         : r == 15 ? 0.09801714032956060199f
                   : 0.0f;
}

// a * e^{DIR 2 pi i e / 64}; e is a constant once the callers' loops unroll,
// so the branches and the constants fold.
template <int DIR> XL_HD float2 cmul_w64(float2 a, int e) {
  e &= 63;
  if (e == 0) return a;
  if (e == 16) return cmul_dir_i<DIR>(a);
  if (e == 32) return make_float2(-a.x, -a.y);
  if (e == 48) return cmul_dir_i<-DIR>(a);
  const int q = e >> 4, r = e & 15;
  const float cr = kcos64(r), sr = kcos64(16 - r);
  const float c = q == 0 ? cr : (q == 1 ? -sr : (q == 2 ? -cr : sr));
  const float s = q == 0 ? sr : (q == 1 ? cr : (q == 2 ? -sr : -cr));
  return cmul(a, make_float2(c, DIR * s));
}

// 8-point DFT of a[0..3] when a[4..7] are zero (not read).
template <int DIR> XL_HD void dft8_half(float2* a) {
  const float2 t0 = a[0], t1 = a[1], t2 = a[2], t3 = a[3];
  const float2 it2 = cmul_dir_i<DIR>(t2), it3 = cmul_dir_i<DIR>(t3);
  const float2 e0 = cadd(t0, t2), e1 = cadd(t0, it2), e2 = csub(t0, t2), e3 = csub(t0, it2);
  float2 o0 = cadd(t1, t3), o1 = cadd(t1, it3), o2 = csub(t1, t3), o3 = csub(t1, it3);
  o1 = cmul_w16<DIR, 2>(o1);
  o2 = cmul_w16<DIR, 4>(o2);
  o3 = cmul_w16<DIR, 6>(o3);
  a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
  a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
  a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
  a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
}

// 8-point DFT whose outputs a[4..7] are not needed (left undefined).
template <int DIR> XL_HD void dft8_lo(float2* a) {
  float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  float2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<DIR>(e0, e1, e2, e3);
  dft4<DIR>(o0, o1, o2, o3);
  o1 = cmul_w16<DIR, 2>(o1);
  o2 = cmul_w16<DIR, 4>(o2);
  o3 = cmul_w16<DIR, 6>(o3);
  a[0] = cadd(e0, o0);
  a[1] = cadd(e1, o1);
  a[2] = cadd(e2, o2);
  a[3] = cadd(e3, o3);
}

// 64-point DFT in registers, natural order in and out, as 8 x 8: inner DFT8s
// over the stride-8 subsequences (n = n2 + 8 n1), twiddles w64^(n2 k1),
// outer DFT8s over n2.  ZIN: a[32..63] are zero and not read.  ZOUT: only
// X[0..31] are produced (a[32..63] undefined on exit).
template <int DIR, bool ZIN, bool ZOUT> XL_HD void dft64(float2 (&a)[64]) {
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) {
    float2 t[8];
#pragma unroll
    for (int n1 = 0; n1 < (ZIN ? 4 : 8); ++n1) t[n1] = a[n2 + 8 * n1];
    if constexpr (ZIN) dft8_half<DIR>(t);
    else dft8<DIR>(t);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) a[n2 + 8 * k1] = cmul_w64<DIR>(t[k1], n2 * k1);
  }
  // slot n2 + 8 k1 holds Y[n2][k1]
  float2 r[64];
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    float2 t[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) t[n2] = a[n2 + 8 * k1];
    if constexpr (ZOUT) dft8_lo<DIR>(t);
    else dft8<DIR>(t);
#pragma unroll
    for (int k2 = 0; k2 < (ZOUT ? 4 : 8); ++k2) r[k1 + 8 * k2] = t[k2];
  }
#pragma unroll
  for (int k = 0; k < (ZOUT ? 32 : 64); ++k) a[k] = r[k];
}

// Pass-0 twiddle table for thread j: tw[k * 64 + j] = e^{-2 pi i j k / 4096},
// from the size-4096 table tw4096[q] = e^{-2 pi i q / 4096}.
XL_HD float2 f64_twiddle_entry(int idx, const float2* tw4096) {
  return tw4096[((idx >> 6) * (idx & 63)) & 4095];
}

// Pass 0, thread j: DFT64 of v (pruned when ZIN) in place; the exchange
// write is separate (f64_write) so that a kernel can put a barrier between.
template <int DIR, bool ZIN> XL_HD void f64_pass0(float2 (&v)[64]) { dft64<DIR, ZIN, false>(v); }

// Twiddle Y[j][k] by w4096^(DIR j k) (DIR < 0: tw, DIR > 0: its conjugate) and
// write it to slot 69 j + k of the line's exchange buffer xb.
template <int DIR> XL_HD void f64_write(const float2 (&v)[64], int j, float2* xb, const float2* tw) {
  float2* d = xb + F64_ROW * j;
  d[0] = v[0];
#pragma unroll
  for (int k = 1; k < 64; ++k) {
    const float2 w = tw[k * 64 + j];
    d[k] = DIR < 0 ? cmul(v[k], w) : cmulc(v[k], w);
  }
}

// Pass 1, thread j: gather Y[b][j] (slot 69 b + j), DFT64 over b; v[k2] =
// X[j + 64 k2] on exit (only k2 < 32 when ZOUT).
template <int DIR, bool ZOUT> XL_HD void f64_pass1(float2 (&v)[64], int j, const float2* xb) {
  const float2* s = xb + j;
#pragma unroll
  for (int b = 0; b < 64; ++b) v[b] = s[b * F64_ROW];
  dft64<DIR, false, ZOUT>(v);
}

}  // namespace xl
