// Two-line complex64 FFT engine on Blackwell's packed FP32 instructions
// (add / mul / fma .rn.f32x2, sm_100 and later).
//
// A thread holds 16 "pair" elements: element m of two independent lines a
// and b, stored split as re = (re_a, re_b) and im = (im_a, im_b).  Every
// butterfly operation is then the same for both lines, so each one is one
// packed instruction for two complex values instead of two scalar ones; the
// FP32 instruction count of a transform, which bounds the propagators' column
// and row passes, halves.  Exchanges between passes move a pair element as
// one 16-byte shared-memory access.
//
// The pass structure is the one of fft_core.cuh (Stockham autosort, radix-16
// passes plus one radix-2/4/8 pass, thread j holding elements j + m T), and
// so are its index tables; only the arithmetic and the slot width differ.
// Twiddle tables hold (wr, wr, wi, wi) per entry, the pair form of the
// float64-derived pass tables (PairTw below).
//
// Every function is host+device: the CPU harness runs the exact pass code
// thread by thread with scalar stand-ins for the packed instructions.
#pragma once

#include "fft_core.cuh"

namespace xl {

#if defined(__CUDACC__)
using f4 = float4;
XL_HD f4 mk4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
#else
struct float4 { float x, y, z, w; };
using f4 = float4;
inline f4 mk4(float a, float b, float c, float d) { f4 r; r.x = a; r.y = b; r.z = c; r.w = d; return r; }
#endif

// ---- packed FP32 on (x, y) lanes ----
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as b * (-1) + a: exact, one instruction
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
#else
inline float2 f2add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
inline float2 f2mul(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
inline float2 f2fma(float2 a, float2 b, float2 c) {
  return make_float2(std::fma(a.x, b.x, c.x), std::fma(a.y, b.y, c.y));
}
inline float2 f2sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif
XL_HD float2 f2s(float s) { return make_float2(s, s); }

// Element m of two lines: re = (re_a, re_b), im = (im_a, im_b).
struct cpair {
  float2 re, im;
};

XL_HD cpair pz() { cpair r; r.re = make_float2(0.f, 0.f); r.im = r.re; return r; }
XL_HD cpair padd(cpair a, cpair b) { cpair r; r.re = f2add(a.re, b.re); r.im = f2add(a.im, b.im); return r; }
XL_HD cpair psub(cpair a, cpair b) { cpair r; r.re = f2sub(a.re, b.re); r.im = f2sub(a.im, b.im); return r; }
// a + DIR i b and a - DIR i b (the multiply by +-i folded into the add)
template <int DIR> XL_HD cpair padd_i(cpair a, cpair b) {
  cpair r;
  if (DIR < 0) { r.re = f2add(a.re, b.im); r.im = f2sub(a.im, b.re); }   // a - i b
  else { r.re = f2sub(a.re, b.im); r.im = f2add(a.im, b.re); }           // a + i b
  return r;
}
template <int DIR> XL_HD cpair psub_i(cpair a, cpair b) { return padd_i<-DIR>(a, b); }

// x * (c + i s) for a constant (c, s), the same for both lines: four instructions.
XL_HD cpair pmul_c(cpair x, float c, float s) {
  cpair r;
  r.re = f2fma(x.im, f2s(-s), f2mul(x.re, f2s(c)));
  r.im = f2fma(x.re, f2s(s), f2mul(x.im, f2s(c)));
  return r;
}
// x * w (CONJ false) or x * conj(w) for a table twiddle w = (wr, wr, wi, wi).
template <bool CONJ> XL_HD cpair pmul_w(cpair x, f4 w) {
  const float2 wr = make_float2(w.x, w.y), wi = make_float2(w.z, w.w);
  cpair r;
  if (!CONJ) {
    r.re = f2sub(f2mul(x.re, wr), f2mul(x.im, wi));
    r.im = f2fma(x.re, wi, f2mul(x.im, wr));
  } else {
    r.re = f2fma(x.im, wi, f2mul(x.re, wr));
    r.im = f2sub(f2mul(x.im, wr), f2mul(x.re, wi));
  }
  return r;
}
// x * s and x * conj(s) for per-line values s = (sr_a, sr_b) + i (si_a, si_b).
template <bool CONJ> XL_HD cpair pmul_pp(cpair x, float2 sr, float2 si) {
  cpair r;
  if (!CONJ) {
    r.re = f2sub(f2mul(x.re, sr), f2mul(x.im, si));
    r.im = f2fma(x.re, si, f2mul(x.im, sr));
  } else {
    r.re = f2fma(x.im, si, f2mul(x.re, sr));
    r.im = f2sub(f2mul(x.im, sr), f2mul(x.re, si));
  }
  return r;
}
XL_HD cpair pscale(cpair x, float2 s) { cpair r; r.re = f2mul(x.re, s); r.im = f2mul(x.im, s); return r; }

// Pack / unpack two interleaved complex64 values (a_re, a_im, b_re, b_im).
XL_HD cpair p_from(f4 v) { cpair r; r.re = make_float2(v.x, v.z); r.im = make_float2(v.y, v.w); return r; }
XL_HD f4 p_to(cpair v) { return mk4(v.re.x, v.im.x, v.re.y, v.im.y); }
XL_HD cpair p_from2(float2 a, float2 b) { cpair r; r.re = make_float2(a.x, b.x); r.im = make_float2(a.y, b.y); return r; }
XL_HD float2 p_lo(cpair v) { return make_float2(v.re.x, v.im.x); }
XL_HD float2 p_hi(cpair v) { return make_float2(v.re.y, v.im.y); }
// Shared-memory slot form: (re_a, re_b, im_a, im_b).
XL_HD f4 p_slot(cpair v) { return mk4(v.re.x, v.re.y, v.im.x, v.im.y); }
XL_HD cpair p_unslot(f4 s) { cpair r; r.re = make_float2(s.x, s.y); r.im = make_float2(s.z, s.w); return r; }

// Twiddle e^{DIR 2 pi i e / 16} applied to x (e a compile-time constant, e != 4).
template <int DIR, int E16> XL_HD cpair pmul_w16(cpair x) {
  constexpr float C1 = 0.92387953251128675613f;  // cos(pi/8)
  constexpr float S1 = 0.38268343236508977173f;  // sin(pi/8)
  constexpr float R2 = 0.70710678118654752440f;  // sqrt(1/2)
  constexpr int e = E16 & 15;
  static_assert(e != 4 && e != 12, "quarter turns are folded into the adds");
  if constexpr (e == 0) return x;
  else if constexpr (e == 8) { cpair r; r.re = f2sub(f2s(0.f), x.re); r.im = f2sub(f2s(0.f), x.im); return r; }
  else {
    constexpr float c = e == 1 ? C1 : e == 2 ? R2 : e == 3 ? S1 : e == 5 ? -S1 : e == 6 ? -R2 : e == 7 ? -C1
                      : e == 9 ? -C1 : e == 10 ? -R2 : e == 11 ? -S1 : e == 13 ? S1 : e == 14 ? R2 : C1;
    constexpr float s = e == 1 ? S1 : e == 2 ? R2 : e == 3 ? C1 : e == 5 ? C1 : e == 6 ? R2 : e == 7 ? S1
                      : e == 9 ? -S1 : e == 10 ? -R2 : e == 11 ? -C1 : e == 13 ? -C1 : e == 14 ? -R2 : -S1;
    return pmul_c(x, c, DIR * s);
  }
}

// ---- small DFTs on pair elements, natural-order output ----

// DFT4 of (a0, a1, a2, a3); ROT2: a2 is first multiplied by DIR i (the w16^4
// twiddle of the DFT16), folded into the first adds.
template <int DIR, bool ROT2 = false>
XL_HD void pdft4(cpair& a0, cpair& a1, cpair& a2, cpair& a3) {
  const cpair s02 = ROT2 ? padd_i<DIR>(a0, a2) : padd(a0, a2);
  const cpair d02 = ROT2 ? psub_i<DIR>(a0, a2) : psub(a0, a2);
  const cpair s13 = padd(a1, a3), t13 = psub(a1, a3);
  a0 = padd(s02, s13);
  a2 = psub(s02, s13);
  a1 = padd_i<DIR>(d02, t13);
  a3 = psub_i<DIR>(d02, t13);
}

template <int DIR> XL_HD void pdft2(cpair* a) {
  const cpair t = a[0];
  a[0] = padd(t, a[1]);
  a[1] = psub(t, a[1]);
}

template <int DIR> XL_HD void pdft8(cpair* a) {
  cpair e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  cpair o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  pdft4<DIR>(e0, e1, e2, e3);
  pdft4<DIR>(o0, o1, o2, o3);
  o1 = pmul_w16<DIR, 2>(o1);
  o3 = pmul_w16<DIR, 6>(o3);
  a[0] = padd(e0, o0); a[4] = psub(e0, o0);
  a[1] = padd(e1, o1); a[5] = psub(e1, o1);
  a[2] = padd_i<DIR>(e2, o2); a[6] = psub_i<DIR>(e2, o2);   // o2 * w16^4 = DIR i o2
  a[3] = padd(e3, o3); a[7] = psub(e3, o3);
}

// Second half of the 4 x 4 DFT16: twiddles w16^(n2 k1), outer DFT4s, transpose.
template <int DIR> XL_HD void pdft16_tail(cpair* a) {
  a[5] = pmul_w16<DIR, 1>(a[5]);
  a[9] = pmul_w16<DIR, 2>(a[9]);
  a[13] = pmul_w16<DIR, 3>(a[13]);
  a[6] = pmul_w16<DIR, 2>(a[6]);
  a[14] = pmul_w16<DIR, 6>(a[14]);
  a[7] = pmul_w16<DIR, 3>(a[7]);
  a[11] = pmul_w16<DIR, 6>(a[11]);
  a[15] = pmul_w16<DIR, 9>(a[15]);
  pdft4<DIR>(a[0], a[1], a[2], a[3]);
  pdft4<DIR>(a[4], a[5], a[6], a[7]);
  pdft4<DIR, true>(a[8], a[9], a[10], a[11]);   // a[10] carries w16^4
  pdft4<DIR>(a[12], a[13], a[14], a[15]);
  cpair t[16];
#pragma unroll
  for (int s = 0; s < 16; ++s) t[s] = a[s];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = t[4 * (k & 3) + (k >> 2)];
}

template <int DIR> XL_HD void pdft16(cpair* a) {
  pdft4<DIR>(a[0], a[4], a[8], a[12]);
  pdft4<DIR>(a[1], a[5], a[9], a[13]);
  pdft4<DIR>(a[2], a[6], a[10], a[14]);
  pdft4<DIR>(a[3], a[7], a[11], a[15]);
  pdft16_tail<DIR>(a);
}

// DFT16 of a[0..7] with a[8..15] zero: the inner DFT4s see two inputs each.
template <int DIR> XL_HD void pdft16_half(cpair* a) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    const cpair x0 = a[n2], x1 = a[n2 + 4];
    a[n2] = padd(x0, x1);
    a[n2 + 4] = padd_i<DIR>(x0, x1);
    a[n2 + 8] = psub(x0, x1);
    a[n2 + 12] = psub_i<DIR>(x0, x1);
  }
  pdft16_tail<DIR>(a);
}

template <int R, int DIR> XL_HD void pdftR(cpair* a) {
  if constexpr (R == 2) pdft2<DIR>(a);
  else if constexpr (R == 4) pdft4<DIR>(a[0], a[1], a[2], a[3]);
  else if constexpr (R == 8) pdft8<DIR>(a);
  else pdft16<DIR>(a);
}

// ---- pair twiddle tables: pass table entry q of FftTw<LOGN, 16> as
// (wr, wr, wi, wi) ----
template <int LOGN> struct PairTw {
  static constexpr int SIZE = FftTw<LOGN, 16>::SIZE;
};
XL_HD f4 pair_tw(float2 w) { return mk4(w.x, w.x, w.y, w.y); }

// Twiddle read: the read-only path for a table in global memory (GTW), an
// ordinary load for one in shared memory.
template <bool GTW> XL_HD f4 tw4_load(const f4* p) {
#if defined(__CUDA_ARCH__)
  if constexpr (GTW) return __ldg(p);
#endif
  return *p;
}

// Slot offset of the two-line exchange buffers: smpad, as fft_core.cuh.
// One Stockham pass for thread j (16 pair elements, layout v[m] = x[j + m T]).
// ZU: first pass of a zero-padded line (v[8..15] zero, never read).
template <int LOGN, int P, int DIR, bool ZU, bool GTW>
XL_HD void pfft_pass(cpair (&v)[16], int j, f4* sm, const f4* stw, int toff) {
  using S = FftShape<LOGN, 16>;
  constexpr int R = S::template radix<P>();
  constexpr int NS = S::template stride<P>();
  constexpr bool LAST = (P == S::NPASS - 1);
  constexpr int BPT = 16 / R;
  constexpr int OFF = FftTw<LOGN, 16>::template off<P>();
  constexpr bool CONJ = DIR > 0;
  static_assert(!ZU || (P == 0 && R == 16), "input pruning is for a first radix-16 pass");
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = j + t * S::T;
    const int k = b & (NS - 1);
    cpair x[R];
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = (ZU && i >= R / 2) ? pz() : v[t + i * BPT];
    if constexpr (R == 16 && NS > 1) {
      // twiddle the inputs of one inner DFT4 at a time, so that only four
      // twiddles are live at once
#pragma unroll
      for (int n2 = 0; n2 < 4; ++n2) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = n2 + 4 * q;
          if (i == 0) continue;
          x[i] = pmul_w<CONJ>(x[i], tw4_load<GTW>(stw + toff + OFF + (i - 1) * NS + k));
        }
        pdft4<DIR>(x[n2], x[n2 + 4], x[n2 + 8], x[n2 + 12]);
      }
      pdft16_tail<DIR>(x);
    } else {
      if constexpr (NS > 1) {
#pragma unroll
        for (int i = 1; i < R; ++i) x[i] = pmul_w<CONJ>(x[i], tw4_load<GTW>(stw + toff + OFF + (i - 1) * NS + k));
      }
      if constexpr (ZU) pdft16_half<DIR>(x);
      else pdftR<R, DIR>(x);
    }
    if constexpr (LAST) {
#pragma unroll
      for (int i = 0; i < R; ++i) v[t + i * BPT] = x[i];
    } else {
      const int base = (b / NS) * (NS * R) + k;
      if constexpr (NS % 16 == 0 || (NS == 1 && R == 16)) {
        constexpr int STEP = NS == 1 ? 1 : NS + NS / 16;
        f4* d = sm + smpad(base);
#pragma unroll
        for (int i = 0; i < R; ++i) d[i * STEP] = p_slot(x[i]);
      } else {
#pragma unroll
        for (int i = 0; i < R; ++i) sm[smpad(base + i * NS)] = p_slot(x[i]);
      }
    }
  }
}

template <int LOGN> XL_HD void pfft_gather(cpair (&v)[16], int j, const f4* sm) {
  using S = FftShape<LOGN, 16>;
  if constexpr (S::T % 16 == 0) {
    const f4* s = sm + smpad(j);
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = p_unslot(s[m * (S::T + S::T / 16)]);
  } else {
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = p_unslot(sm[smpad(j + m * S::T)]);
  }
}

#if defined(__CUDACC__)
// Whole two-line FFT for a thread group; `sync` is the barrier between passes
// (CtaSync or GroupSync of fft_core.cuh).  The twiddle offset is laundered per
// transform, as in block_fft_x, so that back-to-back transforms reload the
// twiddles instead of keeping them live.
template <int LOGN, int DIR, bool ZU, bool GTW, class SYNC = CtaSync, int P = 0>
__device__ __forceinline__ void block_pfft(cpair (&v)[16], int j, f4* sm, const f4* stw, const SYNC& sync = SYNC(),
                                           int toff = -1) {
  using S = FftShape<LOGN, 16>;
  if constexpr (P == 0) {
    toff = 0;
    asm volatile("" : "+r"(toff));
  }
  pfft_pass<LOGN, P, DIR, ZU && P == 0, GTW>(v, j, sm, stw, toff);
  if constexpr (P < S::NPASS - 1) {
    sync();
    pfft_gather<LOGN>(v, j, sm);
    sync();
    block_pfft<LOGN, DIR, false, GTW, SYNC, P + 1>(v, j, sm, stw, sync, toff);
  }
}
#endif

}  // namespace xl
