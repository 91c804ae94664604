// Block-level complex64 FFT engine (Stockham autosort, radix-16 passes plus one
// radix-2/4/8 pass), shared by every propagation kernel of the library.
//
// Layout contract: an FFT of length N = 2^LOGN is computed by a group of
// T = N/E threads (E = 16 or 8 elements per thread); thread j holds
// v[m] = x[j + m*T] (m < E) on entry and X[j + m*T] on exit, so loads and
// stores of whole lines are coalesced.
// Between passes the group exchanges data through a padded shared-memory
// buffer of N + N/16 float2 (one pad slot every 16 elements keeps the
// stride-16 writes of the first pass free of bank conflicts).
//
// Every function here is host+device so the exact pass code can be exercised
// on the CPU by a harness that runs the T "threads" of a group in sequence.
#pragma once

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define XL_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#include <cstdint>
struct float2 { float x, y; };
inline float2 make_float2(float a, float b) { float2 r; r.x = a; r.y = b; return r; }
#define XL_HD inline
#endif

namespace xl {

XL_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
XL_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
XL_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
XL_HD float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
XL_HD float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
XL_HD float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * (DIR * i): DIR = -1 gives a * (-i), DIR = +1 gives a * i
template <int DIR> XL_HD float2 cmul_dir_i(float2 a) {
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// Twiddle w = e^{DIR * 2 pi i * num / den} applied to a, num/den a compile-time fraction.
// cos/sin of multiples of pi/8 written out (exact decimal expansions of the constants).
template <int DIR, int E16> XL_HD float2 cmul_w16(float2 a) {
  // e^{DIR 2 pi i E16/16}
  constexpr float C1 = 0.92387953251128675613f;  // cos(pi/8)
  constexpr float S1 = 0.38268343236508977173f;  // sin(pi/8)
  constexpr float R2 = 0.70710678118654752440f;  // sqrt(1/2)
  constexpr int e = E16 & 15;
  float c, s;
  if (e == 0) { c = 1.f; s = 0.f; }
  else if (e == 1) { c = C1; s = S1; }
  else if (e == 2) { c = R2; s = R2; }
  else if (e == 3) { c = S1; s = C1; }
  else if (e == 4) { c = 0.f; s = 1.f; }
  else if (e == 5) { c = -S1; s = C1; }
  else if (e == 6) { c = -R2; s = R2; }
  else if (e == 7) { c = -C1; s = S1; }
  else if (e == 8) { c = -1.f; s = 0.f; }
  else if (e == 9) { c = -C1; s = -S1; }
  else if (e == 10) { c = -R2; s = -R2; }
  else if (e == 11) { c = -S1; s = -C1; }
  else if (e == 12) { c = 0.f; s = -1.f; }
  else if (e == 13) { c = S1; s = -C1; }
  else if (e == 14) { c = R2; s = -R2; }
  else { c = C1; s = -S1; }
  if (e == 0) return a;
  if (e == 4) return cmul_dir_i<DIR>(a);
  if (e == 8) return make_float2(-a.x, -a.y);
  if (e == 12) return cmul_dir_i<-DIR>(a);
  return cmul(a, make_float2(c, DIR * s));
}

// ---- small DFTs in registers, natural-order output, no normalisation ----

template <int DIR> XL_HD void dft2(float2* a) {
  float2 t = a[0];
  a[0] = cadd(t, a[1]);
  a[1] = csub(t, a[1]);
}

template <int DIR> XL_HD void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 s02 = cadd(a0, a2), d02 = csub(a0, a2);
  float2 s13 = cadd(a1, a3), d13 = cmul_dir_i<DIR>(csub(a1, a3));
  a0 = cadd(s02, s13);
  a2 = csub(s02, s13);
  a1 = cadd(d02, d13);
  a3 = csub(d02, d13);
}

template <int DIR> XL_HD void dft4(float2* a) { dft4<DIR>(a[0], a[1], a[2], a[3]); }

template <int DIR> XL_HD void dft8(float2* a) {
  // X[k] = E[k] + w8^k O[k], X[k+4] = E[k] - w8^k O[k]
  float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  float2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<DIR>(e0, e1, e2, e3);
  dft4<DIR>(o0, o1, o2, o3);
  o1 = cmul_w16<DIR, 2>(o1);
  o2 = cmul_w16<DIR, 4>(o2);
  o3 = cmul_w16<DIR, 6>(o3);
  a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
  a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
  a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
  a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
}

template <int DIR> XL_HD void dft16_tail(float2* a);

template <int DIR> XL_HD void dft16(float2* a) {
  // 4 x 4: inner DFT4 over stride-4 subsequences, twiddle w16^(n2 k1), outer DFT4.
  dft4<DIR>(a[0], a[4], a[8], a[12]);
  dft4<DIR>(a[1], a[5], a[9], a[13]);
  dft4<DIR>(a[2], a[6], a[10], a[14]);
  dft4<DIR>(a[3], a[7], a[11], a[15]);
  dft16_tail<DIR>(a);
}

// 16-point DFT of a[0..7] when a[8..15] are zero (a zero-padded line): the
// inner DFT4s see two nonzero inputs each.
template <int DIR> XL_HD void dft16_half(float2* a) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    const float2 x0 = a[n2], x1 = a[n2 + 4];
    const float2 ix1 = cmul_dir_i<DIR>(x1);
    a[n2] = cadd(x0, x1);
    a[n2 + 4] = cadd(x0, ix1);
    a[n2 + 8] = csub(x0, x1);
    a[n2 + 12] = csub(x0, ix1);
  }
  dft16_tail<DIR>(a);
}

// Second half of the 4 x 4 DFT16: twiddles w16^(n2 k1), outer DFT4s, transpose.
template <int DIR> XL_HD void dft16_tail(float2* a) {
  // slot n2 + 4 k1 holds Y[n2][k1]
  a[5] = cmul_w16<DIR, 1>(a[5]);
  a[9] = cmul_w16<DIR, 2>(a[9]);
  a[13] = cmul_w16<DIR, 3>(a[13]);
  a[6] = cmul_w16<DIR, 2>(a[6]);
  a[10] = cmul_w16<DIR, 4>(a[10]);
  a[14] = cmul_w16<DIR, 6>(a[14]);
  a[7] = cmul_w16<DIR, 3>(a[7]);
  a[11] = cmul_w16<DIR, 6>(a[11]);
  a[15] = cmul_w16<DIR, 9>(a[15]);
  dft4<DIR>(a[0], a[1], a[2], a[3]);
  dft4<DIR>(a[4], a[5], a[6], a[7]);
  dft4<DIR>(a[8], a[9], a[10], a[11]);
  dft4<DIR>(a[12], a[13], a[14], a[15]);
  // slot 4 k1 + k2 holds X[k1 + 4 k2]; transpose the 4x4 index
  float2 t[16];
#pragma unroll
  for (int s = 0; s < 16; ++s) t[s] = a[s];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = t[4 * (k & 3) + (k >> 2)];
}

template <int R, int DIR> XL_HD void dftR(float2* a) {
  if constexpr (R == 2) dft2<DIR>(a);
  else if constexpr (R == 4) dft4<DIR>(a);
  else if constexpr (R == 8) dft8<DIR>(a);
  else dft16<DIR>(a);
}

XL_HD int smpad(int i) { return i + (i >> 4); }

// FFT of length N = 2^LOGN by a group of T = N/E threads, E elements each.
// Passes: radix E while possible, then one radix 2^(LOGN mod log2 E).
template <int LOGN, int E = 16> struct FftShape {
  static_assert(E == 8 || E == 16, "8 or 16 elements per thread");
  static_assert(LOGN >= 4 && LOGN <= 13, "FFT length 16..8192");
  static constexpr int LE = E == 16 ? 4 : 3;
  static constexpr int N = 1 << LOGN;
  static constexpr int T = N / E;       // threads per FFT
  static constexpr int NFULL = LOGN / LE;
  static constexpr int REM = LOGN % LE;
  static constexpr int NPASS = NFULL + (REM ? 1 : 0);
  static constexpr int SMEM = N + N / 16;  // padded float2 slots per exchange buffer
  template <int P> static constexpr int radix() { return P < NFULL ? E : (1 << REM); }
  static constexpr int radix_rt(int P) { return P < NFULL ? E : (1 << REM); }
  static constexpr int stride_rt(int P) {
    int ns = 1;
    for (int q = 0; q < P; ++q) ns *= (q < NFULL ? E : (1 << REM));
    return ns;
  }
  template <int P> static constexpr int stride() { return stride_rt(P); }
};

// One Stockham pass for thread j.  Input layout v[m] = x[j + m T]; tw is the
// size-N table tw[q] = e^{-2 pi i q / N}.  The last pass leaves its outputs
// in v in natural order (same layout); the others write them to sm.
template <int LOGN, int E, int P, int DIR>
XL_HD void fft_pass(float2 (&v)[E], int j, float2* sm, const float2* tw) {
  using S = FftShape<LOGN, E>;
  constexpr int R = S::template radix<P>();
  constexpr int NS = S::template stride<P>();
  constexpr bool LAST = (P == S::NPASS - 1);
  constexpr int BPT = E / R;
  constexpr int TWS = S::N / (NS * R);
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = j + t * S::T;
    const int k = b & (NS - 1);
    float2 x[R];
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = v[t + i * BPT];
    if constexpr (NS > 1) {
#pragma unroll
      for (int i = 1; i < R; ++i) {
        const float2 w = tw[i * k * TWS];
        x[i] = DIR < 0 ? cmul(x[i], w) : cmulc(x[i], w);
      }
    }
    dftR<R, DIR>(x);
    if constexpr (LAST) {
#pragma unroll
      for (int i = 0; i < R; ++i) v[t + i * BPT] = x[i];
    } else {
      const int base = (b / NS) * (NS * R) + k;
#pragma unroll
      for (int i = 0; i < R; ++i) sm[smpad(base + i * NS)] = x[i];
    }
  }
}

template <int LOGN, int E> XL_HD void fft_gather(float2 (&v)[E], int j, const float2* sm) {
  using S = FftShape<LOGN, E>;
#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = sm[smpad(j + m * S::T)];
}

// ---- per-pass twiddle tables (shared memory) ----
// Pass P >= 1 (radix R, stride NS) keeps e^{-2 pi i (i k) / (NS R)} at
// [off<P>() + (i-1) NS + k], i = 1..R-1, k = 0..NS-1: consecutive threads
// (consecutive k) read consecutive slots, so the reads are conflict-free.
template <int LOGN, int E = 16> struct FftTw {
  using S = FftShape<LOGN, E>;
  template <int P> static constexpr int off() {
    int o = 0;
    for (int q = 1; q < P; ++q) o += (S::radix_rt(q) - 1) * S::stride_rt(q);
    return o;
  }
  static constexpr int SIZE = off<S::NPASS>() > 0 ? off<S::NPASS>() : 1;
};

// One slot of the pass tables from the size-N table twN[q] = e^{-2 pi i q/N}.
template <int LOGN, int E = 16> XL_HD float2 pass_twiddle_entry(int idx, const float2* twN) {
  using S = FftShape<LOGN, E>;
  int base = 0;
  for (int q = 1; q < S::NPASS; ++q) {
    const int R = S::radix_rt(q), NS = S::stride_rt(q);
    const int sz = (R - 1) * NS;
    if (idx < base + sz) {
      const int i = (idx - base) / NS + 1, k = (idx - base) % NS;
      return twN[i * k * (S::N / (NS * R))];
    }
    base += sz;
  }
  return make_float2(1.f, 0.f);
}

// Stockham pass with twiddles from the shared pass tables.
template <int LOGN, int E, int P, int DIR>
XL_HD void fft_pass_s(float2 (&v)[E], int j, float2* sm, const float2* stw) {
  using S = FftShape<LOGN, E>;
  constexpr int R = S::template radix<P>();
  constexpr int NS = S::template stride<P>();
  constexpr bool LAST = (P == S::NPASS - 1);
  constexpr int BPT = E / R;
  constexpr int OFF = FftTw<LOGN, E>::template off<P>();
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = j + t * S::T;
    const int k = b & (NS - 1);
    float2 x[R];
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = v[t + i * BPT];
    if constexpr (NS > 1) {
#pragma unroll
      for (int i = 1; i < R; ++i) {
        const float2 w = stw[OFF + (i - 1) * NS + k];
        x[i] = DIR < 0 ? cmul(x[i], w) : cmulc(x[i], w);
      }
    }
    dftR<R, DIR>(x);
    if constexpr (LAST) {
#pragma unroll
      for (int i = 0; i < R; ++i) v[t + i * BPT] = x[i];
    } else {
      const int base = (b / NS) * (NS * R) + k;
#pragma unroll
      for (int i = 0; i < R; ++i) sm[smpad(base + i * NS)] = x[i];
    }
  }
}

// Twiddle read: the read-only data path for tables in global memory (GTW),
// an ordinary load for tables in shared memory.
template <bool GTW> XL_HD float2 tw_load(const float2* p) {
#if defined(__CUDA_ARCH__)
  if constexpr (GTW) return __ldg(p);
#endif
  return *p;
}

// Stockham pass with twiddles from the pass tables (FftTw layout), either in
// shared memory or in global memory (GTW).  ZU: this is pass 0 of a
// zero-padded line whose upper half is zero, so v[E/2..E-1] are zero on entry
// and are not read (E = 16, radix 16 only).
template <int LOGN, int E, int P, int DIR, bool ZU, bool GTW>
XL_HD void fft_pass_x(float2 (&v)[E], int j, float2* sm, const float2* stw, int toff = 0) {
  using S = FftShape<LOGN, E>;
  constexpr int R = S::template radix<P>();
  constexpr int NS = S::template stride<P>();
  constexpr bool LAST = (P == S::NPASS - 1);
  constexpr int BPT = E / R;
  constexpr int OFF = FftTw<LOGN, E>::template off<P>();
  static_assert(!ZU || (P == 0 && R == 16 && E == 16), "input pruning is for a first radix-16 pass");
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = j + t * S::T;
    const int k = b & (NS - 1);
    float2 x[R];
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = (ZU && i >= R / 2) ? make_float2(0.f, 0.f) : v[t + i * BPT];
    if constexpr (R == 16 && NS > 1) {
      // twiddle the inputs of one inner DFT4 at a time (inputs n2 + 4 q), so
      // only four twiddles are live at once
#pragma unroll
      for (int n2 = 0; n2 < 4; ++n2) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = n2 + 4 * q;
          if (i == 0) continue;
          const float2 w = tw_load<GTW>(stw + toff + OFF + (i - 1) * NS + k);
          x[i] = DIR < 0 ? cmul(x[i], w) : cmulc(x[i], w);
        }
        dft4<DIR>(x[n2], x[n2 + 4], x[n2 + 8], x[n2 + 12]);
      }
      dft16_tail<DIR>(x);
    } else {
      if constexpr (NS > 1) {
#pragma unroll
        for (int i = 1; i < R; ++i) {
          const float2 w = tw_load<GTW>(stw + toff + OFF + (i - 1) * NS + k);
          x[i] = DIR < 0 ? cmul(x[i], w) : cmulc(x[i], w);
        }
      }
      if constexpr (ZU) dft16_half<DIR>(x);
      else dftR<R, DIR>(x);
    }
    if constexpr (LAST) {
#pragma unroll
      for (int i = 0; i < R; ++i) v[t + i * BPT] = x[i];
    } else {
      const int base = (b / NS) * (NS * R) + k;
      if constexpr (NS % 16 == 0 || (NS == 1 && R == 16)) {
        // padded slots at constant offsets from the first: base is a multiple
        // of 16 (NS = 1) or the stride is (NS % 16 = 0)
        constexpr int STEP = NS == 1 ? 1 : NS + NS / 16;
        float2* d = sm + smpad(base);
#pragma unroll
        for (int i = 0; i < R; ++i) d[i * STEP] = x[i];
      } else {
#pragma unroll
        for (int i = 0; i < R; ++i) sm[smpad(base + i * NS)] = x[i];
      }
    }
  }
}

// fft_gather with the padded slots at constant offsets (T a multiple of 16).
template <int LOGN, int E> XL_HD void fft_gather_x(float2 (&v)[E], int j, const float2* sm) {
  using S = FftShape<LOGN, E>;
  if constexpr (S::T % 16 == 0) {
    const float2* s = sm + smpad(j);
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = s[m * (S::T + S::T / 16)];
  } else {
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = sm[smpad(j + m * S::T)];
  }
}

#if defined(__CUDACC__)
// Barrier between the passes of a transform: the whole CTA, or a named
// barrier shared by the `count` threads (a multiple of 32) of one group, so
// that groups of a CTA working on different lines do not wait for each other.
struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupSync {
  int id, count;   // barrier 1..15 (0 is __syncthreads)
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};

// Whole FFT for a thread group, twiddles from pass tables (shared or global),
// optional input pruning (ZU).  Every thread of the CTA must call it the same
// number of times (it uses __syncthreads between passes).
//
// The twiddle offset is laundered through an empty asm statement at the start
// of every transform: a kernel that runs several transforms in a row then
// reloads the (identical) twiddles for each one instead of keeping them all
// live in registers, which would cost about a hundred registers per thread.
template <int LOGN, int E, int DIR, bool ZU, bool GTW, class SYNC = CtaSync, int P = 0>
__device__ __forceinline__ void block_fft_x(float2 (&v)[E], int j, float2* sm, const float2* stw,
                                            const SYNC& sync = SYNC(), int toff = -1) {
  using S = FftShape<LOGN, E>;
  if constexpr (P == 0) {
    toff = 0;
    asm volatile("" : "+r"(toff));
  }
  fft_pass_x<LOGN, E, P, DIR, ZU && P == 0, GTW>(v, j, sm, stw, toff);
  if constexpr (P < S::NPASS - 1) {
    sync();
    fft_gather_x<LOGN, E>(v, j, sm);
    sync();
    block_fft_x<LOGN, E, DIR, false, GTW, SYNC, P + 1>(v, j, sm, stw, sync, toff);
  }
}

// Whole FFT for a thread group.  Every thread of the CTA must call these the
// same number of times (they use __syncthreads between passes).
template <int LOGN, int E, int DIR, int P = 0>
__device__ __forceinline__ void block_fft_s(float2 (&v)[E], int j, float2* sm, const float2* stw) {
  using S = FftShape<LOGN, E>;
  fft_pass_s<LOGN, E, P, DIR>(v, j, sm, stw);
  if constexpr (P < S::NPASS - 1) {
    __syncthreads();
    fft_gather<LOGN, E>(v, j, sm);
    __syncthreads();
    block_fft_s<LOGN, E, DIR, P + 1>(v, j, sm, stw);
  }
}

template <int LOGN, int E, int DIR, int P = 0>
__device__ __forceinline__ void block_fft(float2 (&v)[E], int j, float2* sm, const float2* tw) {
  using S = FftShape<LOGN, E>;
  fft_pass<LOGN, E, P, DIR>(v, j, sm, tw);
  if constexpr (P < S::NPASS - 1) {
    __syncthreads();
    fft_gather<LOGN, E>(v, j, sm);
    __syncthreads();
    block_fft<LOGN, E, DIR, P + 1>(v, j, sm, tw);
  }
}
#endif

}  // namespace xl
