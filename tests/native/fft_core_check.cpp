// CPU harness for the device FFT engine: runs the T threads of one FFT group
// in sequence, pass by pass, with the same shared-memory exchange the kernels
// use.  Built by tests/test_fft_core_cpu.py with g++ and called through ctypes.
#include <cmath>
#include <vector>
#include "../../xlumina_gb300/csrc/fft_core.cuh"
#include "../../xlumina_gb300/csrc/fft_pair.cuh"
#include "../../xlumina_gb300/csrc/fft64.cuh"

using namespace xl;

template <int E> struct Regs { float2 v[E]; };

template <int LOGN, int E, int DIR, int P>
static void emu(std::vector<Regs<E>>& V, float2* sm, const float2* tw) {
  using S = FftShape<LOGN, E>;
  for (int j = 0; j < S::T; ++j) fft_pass<LOGN, E, P, DIR>(V[j].v, j, sm, tw);
  if constexpr (P < S::NPASS - 1) {
    for (int j = 0; j < S::T; ++j) fft_gather<LOGN, E>(V[j].v, j, sm);
    emu<LOGN, E, DIR, P + 1>(V, sm, tw);
  }
}

template <int LOGN, int E, int DIR, int P>
static void emu_s(std::vector<Regs<E>>& V, float2* sm, const float2* stw) {
  using S = FftShape<LOGN, E>;
  for (int j = 0; j < S::T; ++j) fft_pass_s<LOGN, E, P, DIR>(V[j].v, j, sm, stw);
  if constexpr (P < S::NPASS - 1) {
    for (int j = 0; j < S::T; ++j) fft_gather<LOGN, E>(V[j].v, j, sm);
    emu_s<LOGN, E, DIR, P + 1>(V, sm, stw);
  }
}

// The pass sequence the zero-padded propagators run: pass tables, the first
// pass pruned for a zero upper half of the input.
template <int LOGN, int E, int DIR, int P>
static void emu_x(std::vector<Regs<E>>& V, float2* sm, const float2* stw) {
  using S = FftShape<LOGN, E>;
  for (int j = 0; j < S::T; ++j) fft_pass_x<LOGN, E, P, DIR, P == 0, false>(V[j].v, j, sm, stw);
  if constexpr (P < S::NPASS - 1) {
    for (int j = 0; j < S::T; ++j) fft_gather_x<LOGN, E>(V[j].v, j, sm);
    emu_x<LOGN, E, DIR, P + 1>(V, sm, stw);
  }
}

static int g_use_stw = 0;

static int g_e = 16;

template <int LOGN, int E, int DIR>
static void run_e(const float* in, float* out) {
  using S = FftShape<LOGN, E>;
  std::vector<float2> tw(S::N), sm(S::SMEM);
  for (int q = 0; q < S::N; ++q) {
    double a = 2.0 * M_PI * q / S::N;
    tw[q] = make_float2((float)std::cos(a), (float)-std::sin(a));
  }
  std::vector<Regs<E>> V(S::T);
  for (int j = 0; j < S::T; ++j)
    for (int m = 0; m < E; ++m) {
      int n = j + m * S::T;
      V[j].v[m] = make_float2(in[2 * n], in[2 * n + 1]);
    }
  if (g_use_stw == 2) {
    if constexpr (E == 16) {
      std::vector<float2> stw(FftTw<LOGN, E>::SIZE);
      for (int i = 0; i < FftTw<LOGN, E>::SIZE; ++i) stw[i] = pass_twiddle_entry<LOGN, E>(i, tw.data());
      emu_x<LOGN, E, DIR, 0>(V, sm.data(), stw.data());
    }
  } else if (g_use_stw) {
    std::vector<float2> stw(FftTw<LOGN, E>::SIZE);
    for (int i = 0; i < FftTw<LOGN, E>::SIZE; ++i) stw[i] = pass_twiddle_entry<LOGN, E>(i, tw.data());
    emu_s<LOGN, E, DIR, 0>(V, sm.data(), stw.data());
  } else {
    emu<LOGN, E, DIR, 0>(V, sm.data(), tw.data());
  }
  for (int j = 0; j < S::T; ++j)
    for (int m = 0; m < E; ++m) {
      int n = j + m * S::T;
      out[2 * n] = V[j].v[m].x;
      out[2 * n + 1] = V[j].v[m].y;
    }
}

template <int LOGN, int DIR>
static void run(const float* in, float* out) {
  if (g_e == 8) run_e<LOGN, 8, DIR>(in, out);
  else run_e<LOGN, 16, DIR>(in, out);
}

template <int DIR>
static int dispatch(int logn, const float* in, float* out) {
  switch (logn) {
    case 4: run<4, DIR>(in, out); return 0;
    case 5: run<5, DIR>(in, out); return 0;
    case 6: run<6, DIR>(in, out); return 0;
    case 7: run<7, DIR>(in, out); return 0;
    case 8: run<8, DIR>(in, out); return 0;
    case 9: run<9, DIR>(in, out); return 0;
    case 10: run<10, DIR>(in, out); return 0;
    case 11: run<11, DIR>(in, out); return 0;
    case 12: run<12, DIR>(in, out); return 0;
    case 13: run<13, DIR>(in, out); return 0;
  }
  return -1;
}

extern "C" void fft_core_set_e(int e) { g_e = e; }

extern "C" int fft_core_check_stw(int logn, int dir, const float* in, float* out) {
  g_use_stw = 1;
  int rc = dir < 0 ? dispatch<-1>(logn, in, out) : dispatch<1>(logn, in, out);
  g_use_stw = 0;
  return rc;
}

// FFT of a line whose upper half is zero (in[N/2..N-1] are ignored), with the
// first pass pruned; 16 elements per thread.
extern "C" int fft_core_check_zu(int logn, int dir, const float* in, float* out) {
  g_use_stw = 2;
  const int saved = g_e;
  g_e = 16;
  int rc = (logn < 5) ? -1 : (dir < 0 ? dispatch<-1>(logn, in, out) : dispatch<1>(logn, in, out));
  g_e = saved;
  g_use_stw = 0;
  return rc;
}

extern "C" int fft_core_check(int logn, int dir, const float* in, float* out) {
  return dir < 0 ? dispatch<-1>(logn, in, out) : dispatch<1>(logn, in, out);
}

// ---- the two-line (packed) engine of fft_pair.cuh: two lines a, b at once ----
struct PRegs { cpair v[16]; };

template <int LOGN, int DIR, bool ZU, int P>
static void emu_p(std::vector<PRegs>& V, f4* sm, const f4* stw) {
  using S = FftShape<LOGN, 16>;
  for (int j = 0; j < S::T; ++j) pfft_pass<LOGN, P, DIR, ZU && P == 0, false>(V[j].v, j, sm, stw, 0);
  if constexpr (P < S::NPASS - 1) {
    for (int j = 0; j < S::T; ++j) pfft_gather<LOGN>(V[j].v, j, sm);
    emu_p<LOGN, DIR, false, P + 1>(V, sm, stw);
  }
}

template <int LOGN, int DIR>
static void run_p(const float* a, const float* b, float* oa, float* ob, int zu) {
  using S = FftShape<LOGN, 16>;
  std::vector<float2> tw(S::N);
  for (int q = 0; q < S::N; ++q) {
    double ang = 2.0 * M_PI * q / S::N;
    tw[q] = make_float2((float)std::cos(ang), (float)-std::sin(ang));
  }
  std::vector<f4> stw(FftTw<LOGN, 16>::SIZE), sm(S::SMEM);
  for (int i = 0; i < FftTw<LOGN, 16>::SIZE; ++i) stw[i] = pair_tw(pass_twiddle_entry<LOGN, 16>(i, tw.data()));
  std::vector<PRegs> V(S::T);
  for (int j = 0; j < S::T; ++j)
    for (int m = 0; m < 16; ++m) {
      const int n = j + m * S::T;
      V[j].v[m] = p_from2(make_float2(a[2 * n], a[2 * n + 1]), make_float2(b[2 * n], b[2 * n + 1]));
    }
  if (zu) emu_p<LOGN, DIR, true, 0>(V, sm.data(), stw.data());
  else emu_p<LOGN, DIR, false, 0>(V, sm.data(), stw.data());
  for (int j = 0; j < S::T; ++j)
    for (int m = 0; m < 16; ++m) {
      const int n = j + m * S::T;
      const float2 x = p_lo(V[j].v[m]), y = p_hi(V[j].v[m]);
      oa[2 * n] = x.x; oa[2 * n + 1] = x.y;
      ob[2 * n] = y.x; ob[2 * n + 1] = y.y;
    }
}

template <int DIR>
static int dispatch_p(int logn, const float* a, const float* b, float* oa, float* ob, int zu) {
  switch (logn) {
    case 5: run_p<5, DIR>(a, b, oa, ob, zu); return 0;
    case 6: run_p<6, DIR>(a, b, oa, ob, zu); return 0;
    case 7: run_p<7, DIR>(a, b, oa, ob, zu); return 0;
    case 8: run_p<8, DIR>(a, b, oa, ob, zu); return 0;
    case 9: run_p<9, DIR>(a, b, oa, ob, zu); return 0;
    case 10: run_p<10, DIR>(a, b, oa, ob, zu); return 0;
    case 11: run_p<11, DIR>(a, b, oa, ob, zu); return 0;
    case 12: run_p<12, DIR>(a, b, oa, ob, zu); return 0;
    case 13: run_p<13, DIR>(a, b, oa, ob, zu); return 0;
  }
  return -1;
}

// Two lines through the packed engine; zu: their upper halves are zero and not read.
extern "C" int fft_pair_check(int logn, int dir, int zu, const float* a, const float* b, float* oa, float* ob) {
  return dir < 0 ? dispatch_p<-1>(logn, a, b, oa, ob, zu) : dispatch_p<1>(logn, a, b, oa, ob, zu);
}

// ---- the radix-64 4096-point engine of fft64.cuh: 64 threads of 64 elements ----
struct R64 { float2 v[64]; };

// One 4096-point transform (zin: the upper half of the input is zero and not
// read; zout: only outputs 0..2047 are produced, the rest of out is untouched).
template <int DIR, bool ZIN, bool ZOUT>
static void run_64(const float* in, float* out) {
  std::vector<float2> tw(4096), stw(4096), xb(F64_XS);
  for (int q = 0; q < 4096; ++q) {
    const double ang = 2.0 * M_PI * q / 4096;
    tw[q] = make_float2((float)std::cos(ang), (float)-std::sin(ang));
  }
  for (int i = 0; i < 4096; ++i) stw[i] = f64_twiddle_entry(i, tw.data());
  std::vector<R64> V(64);
  for (int j = 0; j < 64; ++j)
    for (int m = 0; m < (ZIN ? 32 : 64); ++m) {
      const int n = j + 64 * m;
      V[j].v[m] = make_float2(in[2 * n], in[2 * n + 1]);
    }
  for (int j = 0; j < 64; ++j) {
    f64_pass0<DIR, ZIN>(V[j].v);
    f64_write<DIR>(V[j].v, j, xb.data(), stw.data());
  }
  for (int j = 0; j < 64; ++j) f64_pass1<DIR, ZOUT>(V[j].v, j, xb.data());
  for (int j = 0; j < 64; ++j)
    for (int m = 0; m < (ZOUT ? 32 : 64); ++m) {
      const int n = j + 64 * m;
      out[2 * n] = V[j].v[m].x;
      out[2 * n + 1] = V[j].v[m].y;
    }
}

template <int DIR>
static void run_64d(int zin, int zout, const float* in, float* out) {
  if (zin && zout) run_64<DIR, true, true>(in, out);
  else if (zin) run_64<DIR, true, false>(in, out);
  else if (zout) run_64<DIR, false, true>(in, out);
  else run_64<DIR, false, false>(in, out);
}

extern "C" int fft64_check(int dir, int zin, int zout, const float* in, float* out) {
  if (dir < 0) run_64d<-1>(zin, zout, in, out);
  else run_64d<1>(zin, zout, in, out);
  return 0;
}

// Exchange slots of the radix-64 engine for four interleaved lines (lane =
// 4 (j % 8) + line): for each half-warp access of the pass-0 writes and the
// pass-1 gathers, the number of distinct 8-byte bank pairs (16 when free of
// conflicts); returns the minimum over all accesses.
extern "C" int fft64_min_banks() {
  int worst = 16;
  for (int j0 = 0; j0 < 64; j0 += 8)
    for (int half = 0; half < 2; ++half)
      for (int i = 0; i < 64; ++i)
        for (int phase = 0; phase < 2; ++phase) {
          bool seen[16] = {false};
          int distinct = 0;
          for (int l = 0; l < 16; ++l) {
            const int line = l & 3, j = j0 + half * 4 + (l >> 2);
            const int slot = line * F64_XB + (phase == 0 ? F64_ROW * j + i : F64_ROW * i + j);
            if (!seen[slot & 15]) { seen[slot & 15] = true; ++distinct; }
          }
          if (distinct < worst) worst = distinct;
        }
  return worst;
}
