// Chirp-z (Bluestein) propagation for sm_103a: scalar CZT, vectorial VCZT and
// the high-NA objective-lens focus, forward and adjoint; the kernels and their
// launch code, included by the czt_l*.cu translation units.
//
// The reference (wave_optics.py:333-460) runs Bluestein's algorithm along y
// and then along x, each as: multiply the input line by a pre-chirp,
// zero-pad to L = next_pow2(m+M-1), FFT, multiply by the spectrum of the
// inverse chirp, inverse FFT, keep entries [m, m+M) and multiply by a
// post-chirp.  The 2-D transform is separable, so here the x transform runs
// first over rows (czt_rows) and the y transform second over column tiles
// (czt_cols).  A line is one L-point FFT pair by L/16 threads holding 16
// elements each; when the input window lies in the first half of the line
// (the forward transform: positions 0 .. m-1 <= L/2) the first pass is
// pruned.
//
// czt_rows is persistent: each CTA stages its next rows (field planes and
// per-pixel parameter planes) into shared memory with TMA bulk copies; the
// prologue applies the Jones program (masks, high-NA lens), the VCZT
// Ez = (Ex X/r + Ey Y/r) z/r and the input-plane transfer function F, and
// writes the components to a shared buffer; then one thread group per
// component transforms them.  czt_cols applies the output-plane transfer
// function F0, the constant factor (z dx dy lambda, or -i sin^2(theta_max) /
// (f lambda)) and, for the VCZT adjoint, the fold of the Ez gradient into
// Ex, Ey.  The intermediate (after the x transform) is stored in column tiles
// of 2^lw: element (row r, column l) at ((l >> lw) ny + r) 2^lw + (l mod 2^lw),
// planes of ny x mxp (mx rounded up to the tile width).
#pragma once

#include <math.h>

#include <type_traits>

#include "czt_host.h"
#include "line_fft.cuh"

namespace xl {

template <int LOGL> struct CztCfg {
  static constexpr int L = 1 << LOGL;
  static constexpr int E = 16;
  static constexpr int H = E / 2;
  static constexpr int T = L / E;                              // threads per line
  static constexpr int XS = L + L / 16;                        // exchange slots per line
  static constexpr int G = (256 / T) > 1 ? (256 / T) : 1;      // rows per group in the x transform
  // y transform: W columns per CTA (one tile), interleaved in the lanes of every warp
  static constexpr int W = LOGL >= 13 ? 2 : ((32 / T) > 4 ? (32 / T) : 4);
  static constexpr int CXS = XS + (W >= 8 ? 0 : 16 / W);
  static constexpr int COL_THREADS = W * T;
  static constexpr int COL_MINB = (1024 / COL_THREADS) > 1 ? (1024 / COL_THREADS) : 1;
  static constexpr int NTW = FftTw<LOGL, E>::SIZE;
  static_assert(COL_THREADS >= 32 && COL_THREADS <= 1024, "column CTA shape");
};

// x transform organisation for NC line components: CG component groups of G
// rows of T threads; CG = NC (every component of a row at once) when the CTA
// can hold them, else 1.
template <int LOGL, int NC, bool OG = false> struct CztRowCfg {
  using C = CztCfg<LOGL>;
  // OG: one component group whatever NC (the components one after the other)
  static constexpr int CG = (!OG && NC * C::G * C::T <= 1024) ? NC : 1;
  static constexpr int ITER = (NC + CG - 1) / CG;              // transforms per group and row
  static constexpr int LINES = CG * C::G;
  static constexpr int THREADS = LINES * C::T;
  static constexpr int MINB = (768 / THREADS) > 1 ? (768 / THREADS) : 1;
};

__device__ __forceinline__ long long tiled_rt(int r, int col, int rows, int lw) {
  return ((((long long)(col >> lw)) * rows + r) << lw) + (col & ((1 << lw) - 1));
}

// x transform.  NC: components per row (1, or 3 for VCZT and the high-NA
// focus; a plain transform of 2 components runs as 3 with the third idle).
// ZU: the input window lies in the first half of the line.  MB: resident
// CTAs per SM the registers are sized for (0: CztRowCfg's MINB).  FK: the
// fused program's op kinds fixed at compile time (FixedKinds<...>, for the
// tables' programs), or FixedKinds<>.
template <int LOGL, int NC, bool ZU, int MB = 0, class FK = FixedKinds<>, bool OG = false>
__global__ void __launch_bounds__(CztRowCfg<LOGL, NC, OG>::THREADS, MB ? MB : CztRowCfg<LOGL, NC, OG>::MINB)
    czt_rows(const __grid_constant__ CztLaunch p, const __grid_constant__ RowStage st) {
  using C = CztCfg<LOGL>;
  using F = CztRowCfg<LOGL, NC, OG>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = p.nx, ny = p.ny;
  float2* xch = (float2*)smraw;                                    // LINES x XS
  float2* post = xch + F::LINES * C::XS;                           // NC x G x nx
  const size_t soff = ((size_t)(F::LINES * C::XS + NC * C::G * nx) * 8 + 15) / 16 * 16;
  unsigned char* stage = smraw + soff;
  unsigned long long* mbar = (unsigned long long*)(stage + (size_t)C::G * st.row_bytes);
  const int tid = threadIdx.x;
  const int line = tid / C::T, j = tid % C::T;
  const int cg = line / C::G, gi = line % C::G;
  const int ngb = (ny + C::G - 1) / C::G;
  const int total = p.B * ngb;
  const bool staged = st.n > 0;
  const bool fwd_phase = p.mode != XL_CZT_PLAIN;
  const bool vczt = p.mode == XL_CZT_VECTOR && !p.adjoint;
  constexpr int L = C::L;

  if (tid == 0 && staged) {
    mbar_init(mbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  // row groups are taken batch entries fastest: CTAs that run together read the
  // same rows of planes shared by the batch (the lens coefficients, shared
  // masks), so those rows come from L2 after the first entry
  if (tid == 0 && blockIdx.x < total) {
    const int b = blockIdx.x % p.B, r0 = (blockIdx.x / p.B) * C::G;
    if (staged) stage_rows(st, stage, mbar, b, r0, min(C::G, ny - r0));
    prefetch_rows(st, b, r0, min(C::G, ny - r0));
  }

  unsigned phase = 0;
  for (int grp = blockIdx.x; grp < total; grp += gridDim.x) {
    const int b = grp % p.B;
    const int r0 = (grp / p.B) * C::G;
    const double zd = p.zb ? p.zb[b] : p.z;
    const float zf = (float)zd;
    // a wait that runs out is acted on at the barrier after the prologue
    // (the prologue then works on stale data, and the launch's output is not
    // valid), so that no extra barrier is taken per row group
    const bool got = !staged || mbar_wait_bounded(mbar, phase, g_wait_limit_ns);
    // prologue over the row group's pixels; in CTAs of up to 256 threads, four
    // per thread at a time while four remain, then one: each op of the program
    // is dispatched once for the four, and their loads and arithmetic overlap
    const int lim = min(C::G, ny - r0) * nx;
    auto chunk = [&](auto npx, int base) {
      constexpr int NPX = decltype(npx)::value;
      float2 e[NPX][3];
      PixelCtx px[NPX];
      StagedParams pr[NPX];
#pragma unroll
      for (int q = 0; q < NPX; ++q) {
        const int idx = base + q * F::THREADS;
        const int g2 = C::G == 1 ? 0 : idx / nx, n = idx - g2 * nx, r = r0 + g2;
        const long long pix = (long long)r * nx + n;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          e[q][c] = make_float2(0.f, 0.f);
          if (c < p.cin) {
            const int fo = st.fld[c];
            e[q][c] = fo >= 0 ? ((const float2*)(stage + fo))[g2 * nx + n] : p.in[c][(long long)b * p.ibs + pix];
          }
        }
        px[q] = PixelCtx{r, n, pix, b};
        pr[q] = StagedParams{stage, &st, g2, nx, n};
      }
      if constexpr (FK::n > 0) apply_prog_fixed<FK>(p.pre, e, px, pr);
      else if (p.pre.nops) apply_prog_vec<NPX>(p.pre, e, px, pr);
#pragma unroll
      for (int q = 0; q < NPX; ++q) {
        const int r = px[q].row, n = px[q].col;
        if (fwd_phase) {
          if (vczt) {  // vectorized_optics.py:340-344
            const float X = (float)p.x[n], Y = (float)p.y[r];
            const float rr = sqrtf(X * X + Y * Y + zf * zf);
            e[q][2] = cscale(cadd(cscale(e[q][0], X / rr), cscale(e[q][1], Y / rr)), zf / rr);
          }
          // wave_optics.py:341 (F on the input plane); the adjoint applies conj(F0) here
          float2 Fv = p.fin ? p.fin[px[q].pix] : rs_kernel_value(p.x[n], p.y[r], zd, p.inv_lambda, p.k);
          if (p.adjoint) Fv = cconj(Fv);
#pragma unroll
          for (int c = 0; c < 3; ++c) e[q][c] = cmul(e[q][c], Fv);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) post[(c * C::G + (r - r0)) * nx + n] = e[q][c];
      }
    };
    {
      int base = tid;
      // a fixed program with registers for two CTAs per SM (128): eight at a
      // time first (1932 against 1911 tables/s on the high-NA step)
      if constexpr (F::THREADS <= 256 && FK::n > 0 && MB == 2) {
        for (; base + 7 * F::THREADS < lim; base += 8 * F::THREADS) chunk(std::integral_constant<int, 8>{}, base);
      }
      if constexpr (F::THREADS <= 256) {   // CTAs of 768 threads ran slower with it
        for (; base + 3 * F::THREADS < lim; base += 4 * F::THREADS) chunk(std::integral_constant<int, 4>{}, base);
      }
      for (; base < lim; base += F::THREADS) chunk(std::integral_constant<int, 1>{}, base);
    }
    // every thread has read the stage and written its pixels; every thread
    // takes the timeout branch or none does
    if (__syncthreads_or(!got)) {
      // the copy may still be in flight: let it land, record the event and
      // leave without issuing another
      mbar_wait_bounded(mbar, phase);
      if (tid == 0) record_timeout();
      return;
    }
    phase ^= 1u;
    if (tid == 0 && grp + gridDim.x < total) {
      const int g = grp + gridDim.x, bn = g % p.B, rn = (g / p.B) * C::G;
      if (staged) {
        fence_proxy_async();
        stage_rows(st, stage, mbar, bn, rn, min(C::G, ny - rn));
      }
      prefetch_rows(st, bn, rn, min(C::G, ny - rn));
    }
    const int r = r0 + gi;
    const bool live = r < ny;
#pragma unroll 1
    for (int it = 0; it < F::ITER; ++it) {
      const int c = cg + it * F::CG;
      const bool act = live && c < p.cout;
      float2 v[16];
      const float2* src = post + (c < NC ? c * C::G + gi : 0) * nx;
      const float2* pre_x = czt_entry(p.pre_x, p, b, nx);
      constexpr int MN = ZU ? C::H : 16;
#pragma unroll
      for (int m = 0; m < MN; ++m) {
        const int i = j + m * C::T - p.ioff_x;
        v[m] = (act && i >= 0 && i < nx) ? cmul(src[i], __ldg(pre_x + i)) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int m = MN; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
      block_fft_x<LOGL, 16, -1, ZU, true>(v, j, xch + line * C::XS, pass_tw<LOGL>());
      {
        const float2* g = czt_entry(p.g_x, p, b, L);
        asm volatile("" : "+l"(g) : : "memory");
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], __ldg(g + j + m * C::T));
      }
      block_fft_x<LOGL, 16, 1, false, true>(v, j, xch + line * C::XS, pass_tw<LOGL>());
      if (act) {
        float2* plane = p.work + ((long long)b * p.cout + c) * ny * p.mxp;
        const float2* post_x = czt_entry(p.post_x, p, b, p.mx);
#pragma unroll
        for (int m = 0; m < 16; ++m) {
          const int o = j + m * C::T - p.ooff_x;
          if (o >= 0 && o < p.mx) plane[tiled_rt(r, o, ny, p.lw)] = cmul(v[m], __ldg(post_x + o));
        }
      }
    }
  }
}

// y transform over tiles of W columns, with the epilogue.  Lanes interleave
// the W columns of a tile, so every warp load of the intermediate is one
// contiguous run.
// PERSIST: one CTA per resident slot walks the (column tile, batch entry)
// units in the grid's order; the pass twiddle table is loaded once per CTA
// instead of once per tile.
template <int LOGL, bool ZU, bool PERSIST = false>
__global__ void __launch_bounds__(CztCfg<LOGL>::COL_THREADS, CztCfg<LOGL>::COL_MINB)
    czt_cols(const __grid_constant__ CztLaunch p) {
  using C = CztCfg<LOGL>;
  constexpr int W = C::W, LPW = 32 / W;
  extern __shared__ __align__(16) float2 smem[];
  float2* xch = smem;                  // W x CXS
  float2* stw = smem + W * C::CXS;     // NTW
  const int tid = threadIdx.x, lane = tid & 31;
  const int w = lane % W, j = (tid >> 5) * LPW + lane / W;
  {
    const float2* g = pass_tw<LOGL>();
    for (int i = tid; i < C::NTW; i += blockDim.x) stw[i] = g[i];
  }
  __syncthreads();
  float2* xb = xch + w * C::CXS;
  const bool fold = p.adjoint && p.mode == XL_CZT_VECTOR;
  const int ny = p.ny;
  const int ntiles = (p.mx + W - 1) / W;
  const int units = PERSIST ? ntiles * p.B : 1;
#pragma unroll 1
  for (int u = PERSIST ? (int)blockIdx.x : 0; u < units; u += PERSIST ? (int)gridDim.x : 1) {
    const int t = PERSIST ? u % ntiles : (int)blockIdx.x;
    const int b = PERSIST ? u / ntiles : (int)blockIdx.y;
    const int col = t * W + w;
    const bool live = col < p.mx;
    const double zd = p.zb ? p.zb[b] : p.z;
    const float zf = (float)zd;
    const float2* pre_y = czt_entry(p.pre_y, p, b, ny);
    const float2* g_y = czt_entry(p.g_y, p, b, C::L);
    const float2* post_y = czt_entry(p.post_y, p, b, p.my);
    float2 cte = p.cte;
    if (p.cteb) {
      cte = p.cteb[b];
      if (p.adjoint) cte.y = -cte.y;
    }
#pragma unroll 1
    for (int c = 0; c < p.cout; ++c) {
      const float2* tileT = p.work + ((long long)b * p.cout + c) * ny * p.mxp + (long long)t * ny * W + w;
      float2 v[16];
      constexpr int MN = ZU ? C::H : 16;
#pragma unroll
      for (int m = 0; m < MN; ++m) {
        const int n = j + m * C::T - p.ioff_y;
        v[m] = (live && n >= 0 && n < ny) ? cmul(tileT[(long long)n * W], __ldg(pre_y + n)) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int m = MN; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
      block_fft_x<LOGL, 16, -1, ZU, false>(v, j, xb, stw);
      {
        const float2* g = g_y;
        asm volatile("" : "+l"(g));
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], __ldg(g + j + m * C::T));
      }
      block_fft_x<LOGL, 16, 1, false, false>(v, j, xb, stw);
      if (!live) continue;
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int o = j + m * C::T - p.ooff_y;
        if (o < 0 || o >= p.my) continue;
        float2 val = cmul(v[m], __ldg(post_y + o));
        if (p.mode != XL_CZT_PLAIN) {  // wave_optics.py:340, 355: F0 * U (adjoint: conj F)
          const float2 Fv = p.fout ? p.fout[(long long)o * p.mx + col]
                                   : rs_kernel_value(p.xo[col], p.yo[o], zd, p.inv_lambda, p.k);
          val = p.adjoint ? cmulc(val, Fv) : cmul(val, Fv);
        }
        val = cmul(val, cte);
        const long long pix = (long long)b * p.obs + (long long)o * p.mx + col;
        if (fold && c == 2) {  // adjoint of Ez = (Ex X/r + Ey Y/r) z/r, vectorized_optics.py:341-344
          const float X = (float)p.xo[col], Y = (float)p.yo[o];
          const float r2 = X * X + Y * Y + zf * zf;
          p.out[0][pix] = cadd(p.out[0][pix], cscale(val, X * zf / r2));
          p.out[1][pix] = cadd(p.out[1][pix], cscale(val, Y * zf / r2));
        } else {
          p.out[c][pix] = val;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Launch code.

template <int LOGL, int NC, bool ZU, int MB = 0, class FK = FixedKinds<>, bool OG = false>
static int launch_czt_rows(cudaStream_t s, const CztLaunch& p) {
  using C = CztCfg<LOGL>;
  using F = CztRowCfg<LOGL, NC, OG>;
  const size_t fixed = ((size_t)(F::LINES * C::XS + NC * C::G * p.nx) * 8 + 15) / 16 * 16;
  // kernel variant: 0 cap the stage so that two CTAs fit per SM where the
  // registers allow two (the one-component transforms; three components keep
  // one CTA per SM and stage every plane that fits); 1 stage every plane
  // that fits one CTA per SM; 2 stage nothing (all planes read from global
  // memory, as many CTAs as the registers allow); 3 as 0 with the registers
  // sized for two CTAs per SM instead of three (MB = 2: no spills).
  // Measured on the Ez-only high-NA step (32 x 2048^2): 1354 (0), 1138 (1),
  // 1348 (2) tables/s.
  // 4 (three components, 4096 points): one component group transforming
  // the components one after the other, two CTAs per SM as in 3.
  int var = kernel_variant(XL_PASS_CZT_ROWS, LOGL);
  if (var == 4 && NC == 1) var = 3;   // a single component is one group already
  if constexpr (NC == 3 && LOGL == 12 && !OG) {
    if (var == 4) return launch_czt_rows<LOGL, NC, ZU, 2, FK, true>(s, p);
  }
  constexpr int MB2 = 512 / F::THREADS;   // two CTAs of 256 threads
  if constexpr (NC == 1 && MB == 0 && MB2 >= 1 && MB2 < F::MINB) {
    if (var == 3) return launch_czt_rows<LOGL, NC, ZU, MB2, FK>(s, p);
  }
  const size_t one_cta = (size_t)226 * 1024, two_cta = (size_t)(227 * 1024) / 2 - 1024;
  const size_t cap = (var == 0 || var == 3 || var == 4) ? ((NC == 1 || OG) ? two_cta : one_cta)
                     : var == 1 ? one_cta : 0;
  RowStage st;
  plan_row_stage(p.cin, p.in, p.ibs, p.nx, p.pre, C::G, fixed, st, cap);
  const size_t sm = fixed + (size_t)C::G * st.row_bytes + 16;
  if (sm > 227 * 1024) {
    set_error("czt: input row of %d columns too long for shared memory", p.nx);
    return XL_EUNSUPPORTED;
  }
  cudaError_t e = allow_smem(czt_rows<LOGL, NC, ZU, MB, FK, OG>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "czt_rows smem");
  const int total = p.B * ((p.ny + C::G - 1) / C::G);
  const int grid = persistent_grid(czt_rows<LOGL, NC, ZU, MB, FK, OG>, F::THREADS, sm, total);
  czt_rows<LOGL, NC, ZU, MB, FK, OG><<<grid, F::THREADS, sm, s>>>(p, st);
  XL_CHECK_LAUNCH("czt_rows");
  return XL_OK;
}

template <int LOGL>
int czt_rows_launch(cudaStream_t s, const CztLaunch& p) {
  const bool zu = p.ioff_x >= 0 && p.ioff_x + p.nx <= (1 << LOGL) / 2;
  // the tables' forward programs get a kernel with their op kinds fixed: the
  // high-NA table's LCD, sSLM and lens Ez row (4096-point lines), the 4f
  // table's thin lens (2048-point lines) and second phase SLM (1024-point)
  if constexpr (LOGL == 12) {
    using HighNaEz = FixedKinds<XL_OP_LCD, XL_OP_SSLM, XL_OP_HIGHNA_EZ>;
    if (p.cout == 1 && zu && HighNaEz::matches(p.pre)) return launch_czt_rows<LOGL, 1, true, 0, HighNaEz>(s, p);
  }
  if constexpr (LOGL == 11) {
    using LensOnly = FixedKinds<XL_OP_SEPMASK>;
    if (p.cout == 1 && zu && LensOnly::matches(p.pre)) return launch_czt_rows<LOGL, 1, true, 0, LensOnly>(s, p);
  }
  if constexpr (LOGL == 10) {
    using SlmOnly = FixedKinds<XL_OP_PHASE>;
    if (p.cout == 1 && zu && SlmOnly::matches(p.pre)) return launch_czt_rows<LOGL, 1, true, 0, SlmOnly>(s, p);
  }
  if (p.cout == 1) return zu ? launch_czt_rows<LOGL, 1, true>(s, p) : launch_czt_rows<LOGL, 1, false>(s, p);
  // (a fixed LCD-sSLM-lens program in the three-component kernel ran slower:
  // 1.96 against 1.90 ms per 8 x 2048^2 high-NA focuses)
  return zu ? launch_czt_rows<LOGL, 3, true>(s, p) : launch_czt_rows<LOGL, 3, false>(s, p);
}

template <int LOGL, bool ZU>
static int launch_czt_cols(cudaStream_t s, const CztLaunch& p) {
  using C = CztCfg<LOGL>;
  const size_t sm = (size_t)(C::W * C::CXS + C::NTW) * sizeof(float2);
  // kernel variant: 0 one CTA per column tile and entry; 1 persistent
  if (kernel_variant(XL_PASS_CZT_COLS, LOGL) == 1) {
    cudaError_t e = allow_smem(czt_cols<LOGL, ZU, true>, sm);
    if (e != cudaSuccess) return cuda_fail(e, "czt_cols smem");
    const int grid = persistent_grid(czt_cols<LOGL, ZU, true>, C::COL_THREADS, sm,
                                     ((p.mx + C::W - 1) / C::W) * p.B);
    czt_cols<LOGL, ZU, true><<<grid, C::COL_THREADS, sm, s>>>(p);
  } else {
    cudaError_t e = allow_smem(czt_cols<LOGL, ZU>, sm);
    if (e != cudaSuccess) return cuda_fail(e, "czt_cols smem");
    czt_cols<LOGL, ZU><<<dim3((p.mx + C::W - 1) / C::W, p.B), C::COL_THREADS, sm, s>>>(p);
  }
  XL_CHECK_LAUNCH("czt_cols");
  return XL_OK;
}

template <int LOGL>
int czt_cols_launch(cudaStream_t s, const CztLaunch& p) {
  if ((1 << p.lw) != CztCfg<LOGL>::W) {
    set_error("czt: intermediate tile width does not match the y transform");
    return XL_EINVAL;
  }
  const bool zu = p.ioff_y >= 0 && p.ioff_y + p.ny <= (1 << LOGL) / 2;
  return zu ? launch_czt_cols<LOGL, true>(s, p) : launch_czt_cols<LOGL, false>(s, p);
}

}  // namespace xl

#define XL_CZT_INSTANTIATE(L)                                                 \
  template int xl::czt_rows_launch<L>(cudaStream_t, const xl::CztLaunch&);    \
  template int xl::czt_cols_launch<L>(cudaStream_t, const xl::CztLaunch&);
