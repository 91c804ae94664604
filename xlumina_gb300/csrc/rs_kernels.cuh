// Rayleigh-Sommerfeld propagation (scalar RS and vectorial VRS) for sm_103a:
// the kernels and their launch code, included by the rs_q*.cu translation units.
//
// The reference (wave_optics.py:281-289) zero-pads the N x N field to
// (2N-1)^2, multiplies fft2(U) by fft2(H) and crops [N-1:, N-1:].  Here the
// same linear convolution runs on a P x P grid, P = 2Q and Q the next power
// of two >= N, which gives the identical result because the impulse response
// is placed at wrapped offsets.  Three passes:
//
//   row pass (rs_rows_fwd): for each of the N input rows, the P-point
//       spectrum of the zero-padded row (the first FFT pass is pruned: half
//       its inputs are zero).  The Jones program and the VRS Ez derivation run
//       here.  The kernel is persistent; each CTA stages its next rows (field
//       planes and per-pixel parameter planes) into shared memory with TMA
//       bulk copies while it transforms the current ones.
//   column pass (rs_cols_conv): for each of the P spectrum columns, the
//       P-point FFT along y (pruned input), the multiply by the transfer
//       spectrum, the inverse FFT, and the N output rows that survive the crop
//       (the last pass computes only those), written back in place.
//   inverse row pass (rs_rows_inv): inverse P-point FFT of each row, crop to
//       N columns, optional fused epilogue program, store.  The loads of the
//       next row are in flight while the current one is transformed.
//
// Intermediate data per component: N rows x P complex64 in column tiles of W:
// element (row r, column c) at ((c / W) * N + r) * W + c % W, so a column
// tile is contiguous and a row is W-wide contiguous runs.  Transfer spectra
// (P x P complex64, natural frequency order) are built once per
// (z, wavelength, grid) by rs_hhat_rows / rs_hhat_cols in column tiles of SW
// with P rows: S[((kx / SW) * P + ky) * SW + kx % SW].
#pragma once

#include <math.h>
#include <stdint.h>

#include <type_traits>
#include <vector>

#include "fft64.cuh"
#include "line_fft.cuh"
#include "rs_host.h"

namespace xl {

// Shapes of the RS kernels for Q = 2^LOGQ.  Every line transform is a
// P-point FFT by T = P / 16 threads holding 16 elements each; thread j holds
// elements j + m T, so the nonzero (and surviving) half of a line is m < 8.
template <int LOGQ> struct RsCfg {
  static constexpr int LOGP = LOGQ + 1;
  static constexpr int Q = 1 << LOGQ;
  static constexpr int P = 2 * Q;
  static constexpr int E = 16;
  static constexpr int H = E / 2;
  static constexpr int T = P / E;
  static constexpr int XS = P + P / 16;                       // exchange slots per line
  static constexpr int G = (256 / T) > 1 ? (256 / T) : 1;     // lines per CTA in the row passes
  static constexpr int ROW_THREADS = G * T;
  // Column-tile width of the intermediate and spectrum layouts.  At Q = 2048
  // the tiles are 8 columns wide, so a warp's row access is four 64-byte
  // pieces; the column pass takes half a tile per CTA.
  static constexpr int W = LOGQ >= 12 ? 2 : (LOGQ == 11 ? 8 : ((32 / T) > 4 ? (32 / T) : 4));
  // Column-pass (and spectrum-build) CTAs take CW columns of a tile,
  // interleaved in the lanes of every warp.
  static constexpr int CW = LOGQ == 11 ? 4 : W;
  // the transfer spectrum is tiled CW wide: exactly the columns of one
  // column-pass CTA, so its reads are whole 32-byte pieces
  static constexpr int SW = CW;
  // per-column padding of the exchange buffers: without it the CW
  // interleaved buffers would start on the same bank
  static constexpr int CXS = XS + (CW >= 8 ? 0 : 16 / CW);
  static constexpr int COL_THREADS = CW * T;
  static constexpr int COL_MINB = (1024 / COL_THREADS) > 1 ? (1024 / COL_THREADS) : 1;
  static constexpr int NTW = FftTw<LOGP, E>::SIZE;           // pass twiddle table entries
  static_assert(COL_THREADS >= 32 && COL_THREADS <= 1024, "column CTA shape");
  static_assert(W % CW == 0, "column-pass CTAs cover whole tiles");
};

// Element addresses of one row (columns j + m T) in a column-tiled plane.
// The base pointer and stride pass through empty asm statements so that the
// compiler recomputes them per row and component instead of keeping sixteen
// 64-bit addresses live across the unrolled component loop.
template <int LOGQ, class Tp>
struct RowPtr {
  Tp* q;
  long long step;
  __device__ __forceinline__ RowPtr(Tp* plane, int r, int j, int rows) {
    using C = RsCfg<LOGQ>;
    q = plane + tiled<C::W>(r, j, rows);
    step = (long long)C::T * rows;
    asm volatile("" : "+l"(q), "+l"(step));
  }
  __device__ __forceinline__ Tp& operator[](int m) const { return q[m * step]; }
};

// ---------------------------------------------------------------------------
// Transfer spectrum, step 0: the wrapped offsets split into float-float
// (hi, lo) pairs, offx into off[0 .. P), offy into off[P .. 2P).  `off` is the
// spectrum buffer, which step 2 overwrites afterwards.
static __global__ void rs_split_offsets(const double* __restrict__ offx, const double* __restrict__ offy, int P,
                                 float2* __restrict__ off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * P) return;
  const ffloat v = ff_split(i < P ? offx[i] : offy[i - P]);
  off[i] = make_float2(v.hi, v.lo);
}

// Transfer spectrum, step 1: rows of the wrapped impulse response -> P-point
// row spectra, row-major in natural order.
// DZ: the rows of dH/dz instead (the spectrum of the z-derivative).
template <int LOGQ, bool DZ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::ROW_THREADS)
    rs_hhat_rows(int ny, int nx, const float2* __restrict__ off, double zh, const double* __restrict__ zp,
                 double inv_lambda, float k, float2* __restrict__ out) {
  using C = RsCfg<LOGQ>;
  // a distance in device memory, or the host's value
  const RsGeom g = rs_geom(zp ? __ldg(zp) : zh, inv_lambda, k);
  extern __shared__ __align__(16) float2 smem[];
  const int tid = threadIdx.x;
  const int gi = tid / C::T, j = tid % C::T;
  const int i = blockIdx.x * C::G + gi;   // row of the wrapped response (< P)
  const bool vy = (i < ny) || (i > C::P - ny);
  const float2 oy = off[C::P + i];
  const ffloat y = {oy.x, oy.y};
  const ffloat zy = ff_add(g.z2, ff_mul(y, y));
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int col = j + m * C::T;
    const bool vx = (col < nx) || (col > C::P - nx);
    v[m] = make_float2(0.f, 0.f);
    if (vy && vx) {
      const float2 ox = off[col];
      const ffloat x = {ox.x, ox.y};
      const ffloat sq = ff_add(zy, ff_mul(x, x));
      v[m] = DZ ? rs_dz_value_s(g, sq) : rs_value_s(g, sq);
    }
  }
  block_fft_x<C::LOGP, 16, -1, false, true>(v, j, smem + gi * C::XS, pass_tw<C::LOGP>());
  float2* dst = out + (long long)i * C::P;
#pragma unroll
  for (int m = 0; m < 16; ++m) dst[j + m * C::T] = v[m];
}

// Transfer spectrum, step 2: P-point column transforms of the row spectra,
// times `scale`, stored column-tiled: S[((kx / SW) * P + ky) * SW + kx % SW].
template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::COL_THREADS)
    rs_hhat_cols(const float2* __restrict__ in, float scale, float2* __restrict__ out) {
  using C = RsCfg<LOGQ>;
  constexpr int W = C::W, CW = C::CW, LPW = 32 / CW;
  extern __shared__ __align__(16) float2 smem[];
  const int tid = threadIdx.x, lane = tid & 31;
  const int wc = lane % CW, j = (tid >> 5) * LPW + lane / CW;
  const int t = blockIdx.x / (W / CW);                      // column tile
  const int w = (blockIdx.x % (W / CW)) * CW + wc;          // column within the tile
  float2 v[16];
  const float2* src = in + t * W + w;
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = src[(long long)(j + m * C::T) * C::P];
  block_fft_x<C::LOGP, 16, -1, false, true>(v, j, smem + wc * C::CXS, pass_tw<C::LOGP>());
  const int kx = t * W + w;
  float2* dst = out + (long long)(kx / C::SW) * C::P * C::SW + kx % C::SW;
#pragma unroll
  for (int m = 0; m < 16; ++m) dst[(long long)(j + m * C::T) * C::SW] = cscale(v[m], scale);
}

// Thread organisation of the row passes for NC transformed components: CG
// component groups of G lines of T threads, where CG = NC (every component of
// a row transformed at once) when the CTA can hold them, else 1 (the
// components one after the other).
template <int LOGQ, int NC> struct RowCfg {
  using C = RsCfg<LOGQ>;
  static constexpr int CG = (NC * C::G * C::T <= 1024) ? NC : 1;
  static constexpr int LINES = CG * C::G;
  static constexpr int THREADS = LINES * C::T;
  static constexpr int MINB = (768 / THREADS) > 1 ? (768 / THREADS) : 1;   // resident CTAs per SM
};

// Forward row pass.  MODE 1: scalar RS (one component); 2: VRS (Ex, Ey in;
// Ex, Ey, Ez out, Ez derived); 3: VRS adjoint (three gradients in and out).
// Persistent: CTA c handles row groups c, c + grid, ...  Per row group the
// prologue runs the fused program over every pixel and writes the components
// to a shared buffer; the stage is then free, so the bulk copies of the next
// row group start while the component groups transform this one.
// FK: the fused program's op kinds fixed at compile time (FixedKinds<...>,
// for the programs the benchmarks and tables run), or FixedKinds<>.
template <int LOGQ, int MODE, class FK = FixedKinds<>>
__global__ void __launch_bounds__(RowCfg<LOGQ, MODE == 1 ? 1 : 3>::THREADS, RowCfg<LOGQ, MODE == 1 ? 1 : 3>::MINB)
    rs_rows_fwd(const __grid_constant__ RsLaunch p, const __grid_constant__ RowStage st) {
  using C = RsCfg<LOGQ>;
  constexpr int NC = MODE == 1 ? 1 : 3;
  constexpr int CIN = MODE;
  using F = RowCfg<LOGQ, NC>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nx = p.nx, ny = p.ny;
  float2* xch = (float2*)smraw;                                      // LINES x XS
  float2* post = xch + F::LINES * C::XS;                             // NC x G x nx
  float* xf = (float*)(post + (size_t)NC * C::G * nx);               // nx (VRS: x as float32)
  const size_t soff = ((size_t)(F::LINES * C::XS + NC * C::G * nx) * 8 + (MODE == 2 ? (size_t)nx * 4 : 0) + 15) /
                      16 * 16;
  unsigned char* stage = smraw + soff;
  unsigned long long* mbar = (unsigned long long*)(stage + (size_t)C::G * st.row_bytes);
  const int tid = threadIdx.x;
  const int line = tid / C::T, j = tid % C::T;
  const int cg = line / C::G, gi = line % C::G;
  const int ngb = (ny + C::G - 1) / C::G;
  const int total = p.B * ngb;
  const bool staged = st.n > 0;

  if (tid == 0 && staged) {
    mbar_init(mbar, 1);
    fence_mbar_init();
  }
  if constexpr (MODE == 2)
    for (int i = tid; i < nx; i += blockDim.x) xf[i] = (float)p.x[i];
  __syncthreads();

  // row groups are taken batch entries fastest: CTAs that run together read the
  // same rows of the parameter planes a batch shares, which then come from L2
  auto issue = [&](int grp) {
    const int b = grp % p.B, r0 = (grp / p.B) * C::G;
    stage_rows(st, stage, mbar, b, r0, min(C::G, ny - r0));
  };
  if (tid == 0 && staged && blockIdx.x < total) issue(blockIdx.x);

  unsigned phase = 0;
  for (int grp = blockIdx.x; grp < total; grp += gridDim.x) {
    const int b = grp % p.B;
    const int r0 = (grp / p.B) * C::G;
    // a wait that runs out is acted on at the barrier after the prologue
    // (the prologue then works on stale data, and the launch's output is not
    // valid), so that no extra barrier is taken per row group
    const bool got = !staged || mbar_wait_bounded(mbar, phase, g_wait_limit_ns);
    // prologue over the row group's pixels, one per thread at a time (CTAs of
    // more than 256 threads: the four-pixel form below ran slower in them)
    if constexpr (F::THREADS > 256) {
      int last = -1;
      float Y = 0.f, z2 = 0.f;
      for (int idx = tid; idx < C::G * nx; idx += F::THREADS) {
        const int g2 = C::G == 1 ? 0 : idx / nx, n = idx - g2 * nx, r = r0 + g2;
        if (r >= ny) break;
        const long long pix = (long long)r * nx + n;
        float2 e[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int c = 0; c < CIN; ++c) {
          const int fo = st.fld[c];
          e[c] = fo >= 0 ? ((const float2*)(stage + fo))[g2 * nx + n] : p.in[c][(long long)b * p.ibs + pix];
        }
        if constexpr (FK::n > 0) {
          apply_prog_fixed1<FK>(p.pre, e, PixelCtx{r, n, pix, b}, StagedParams{stage, &st, g2, nx, n});
        } else if (p.pre.nops) {
          PixelCtx px{r, n, pix, b};
          apply_prog_r(p.pre, e, px, StagedParams{stage, &st, g2, nx, n});
        }
        if constexpr (MODE == 2) {  // vectorized_optics.py:258-261, Ez = Ex X/r + Ey Y/r
          if (g2 != last) {
            last = g2;
            Y = (float)p.y[r];
            const float zb = (float)p.z[b];
            z2 = Y * Y + zb * zb;
          }
          const float X = xf[n];
          const float inv = rsqrtf(X * X + z2);
          e[2] = cadd(cscale(e[0], X * inv), cscale(e[1], Y * inv));
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) post[(c * C::G + g2) * nx + n] = e[c];
      }
    } else
    // CTAs of up to 256 threads: four pixels per thread at a time while four
    // remain, then one; each op of the program is dispatched once for the
    // four, and their loads and arithmetic overlap
    {
      const int lim = min(C::G, ny - r0) * nx;
      const float zb = MODE == 2 ? (float)p.z[b] : 0.f;
      // one row per group (every 2048-point line and longer): its y and
      // y^2 + z^2 once for the group instead of once per pixel
      const float Y0 = MODE == 2 && C::G == 1 ? (float)p.y[r0] : 0.f;
      const float z20 = Y0 * Y0 + zb * zb;
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
            if (c < CIN) {
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
          if constexpr (MODE == 2) {  // vectorized_optics.py:258-261, Ez = Ex X/r + Ey Y/r
            const float Y = C::G == 1 ? Y0 : (float)p.y[r];
            const float z2 = C::G == 1 ? z20 : Y * Y + zb * zb;
            const float X = xf[n];
            const float inv = rsqrtf(X * X + z2);
            e[q][2] = cadd(cscale(e[q][0], X * inv), cscale(e[q][1], Y * inv));
          }
#pragma unroll
          for (int c = 0; c < NC; ++c) post[(c * C::G + (r - r0)) * nx + n] = e[q][c];
        }
      };
      int base = tid;
      for (; base + 3 * F::THREADS < lim; base += 4 * F::THREADS) chunk(std::integral_constant<int, 4>{}, base);
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
    if (tid == 0 && staged && grp + gridDim.x < total) {
      fence_proxy_async();
      issue(grp + gridDim.x);
    }
    const int r = r0 + gi;
    const bool live = r < ny;
    for (int c = cg; c < NC; c += F::CG) {
      float2 v[16];
      const float2* src = post + (c * C::G + gi) * nx;
#pragma unroll
      for (int m = 0; m < C::H; ++m) {
        const int n = j + m * C::T;
        v[m] = (live && n < nx) ? src[n] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int m = C::H; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
      block_fft_x<C::LOGP, 16, -1, true, true>(v, j, xch + line * C::XS, pass_tw<C::LOGP>());
      if (live) {
        float2* plane = p.work + ((long long)b * NC + c) * ny * C::P;
        if constexpr (C::T % C::W == 0) {
          const RowPtr<LOGQ, float2> o(plane, r, j, ny);
#pragma unroll
          for (int m = 0; m < 16; ++m) o[m] = v[m];
        } else {
#pragma unroll
          for (int m = 0; m < 16; ++m) plane[tiled<C::W>(r, j + m * C::T, ny)] = v[m];
        }
      }
    }
  }
}

// ---- Tensor Memory (tcgen05) as per-thread storage ----
// TMEM is 128 lanes x 512 columns of 32-bit cells per SM.  With the 32x32b
// access shape, thread i of warp w reads and writes lane 32 (w mod 4) + i, so
// each thread owns its own cells; the kernels below give a thread 32
// consecutive columns of its lane (16 complex values).  One warp allocates
// the CTA's columns and hands the base address out through shared memory;
// the same warp frees them before the CTA exits.
__device__ __forceinline__ void tmem_alloc(unsigned* dst_smem, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// four complex values into this thread's cells [col, col + 8)
__device__ __forceinline__ void tmem_st4(unsigned taddr, float2 a, float2 b, float2 c, float2 d) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y), "f"(d.x), "f"(d.y)
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// four complex values back; the values pass through the wait so that no use
// is scheduled before the load has completed
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float2 (&o)[4]) {
  float r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+f"(r[0]), "+f"(r[1]), "+f"(r[2]), "+f"(r[3]), "+f"(r[4]), "+f"(r[5]), "+f"(r[6]), "+f"(r[7])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = make_float2(r[2 * i], r[2 * i + 1]);
}

// Column pass, in place on one tile of W spectrum columns: FFT along y of the
// ny nonzero rows (pruned first pass), multiply by the transfer spectrum
// (conjugate for the adjoint), inverse FFT, keep the ny surviving rows.
// A CTA takes CW columns of a tile; lanes interleave them, so every warp
// access is one contiguous run of CW columns.
// L2 prefetch (PF): the CTA's spectrum columns at the start, and the next
// component's column tile while this one is transformed, so that their loads
// meet L2 rather than DRAM latency.
// PERSIST: one CTA per resident slot walks the (batch entry, column group)
// units batch entries fastest, as the grid does otherwise; the pass twiddle
// table is then loaded once per CTA instead of once per unit.
// TM (with PERSIST): the unit's spectrum values are read from global memory
// for its first component only and kept in Tensor Memory for the others
// (each thread's 16 values in its own TMEM cells), so the three components of
// a VRS field read the spectrum tile from L2 once instead of three times.
// The CTA allocates 256 of an SM's 512 TMEM columns; its shared memory allows
// one such CTA per SM and no other kernel of the library allocates Tensor
// Memory, so the allocation never has to wait for columns to be freed.
template <int LOGQ, bool PF, bool PERSIST = false, bool TM = false>
__global__ void __launch_bounds__(RsCfg<LOGQ>::COL_THREADS, RsCfg<LOGQ>::COL_MINB)
    rs_cols_conv(const __grid_constant__ RsLaunch p) {
  using C = RsCfg<LOGQ>;
  constexpr int W = C::W, CW = C::CW, LPW = 32 / CW;
  // TMEM columns: 32 per thread, the warps of a lane quarter side by side
  constexpr unsigned TM_COLS = (unsigned)(C::COL_THREADS / 128) * 32u;
  static_assert(!TM || (PERSIST && C::COL_THREADS % 128 == 0 && TM_COLS >= 32 && TM_COLS <= 256 &&
                        (TM_COLS & (TM_COLS - 1)) == 0),
                "TMEM spectrum cache: persistent CTAs of whole warp quarters, a power-of-two column count");
  extern __shared__ __align__(16) float2 smem[];
  __shared__ unsigned s_tmem;
  float2* xch = smem;                  // CW x CXS
  float2* stw = smem + CW * C::CXS;    // NTW
  const int tid = threadIdx.x, lane = tid & 31;
  const int wc = lane % CW, j = (tid >> 5) * LPW + lane / CW;
  if constexpr (TM) {
    if (tid < 32) tmem_alloc(&s_tmem, TM_COLS);
  }
  {
    const float2* g = pass_tw<C::LOGP>();
    for (int i = tid; i < C::NTW; i += blockDim.x) stw[i] = g[i];
  }
  if constexpr (TM) tmem_fence_before_sync();
  __syncthreads();
  unsigned tcell = 0;   // this thread's first TMEM cell: lane 32 (warp mod 4) + lane, 32 columns per warp
  if constexpr (TM) {
    tmem_fence_after_sync();
    tcell = s_tmem + ((32u * ((unsigned)(tid >> 5) & 3u)) << 16) + (unsigned)(tid >> 7) * 32u;
  }
  float2* xb = xch + wc * C::CXS;
  const int ny = p.ny;
  const int units = PERSIST ? p.B * (C::P / CW) : 1;
#pragma unroll 1
  for (int u = PERSIST ? (int)blockIdx.x : 0; u < units; u += PERSIST ? (int)gridDim.x : 1) {
    // batch entries fastest: the CTAs of one column tile run together and share
    // its transfer-spectrum columns in L2
    const int b = PERSIST ? u % p.B : (int)blockIdx.x;
    const int g = PERSIST ? u / p.B : (int)blockIdx.y;
    const int t = g / (W / CW);                      // column tile
    const int w = (g % (W / CW)) * CW + wc;          // column within the tile
    const int kx = t * W + w;
    const float2* sbase = p.specs ? p.specs[b] : p.spec + (long long)(p.sidx ? p.sidx[b] : 0) * p.sstride;
    const float2* spec = sbase + (long long)(kx / C::SW) * C::P * C::SW + kx % C::SW;
    if (PF && tid == 0) l2_prefetch(sbase + (long long)(kx / C::SW) * C::P * C::SW, (unsigned)(C::P * C::SW * 8));
#pragma unroll 1
    for (int c = 0; c < p.cout; ++c) {
      float2* tile = p.work + ((long long)b * p.cout + c) * ny * C::P + (long long)t * ny * W + w;
      if (PF && tid == 0 && c + 1 < p.cout)
        l2_prefetch(p.work + ((long long)b * p.cout + c + 1) * ny * C::P + (long long)t * ny * W,
                    (unsigned)(ny * W * 8));
      float2 v[16];
#pragma unroll
      for (int m = 0; m < C::H; ++m) {
        const int n = j + m * C::T;
        v[m] = n < ny ? tile[(long long)n * W] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int m = C::H; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
      block_fft_x<C::LOGP, 16, -1, true, false>(v, j, xb, stw);
      // the spectrum loads stay here rather than ahead of the transform, where
      // they would hold 32 registers through it
      if (TM && c > 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 s[4];
          tmem_ld4(tcell + 8u * q, s);
#pragma unroll
          for (int i = 0; i < 4; ++i) v[4 * q + i] = p.adjoint ? cmulc(v[4 * q + i], s[i]) : cmul(v[4 * q + i], s[i]);
        }
      } else if (TM) {
        const float2* sp = spec;
        asm volatile("" : "+l"(sp));
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 s[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) s[i] = __ldg(sp + (long long)(j + (4 * q + i) * C::T) * C::SW);
          tmem_st4(tcell + 8u * q, s[0], s[1], s[2], s[3]);
#pragma unroll
          for (int i = 0; i < 4; ++i) v[4 * q + i] = p.adjoint ? cmulc(v[4 * q + i], s[i]) : cmul(v[4 * q + i], s[i]);
        }
        tmem_wait_st();   // the stores are complete before the next component's loads
      } else {
        const float2* sp = spec;
        asm volatile("" : "+l"(sp));
        if (p.adjoint) {
#pragma unroll
          for (int m = 0; m < 16; ++m) v[m] = cmulc(v[m], __ldg(sp + (long long)(j + m * C::T) * C::SW));
        } else {
#pragma unroll
          for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], __ldg(sp + (long long)(j + m * C::T) * C::SW));
        }
      }
      block_fft_x<C::LOGP, 16, 1, false, false>(v, j, xb, stw);
#pragma unroll
      for (int m = 0; m < C::H; ++m) {
        const int n = j + m * C::T;
        if (n < ny) tile[(long long)n * W] = v[m];
      }
    }
  }
  if constexpr (TM) {
    // every thread is done with its cells before the allocating warp frees them
    tmem_fence_before_sync();
    __syncthreads();
    if (tid < 32) {
      tmem_fence_after_sync();
      tmem_dealloc(s_tmem, TM_COLS);
    }
  }
}

// Column pass at P = 4096 with the radix-64 engine (fft64.cuh): 64 threads
// per column hold 64 elements each, so a transform has one exchange instead
// of two and the CTA (4 columns, 256 threads, one per SM) runs four barriers
// per component instead of eight.  Persistent: each CTA builds the pass-0
// twiddle table once and walks (batch entry, column group) units batch
// entries fastest, as the one-line kernel's grid does.
template <int LOGQ>
__global__ void __launch_bounds__(256, 1) rs_cols_conv64(const __grid_constant__ RsLaunch p) {
  using C = RsCfg<LOGQ>;
  static_assert(C::P == 4096 && C::CW == 4, "radix-64 column pass: P = 4096, 4 columns per CTA");
  constexpr int W = C::W, CW = C::CW;
  extern __shared__ __align__(16) float2 smem[];
  float2* xch = smem;                    // CW lines, F64_XB slots apart
  float2* stw = smem + CW * F64_XB;      // 4096: w4096^(j k) at k * 64 + j
  const int tid = threadIdx.x, lane = tid & 31;
  const int wc = lane & 3, j = (tid >> 5) * 8 + (lane >> 2);
  {
    const float2* g = tw_table(12);
    for (int i = tid; i < 4096; i += 256) stw[i] = f64_twiddle_entry(i, g);
  }
  float2* xb = xch + wc * F64_XB;
  const int ny = p.ny;
  const int units = p.B * (C::P / CW);
#pragma unroll 1
  for (int u = blockIdx.x; u < units; u += gridDim.x) {
    const int b = u % p.B, grp = u / p.B;
    const int t = grp / (W / CW);                      // column tile
    const int w = (grp % (W / CW)) * CW + wc;          // column within the tile
    const int kx = t * W + w;
    const float2* sbase = p.specs ? p.specs[b] : p.spec + (long long)(p.sidx ? p.sidx[b] : 0) * p.sstride;
    const float2* spec = sbase + (long long)(kx / C::SW) * C::P * C::SW + kx % C::SW;
#pragma unroll 1
    for (int c = 0; c < p.cout; ++c) {
      float2* tile = p.work + ((long long)b * p.cout + c) * ny * C::P + (long long)t * ny * W + w;
      float2 v[64];
#pragma unroll
      for (int m = 0; m < 32; ++m) {
        const int n = j + 64 * m;
        v[m] = n < ny ? tile[(long long)n * W] : make_float2(0.f, 0.f);
      }
      f64_pass0<-1, true>(v);
      __syncthreads();   // the previous transform's gathers are done (and the table is built)
      f64_write<-1>(v, j, xb, stw);
      __syncthreads();
      f64_pass1<-1, false>(v, j, xb);
      const float2* sp = spec;
      asm volatile("" : "+l"(sp));
      if (p.adjoint) {
#pragma unroll
        for (int m = 0; m < 64; ++m) v[m] = cmulc(v[m], __ldg(sp + (long long)(j + 64 * m) * C::SW));
      } else {
#pragma unroll
        for (int m = 0; m < 64; ++m) v[m] = cmul(v[m], __ldg(sp + (long long)(j + 64 * m) * C::SW));
      }
      f64_pass0<1, false>(v);
      __syncthreads();
      f64_write<1>(v, j, xb, stw);
      __syncthreads();
      f64_pass1<1, true>(v, j, xb);
#pragma unroll
      for (int m = 0; m < 32; ++m) {
        const int n = j + 64 * m;
        if (n < ny) tile[(long long)n * W] = v[m];
      }
    }
  }
}

// One-line column pass in other CTA shapes: CWK columns per CTA (CWK = CW:
// one CTA per SM; CWK = CW / 2: two), split into NGRP groups of CWK / NGRP
// columns with their own named barriers, so that groups (or co-resident CTAs)
// in different phases overlap one's exchanges with another's arithmetic.
// With L2 prefetch of the spectrum and of the next component's tile.
template <int LOGQ, int CWK, int NGRP> struct RsColShape {
  using C = RsCfg<LOGQ>;
  static constexpr int CWG = CWK / NGRP;                  // columns per group
  static constexpr int THREADS = CWK * C::T;
  static constexpr int MINB = (1024 / THREADS) > 1 ? (1024 / THREADS) : 1;
  static constexpr int XSK = C::XS + (CWG >= 8 ? 0 : 16 / CWG);
  static constexpr size_t SMEM = ((size_t)CWK * XSK + C::NTW) * sizeof(float2);
  static_assert(C::CW % CWK == 0 && CWK % NGRP == 0 && (CWG * C::T) % 32 == 0, "column CTA shape");
};

// STAGGER (two groups): group 1 starts its first component only once group 0
// has finished that component's forward transform, so that the groups run
// half a component apart and one's loads and exchanges meet the other's
// arithmetic instead of its own.
template <int LOGQ, int CWK, int NGRP, bool STAGGER = false>
__global__ void __launch_bounds__(RsColShape<LOGQ, CWK, NGRP>::THREADS, RsColShape<LOGQ, CWK, NGRP>::MINB)
    rs_cols_conv_g(const __grid_constant__ RsLaunch p) {
  using C = RsCfg<LOGQ>;
  using K = RsColShape<LOGQ, CWK, NGRP>;
  constexpr int W = C::W, CWG = K::CWG, LPW = 32 / CWG;
  extern __shared__ __align__(16) float2 smem[];
  float2* stw = smem + CWK * K::XSK;
  const int tid = threadIdx.x, lane = tid & 31;
  const int grp = tid / (CWG * C::T), gtid = tid % (CWG * C::T);
  const int wc = lane % CWG, j = (gtid >> 5) * LPW + lane / CWG;
  const int t = blockIdx.y / (W / CWK);
  const int w = (blockIdx.y % (W / CWK)) * CWK + grp * CWG + wc;
  const int b = blockIdx.x;
  const int ny = p.ny;
  {
    const float2* g = pass_tw<C::LOGP>();
    for (int i = tid; i < C::NTW; i += blockDim.x) stw[i] = g[i];
  }
  __syncthreads();
  const int kx = t * W + w;
  const float2* sbase = p.specs ? p.specs[b] : p.spec + (long long)(p.sidx ? p.sidx[b] : 0) * p.sstride;
  const float2* spec = sbase + (long long)(kx / C::SW) * C::P * C::SW + kx % C::SW;
  float2* xb = smem + (grp * CWG + wc) * K::XSK;
  using Sync = typename std::conditional<(NGRP > 1), GroupSync, CtaSync>::type;
  Sync sync;
  if constexpr (NGRP > 1) sync = GroupSync{1 + grp, CWG * C::T};
  if (tid == 0) l2_prefetch(sbase + (long long)(kx / C::SW) * C::P * C::SW, (unsigned)(C::P * C::SW * 8));
  if constexpr (STAGGER && NGRP == 2) {
    if (grp == 1) asm volatile("bar.sync 3, %0;" ::"r"(K::THREADS) : "memory");
  }
#pragma unroll 1
  for (int c = 0; c < p.cout; ++c) {
    const long long tbase = ((long long)b * p.cout + c) * ny * C::P + (long long)t * ny * W;
    float2* tile = p.work + tbase + w;
    if (tid == 0 && c + 1 < p.cout) l2_prefetch(p.work + tbase + (long long)ny * C::P, (unsigned)(ny * W * 8));
    float2 v[16];
#pragma unroll
    for (int m = 0; m < C::H; ++m) {
      const int n = j + m * C::T;
      v[m] = n < ny ? tile[(long long)n * W] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int m = C::H; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
    block_fft_x<C::LOGP, 16, -1, true, false>(v, j, xb, stw, sync);
    if constexpr (STAGGER && NGRP == 2) {
      if (grp == 0 && c == 0) asm volatile("bar.arrive 3, %0;" ::"r"(K::THREADS) : "memory");
    }
    const float2* sp = spec;
    asm volatile("" : "+l"(sp));
    if (p.adjoint) {
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = cmulc(v[m], __ldg(sp + (long long)(j + m * C::T) * C::SW));
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], __ldg(sp + (long long)(j + m * C::T) * C::SW));
    }
    block_fft_x<C::LOGP, 16, 1, false, false>(v, j, xb, stw, sync);
#pragma unroll
    for (int m = 0; m < C::H; ++m) {
      const int n = j + m * C::T;
      if (n < ny) tile[(long long)n * W] = v[m];
    }
  }
}

// Column pass on the packed two-line engine (fft_pair.cuh): each thread
// transforms two adjacent columns of the CTA's CW at once, so every butterfly
// instruction works on both, and loads, stores and exchanges move the two
// columns' elements as one 16-byte access.  NG = CW / 2 column pairs per CTA.
// GROUPED: pair g is a group of T threads (whole warps) with its own named
// barrier, so the groups drift apart and one group's loads overlap another's
// arithmetic; otherwise the pairs interleave in the lanes of every warp (a
// warp load covers whole 32-byte sectors) under one CTA barrier.
template <int LOGQ, bool GROUPED> struct RsColPair {
  using C = RsCfg<LOGQ>;
  static constexpr int NG = C::CW / 2;
  static constexpr int THREADS = NG * C::T;
  // pair buffers offset by 8 / NG slots mod 8 when the pairs share a warp, so
  // that one quarter-warp's 16-byte accesses fall in distinct banks
  static constexpr int XSP = C::XS + (GROUPED ? 0 : 8 / NG);
  static constexpr size_t SMEM = ((size_t)NG * XSP + C::NTW) * 16;
  static constexpr int MINB = (512 / THREADS) > 1 ? (512 / THREADS) : 1;   // at most 128 registers
  static_assert(C::CW % 2 == 0 && C::T % 32 == 0, "two-line column pass shape");
  static_assert(GROUPED || (32 % NG == 0 && C::T % (32 / NG) == 0), "interleaved lanes");
};

// PF: L2 prefetch as in rs_cols_conv; RP: the next component's inputs are
// loaded into registers at the start of this component's transforms, so their
// latency is spent under the arithmetic.
template <int LOGQ, bool GROUPED, bool PF = false, bool RP = false>
__global__ void __launch_bounds__(RsColPair<LOGQ, GROUPED>::THREADS, RsColPair<LOGQ, GROUPED>::MINB)
    rs_cols_conv_p(const __grid_constant__ RsLaunch p) {
  using C = RsCfg<LOGQ>;
  using K = RsColPair<LOGQ, GROUPED>;
  constexpr int W = C::W, CW = C::CW, NG = K::NG;
  extern __shared__ __align__(16) float4 smem4[];
  float4* stw = smem4 + NG * K::XSP;   // NTW pair twiddles
  const int tid = threadIdx.x, lane = tid & 31;
  const int pr = GROUPED ? tid / C::T : lane % NG;
  const int j = GROUPED ? tid % C::T : (tid >> 5) * (32 / NG) + lane / NG;
  const int t = blockIdx.y / (W / CW);                       // column tile
  const int w = (blockIdx.y % (W / CW)) * CW + 2 * pr;       // first column of the pair within the tile
  const int b = blockIdx.x;
  const int ny = p.ny;
  {
    const float4* g = pass_tw4<C::LOGP>();
    for (int i = tid; i < C::NTW; i += blockDim.x) stw[i] = g[i];
  }
  __syncthreads();
  const int kx = t * W + w;
  const float2* sbase = p.specs ? p.specs[b] : p.spec + (long long)(p.sidx ? p.sidx[b] : 0) * p.sstride;
  const float2* spec = sbase + (long long)(kx / C::SW) * C::P * C::SW + kx % C::SW;
  float4* xb = smem4 + pr * K::XSP;
  using Sync = typename std::conditional<GROUPED, GroupSync, CtaSync>::type;
  Sync sync;
  if constexpr (GROUPED) sync = GroupSync{1 + pr, C::T};
  auto tile_of = [&](int c) {
    return p.work + ((long long)b * p.cout + c) * ny * C::P + (long long)t * ny * W + w;
  };
  auto load_in = [&](int c, float4 (&dst)[C::H]) {
    const float2* tl = tile_of(c);
#pragma unroll
    for (int m = 0; m < C::H; ++m) {
      const int n = j + m * C::T;
      dst[m] = n < ny ? *(const float4*)(tl + (long long)n * W) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  if (PF && tid == 0) l2_prefetch(sbase + (long long)(kx / C::SW) * C::P * C::SW, (unsigned)(C::P * C::SW * 8));
  float4 nxt[RP ? C::H : 1];
  if constexpr (RP) load_in(0, nxt);
#pragma unroll 1
  for (int c = 0; c < p.cout; ++c) {
    float2* tile = tile_of(c);
    if (PF && tid == 0 && c + 1 < p.cout) l2_prefetch(tile_of(c + 1) - w, (unsigned)(ny * W * 8));
    cpair v[16];
    if constexpr (RP) {
#pragma unroll
      for (int m = 0; m < C::H; ++m) v[m] = p_from(nxt[m]);
      if (c + 1 < p.cout) load_in(c + 1, nxt);
    } else {
#pragma unroll
      for (int m = 0; m < C::H; ++m) {
        const int n = j + m * C::T;
        v[m] = n < ny ? p_from(*(const float4*)(tile + (long long)n * W)) : pz();
      }
    }
#pragma unroll
    for (int m = C::H; m < 16; ++m) v[m] = pz();
    block_pfft<C::LOGP, -1, true, false>(v, j, xb, stw, sync);
    const float2* sp = spec;
    asm volatile("" : "+l"(sp));
    if (p.adjoint) {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const float4 s = __ldg((const float4*)(sp + (long long)(j + m * C::T) * C::SW));
        v[m] = pmul_pp<true>(v[m], make_float2(s.x, s.z), make_float2(s.y, s.w));
      }
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const float4 s = __ldg((const float4*)(sp + (long long)(j + m * C::T) * C::SW));
        v[m] = pmul_pp<false>(v[m], make_float2(s.x, s.z), make_float2(s.y, s.w));
      }
    }
    block_pfft<C::LOGP, 1, false, false>(v, j, xb, stw, sync);
#pragma unroll
    for (int m = 0; m < C::H; ++m) {
      const int n = j + m * C::T;
      if (n < ny) *(float4*)(tile + (long long)n * W) = p_to(v[m]);
    }
  }
}

// Inverse row pass: inverse P-point FFT per row and component, crop to nx
// columns (the last pass computes only the surviving half), optional fused
// epilogue program (or, for the VRS adjoint, the fold of the Ez gradient into
// Ex, Ey), store.  Persistent, with the component groups of RowCfg; each
// thread's loads of its next row are in flight in registers while the
// current one is transformed.  With an epilogue the transformed rows go to a
// shared buffer first, since the program needs every component of a pixel.
template <int LOGQ, int COUT, bool EPI>
__global__ void __launch_bounds__(RowCfg<LOGQ, COUT>::THREADS, RowCfg<LOGQ, COUT>::MINB) rs_rows_inv(const __grid_constant__ RsLaunch p) {
  using C = RsCfg<LOGQ>;
  using F = RowCfg<LOGQ, COUT>;
  extern __shared__ __align__(16) float2 smem[];
  const int tid = threadIdx.x;
  const int line = tid / C::T, j = tid % C::T;
  const int cg = line / C::G, gi = line % C::G;
  const int nx = p.nx, ny = p.ny;
  const int ngb = (ny + C::G - 1) / C::G;
  const int total = p.B * ngb;
  float2* xb = smem + line * C::XS;
  float2* post = smem + F::LINES * C::XS;     // COUT x G x nx (epilogue only)

  auto load = [&](int grp, int c, float2 (&dst)[16]) {   // row groups batch entries fastest
    const int b = grp % p.B;
    int r = (grp / p.B) * C::G + gi;
    r = r < ny ? r : ny - 1;    // rows past the end load a valid row and discard it
    const float2* plane = p.work + ((long long)b * COUT + c) * ny * C::P;
    if constexpr (C::T % C::W == 0) {
      const RowPtr<LOGQ, const float2> q(plane, r, j, ny);
#pragma unroll
      for (int m = 0; m < 16; ++m) dst[m] = q[m];
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) dst[m] = plane[tiled<C::W>(r, j + m * C::T, ny)];
    }
  };

  float2 nxt[16];
  if (blockIdx.x < total) load(blockIdx.x, cg, nxt);
  for (int grp = blockIdx.x; grp < total; grp += gridDim.x) {
    const int b = grp % p.B;
    const int r0 = (grp / p.B) * C::G;
    const int r = r0 + gi;
    const bool live = r < ny;
    for (int c = cg; c < COUT; c += F::CG) {
      float2 v[16];
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = nxt[m];
      if (c + F::CG < COUT) load(grp, c + F::CG, nxt);
      else if (grp + gridDim.x < total) load(grp + gridDim.x, cg, nxt);
      if constexpr (!EPI && F::CG > 1)   // the component groups never meet: own barriers
        block_fft_x<C::LOGP, 16, 1, false, true>(v, j, xb, pass_tw<C::LOGP>(),
                                                 GroupSync{1 + cg, C::G * C::T});
      else
        block_fft_x<C::LOGP, 16, 1, false, true>(v, j, xb, pass_tw<C::LOGP>());
      if constexpr (!EPI) {
        if (live) {
          float2* o = p.out[c] + (long long)b * p.obs + (long long)r * nx;
#pragma unroll
          for (int m = 0; m < C::H; ++m) {
            const int n = j + m * C::T;
            if (n < nx) o[n] = v[m];
          }
        }
      } else {
        float2* d = post + (c * C::G + gi) * nx;
#pragma unroll
        for (int m = 0; m < C::H; ++m) {
          const int n = j + m * C::T;
          if (n < nx) d[n] = v[m];
        }
      }
    }
    if constexpr (EPI) {
      __syncthreads();
      const bool fold = p.adjoint && COUT == 3;   // VRS adjoint: Ez gradient folded into Ex, Ey
      int last = -1;
      float Y = 0.f, z2 = 0.f;
      for (int idx = tid; idx < C::G * nx; idx += F::THREADS) {
        const int g2 = C::G == 1 ? 0 : idx / nx, n = idx - g2 * nx, ro = r0 + g2;
        if (ro >= ny) break;
        const long long o = (long long)b * p.obs + (long long)ro * nx + n;
        float2 e[3];
        const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 3; ++c) e[c] = c < COUT ? post[(c * C::G + g2) * nx + n] : zero;
        if (fold) {  // adjoint of Ez = Ex X/r + Ey Y/r (vectorized_optics.py:258-261)
          if (g2 != last) {
            last = g2;
            Y = (float)p.y[ro];
            const float zb = (float)p.z[b];
            z2 = Y * Y + zb * zb;
          }
          const float X = (float)p.x[n];
          const float inv = rsqrtf(X * X + z2);
          p.out[0][o] = cadd(e[0], cscale(e[2], X * inv));
          p.out[1][o] = cadd(e[1], cscale(e[2], Y * inv));
          if (p.out[2]) p.out[2][o] = e[2];   // the unfolded Ez gradient, when asked for
          continue;
        }
        PixelCtx px{ro, n, (long long)ro * nx + n, b};
        apply_prog(p.post, e, px);
#pragma unroll
        for (int c = 0; c < COUT; ++c) p.out[c][o] = e[c];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host side.

template <int LOGQ>
int rs_spectrum(cudaStream_t st, int ny, int nx, const double* offx, const double* offy, double z,
                const double* zp, double wavelength, double scale, float2* spec, float2* work, int dz) {
  using C = RsCfg<LOGQ>;
  const size_t sm1 = (size_t)C::G * C::XS * sizeof(float2);
  const float k = (float)(2.0 * M_PI / wavelength);
  cudaError_t e;
  rs_split_offsets<<<(2 * C::P + 255) / 256, 256, 0, st>>>(offx, offy, C::P, spec);
  XL_CHECK_LAUNCH("rs_split_offsets");
  if (dz) {
    if ((e = allow_smem(rs_hhat_rows<LOGQ, true>, sm1)) != cudaSuccess) return cuda_fail(e, "rs_hhat_rows smem");
    rs_hhat_rows<LOGQ, true><<<C::P / C::G, C::ROW_THREADS, sm1, st>>>(ny, nx, spec, z, zp, 1.0 / wavelength,
                                                                          k, work);
  } else {
    if ((e = allow_smem(rs_hhat_rows<LOGQ, false>, sm1)) != cudaSuccess) return cuda_fail(e, "rs_hhat_rows smem");
    rs_hhat_rows<LOGQ, false><<<C::P / C::G, C::ROW_THREADS, sm1, st>>>(ny, nx, spec, z, zp, 1.0 / wavelength,
                                                                           k, work);
  }
  XL_CHECK_LAUNCH("rs_hhat_rows");
  const size_t sm2 = (size_t)C::CW * C::CXS * sizeof(float2);
  e = allow_smem(rs_hhat_cols<LOGQ>, sm2);
  if (e != cudaSuccess) return cuda_fail(e, "rs_hhat_cols smem");
  rs_hhat_cols<LOGQ><<<C::P / C::CW, C::COL_THREADS, sm2, st>>>(work, (float)scale, spec);
  XL_CHECK_LAUNCH("rs_hhat_cols");
  return XL_OK;
}

template <int LOGQ, int MODE, class FK = FixedKinds<>>
static int launch_rows_fwd(cudaStream_t s, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  constexpr int NC = MODE == 1 ? 1 : 3;
  using F = RowCfg<LOGQ, NC>;
  const size_t fixed = ((size_t)(F::LINES * C::XS + NC * C::G * p.nx) * 8 + (MODE == 2 ? (size_t)p.nx * 4 : 0) +
                        15) / 16 * 16;
  RowStage st;
  plan_row_stage(p.cin, p.in, p.ibs, p.nx, p.pre, C::G, fixed, st);
  const size_t sm = fixed + (size_t)C::G * st.row_bytes + 16;
  if (sm > 227 * 1024) {
    set_error("rs: row of %d columns too long for shared memory", p.nx);
    return XL_EUNSUPPORTED;
  }
  cudaError_t e = allow_smem(rs_rows_fwd<LOGQ, MODE, FK>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "rs_rows_fwd smem");
  const int total = p.B * ((p.ny + C::G - 1) / C::G);
  const int grid = persistent_grid(rs_rows_fwd<LOGQ, MODE, FK>, F::THREADS, sm, total);
  rs_rows_fwd<LOGQ, MODE, FK><<<grid, F::THREADS, sm, s>>>(p, st);
  XL_CHECK_LAUNCH("rs_rows_fwd");
  return XL_OK;
}

template <int LOGQ, int COUT, bool EPI>
static int launch_rows_inv(cudaStream_t s, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  using F = RowCfg<LOGQ, COUT>;
  const size_t sm = (size_t)(F::LINES * C::XS + (EPI ? COUT * C::G * p.nx : 0)) * sizeof(float2);
  if (sm > 227 * 1024) {
    set_error("rs: row of %d columns too long for shared memory", p.nx);
    return XL_EUNSUPPORTED;
  }
  cudaError_t e = allow_smem(rs_rows_inv<LOGQ, COUT, EPI>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "rs_rows_inv smem");
  const int total = p.B * ((p.ny + C::G - 1) / C::G);
  const int grid = persistent_grid(rs_rows_inv<LOGQ, COUT, EPI>, F::THREADS, sm, total);
  rs_rows_inv<LOGQ, COUT, EPI><<<grid, F::THREADS, sm, s>>>(p);
  XL_CHECK_LAUNCH("rs_rows_inv");
  return XL_OK;
}

template <int LOGQ, bool GROUPED, bool PF = false, bool RP = false>
static int launch_cols_pair(cudaStream_t st, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  using K = RsColPair<LOGQ, GROUPED>;
  cudaError_t e = allow_smem(rs_cols_conv_p<LOGQ, GROUPED, PF, RP>, K::SMEM);
  if (e != cudaSuccess) return cuda_fail(e, "rs_cols_conv_p smem");
  rs_cols_conv_p<LOGQ, GROUPED, PF, RP><<<dim3(p.B, C::P / C::CW), K::THREADS, K::SMEM, st>>>(p);
  XL_CHECK_LAUNCH("rs_cols_conv_p");
  return XL_OK;
}

template <int LOGQ, int CWK, int NGRP, bool STAGGER = false>
static int launch_cols_g(cudaStream_t st, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  using K = RsColShape<LOGQ, CWK, NGRP>;
  cudaError_t e = allow_smem(rs_cols_conv_g<LOGQ, CWK, NGRP, STAGGER>, K::SMEM);
  if (e != cudaSuccess) return cuda_fail(e, "rs_cols_conv_g smem");
  rs_cols_conv_g<LOGQ, CWK, NGRP, STAGGER><<<dim3(p.B, C::P / CWK), K::THREADS, K::SMEM, st>>>(p);
  XL_CHECK_LAUNCH("rs_cols_conv_g");
  return XL_OK;
}

template <int LOGQ>
static int launch_cols64(cudaStream_t st, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  const size_t sm = (size_t)(C::CW * F64_XB + 4096) * sizeof(float2);
  cudaError_t e = allow_smem(rs_cols_conv64<LOGQ>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "rs_cols_conv64 smem");
  const int grid = persistent_grid(rs_cols_conv64<LOGQ>, 256, sm, p.B * (C::P / C::CW));
  rs_cols_conv64<LOGQ><<<grid, 256, sm, st>>>(p);
  XL_CHECK_LAUNCH("rs_cols_conv64");
  return XL_OK;
}

template <int LOGQ, bool PF, bool PERSIST = false, bool TM = false>
static int launch_cols(cudaStream_t st, const RsLaunch& p) {
  using C = RsCfg<LOGQ>;
  const size_t sm = (size_t)(C::CW * C::CXS + C::NTW) * sizeof(float2);
  cudaError_t e = allow_smem(rs_cols_conv<LOGQ, PF, PERSIST, TM>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "rs_cols_conv smem");
  if constexpr (PERSIST) {
    const int grid = persistent_grid(rs_cols_conv<LOGQ, PF, true, TM>, C::COL_THREADS, sm, p.B * (C::P / C::CW));
    rs_cols_conv<LOGQ, PF, true, TM><<<grid, C::COL_THREADS, sm, st>>>(p);
  } else {
    rs_cols_conv<LOGQ, PF><<<dim3(p.B, C::P / C::CW), C::COL_THREADS, sm, st>>>(p);
  }
  XL_CHECK_LAUNCH("rs_cols_conv");
  return XL_OK;
}

template <int LOGQ>
static int launch_stage(cudaStream_t st, const RsLaunch& p, int stage) {
  using C = RsCfg<LOGQ>;
  if (stage == 0) {
    // the programs of the benchmarks' fields (1024^2 and larger) get a kernel
    // with their op kinds fixed: a phase SLM before scalar RS, an LCD and a
    // polarizer before VRS
    using SlmOnly = FixedKinds<XL_OP_PHASE>;
    using LcdLp = FixedKinds<XL_OP_LCD, XL_OP_LP>;
    if (p.cout == 1) {
      if constexpr (LOGQ >= 10)
        if (SlmOnly::matches(p.pre)) return launch_rows_fwd<LOGQ, 1, SlmOnly>(st, p);
      return launch_rows_fwd<LOGQ, 1>(st, p);
    }
    if (p.cin == 2) {
      if constexpr (LOGQ >= 10)
        if (LcdLp::matches(p.pre)) return launch_rows_fwd<LOGQ, 2, LcdLp>(st, p);
      return launch_rows_fwd<LOGQ, 2>(st, p);
    }
    return launch_rows_fwd<LOGQ, 3>(st, p);
  } else if (stage == 1) {
    const int var = kernel_variant(XL_PASS_RS_COLS, C::LOGP);
    if constexpr (LOGQ >= 9 && LOGQ <= 11) {
      if (var == 1) return launch_cols_pair<LOGQ, false>(st, p);
      if (var == 2) return launch_cols_pair<LOGQ, true>(st, p);
      if (var == 3) return launch_cols<LOGQ, true>(st, p);
      if (var == 4) return launch_cols_pair<LOGQ, false, true, true>(st, p);
      if (var == 5) return launch_cols_g<LOGQ, C::CW, 2>(st, p);
      if (var == 6) return launch_cols_g<LOGQ, C::CW / 2, 1>(st, p);
      if (var == 7) return launch_cols_g<LOGQ, C::CW, 2, true>(st, p);
    }
    if constexpr (LOGQ >= 9 && LOGQ <= 11) {
      if (var == 8) return launch_cols<LOGQ, false, true>(st, p);
    }
    if constexpr (LOGQ == 11) {
      if (var == 9) return launch_cols64<LOGQ>(st, p);
      if (var == 10) return launch_cols<LOGQ, false, true, true>(st, p);
    }
    return launch_cols<LOGQ, false>(st, p);
  } else {
    const bool epi = p.post.nops > 0 || (p.adjoint && p.cout == 3);
    if (p.cout == 1) return epi ? launch_rows_inv<LOGQ, 1, true>(st, p) : launch_rows_inv<LOGQ, 1, false>(st, p);
    return epi ? launch_rows_inv<LOGQ, 3, true>(st, p) : launch_rows_inv<LOGQ, 3, false>(st, p);
  }
  return XL_OK;
}

template <int LOGQ>
int rs_propagate(cudaStream_t st, const RsLaunch& p, int stage) {
  if (stage >= 0) return launch_stage<LOGQ>(st, p, stage);
  for (int s = 0; s < 3; ++s)
    if (int rc = launch_stage<LOGQ>(st, p, s)) return rc;
  return XL_OK;
}

}  // namespace xl

#define XL_RS_INSTANTIATE(L)                                                                        \
  template int xl::rs_spectrum<L>(cudaStream_t, int, int, const double*, const double*, double,      \
                                  const double*, double, double, float2*, float2*, int);           \
  template int xl::rs_propagate<L>(cudaStream_t, const RsLaunch&, int);
