// Rayleigh-Sommerfeld propagation (scalar RS and vectorial VRS) for sm_103a.
//
// The reference (wave_optics.py:281-289) zero-pads the N x N field to
// (2N-1)^2, multiplies fft2(U) by fft2(H) and crops [N-1:, N-1:].  Here the
// same linear convolution runs on a P = 2Q grid (Q = next power of two >= N),
// which gives the identical result because the impulse response is placed
// at wrapped offsets, and the transform is split into Q-point halves:
//
//   row pass (rs_rows_fwd):  for each of the N input rows, the P-point
//       spectrum of the zero-padded row as two Q-point FFTs (even and odd
//       frequencies; the odd half of the input is pre-twiddled by w_P^n).
//       The Jones program and the VRS Ez derivation run in this pass.
//   column pass (rs_cols_conv): for each of the 2Q spectrum columns, the same
//       split along y, a multiply by the transfer spectrum, the inverse split,
//       and only the N output rows that survive the crop are written back.
//   inverse row pass (rs_rows_inv): inverse split along x, crop to N
//       columns, optional fused epilogue program, store.
//
// Intermediate data per component: N rows x 2Q complex64 (one buffer, the
// column pass works in place).  Transfer spectra are built once per
// (z, wavelength, grid) by rs_hhat_rows / rs_hhat_cols and stored
// column-major for the column pass: S[(col*2 + parity)*Q + k].
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace xl {

#ifndef XL_RS_ROW_E
#define XL_RS_ROW_E 8
#endif
#ifndef XL_RS_COL_E
#define XL_RS_COL_E 16
#endif

template <int LOGQ> struct RsCfg {
  static constexpr int Q = 1 << LOGQ;
  static constexpr int P = 2 * Q;
  static constexpr int XS = Q + Q / 16;         // exchange buffer slots
  // row passes: one group of TR threads (ER elements each) per row
  static constexpr int ER = (Q / XL_RS_ROW_E) >= 1 ? XL_RS_ROW_E : 16;
  static constexpr int TR = Q / ER;
  static constexpr int TWR = FftTw<LOGQ, ER>::SIZE;
  static constexpr int RPC = (128 / TR) > 1 ? (128 / TR) : 1;  // rows per CTA
  static constexpr int ROW_THREADS = RPC * TR;
  static constexpr int ROW_MINB = ((ER == 8 ? 1024 : 512) / ROW_THREADS) > 1 ? ((ER == 8 ? 1024 : 512) / ROW_THREADS) : 1;
  // column pass: W groups of TC threads (EC elements each), one per column
  static constexpr int EC = XL_RS_COL_E;
  static constexpr int TC = Q / EC;
  static constexpr int TWC = FftTw<LOGQ, EC>::SIZE;
  // Column-block width of the blocked intermediate and spectrum layouts:
  // element (row r, column col) of a plane with ny rows lives at
  // ((col / W) * ny + r) * W + col % W, so W adjacent columns of one row are
  // contiguous and a column tile is one contiguous block.
  static constexpr int W = (LOGQ >= 12 && EC == 16) ? 2 : ((32 / TC) > 4 ? (32 / TC) : 4);
  static constexpr int CONV_THREADS = W * TC;
  // per-group padding of the column-pass shared buffers: with W groups
  // interleaved in every warp, unpadded buffers would start on the same bank
  static constexpr int CPAD = W >= 8 ? 0 : 4;
  static constexpr int CXS = XS + CPAD;
  static constexpr int CYS = Q + CPAD;
  // the column tile is staged by TMA when the shared memory allows it (Q <= 2048)
  static constexpr bool TMA = LOGQ <= 11;
  // float2 offset of the staged tile: after the exchange, twiddle and even-chain
  // buffers, rounded up to 16 bytes
  static constexpr int TBASE = (W * CXS + TWC + W * CYS + 1) / 2 * 2;
  // one-time spectrum build (16 elements per thread)
  static constexpr int T = Q / 16;
  static constexpr int HRPC = (256 / (2 * T)) > 1 ? (256 / (2 * T)) : 1;
  static constexpr int HROW_THREADS = 2 * HRPC * T;
  static constexpr int WH = (256 / T) < 1 ? 1 : ((256 / T) > 32 ? 32 : (256 / T));
  static constexpr int HCOL_THREADS = 2 * WH * T;
};

template <int LOGQ>
__device__ __forceinline__ long long blk(int r, int col, int ny) {
  constexpr int W = RsCfg<LOGQ>::W;
  return ((long long)(col / W) * ny + r) * W + (col % W);
}

template <int LOGQ, int E>
__device__ __forceinline__ void fill_pass_twiddles(float2* stw) {
  const float2* twQ = tw_table(LOGQ);
  for (int idx = threadIdx.x; idx < FftTw<LOGQ, E>::SIZE; idx += blockDim.x)
    stw[idx] = pass_twiddle_entry<LOGQ, E>(idx, twQ);
}

// ---------------------------------------------------------------------------
// Transfer spectrum, step 1: rows of the wrapped impulse response -> P-point
// row spectra, written row-major in parity-split order (even, then odd).
template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::HROW_THREADS)
    rs_hhat_rows(int ny, int nx, const double* __restrict__ offx, const double* __restrict__ offy, double z,
                 double inv_lambda, float k, float2* __restrict__ out) {
  using C = RsCfg<LOGQ>;
  extern __shared__ float2 smem[];
  float2* row = smem;                         // HRPC x P
  float2* xch = smem + C::HRPC * C::P;        // 2 HRPC x XS
  const int tid = threadIdx.x;
  const int slot = tid / (2 * C::T);
  const int par = (tid / C::T) & 1;
  const int j = tid % C::T;
  const int i0 = blockIdx.x * C::HRPC;

  for (int idx = tid; idx < C::HRPC * C::P; idx += blockDim.x) {
    const int s = idx / C::P, col = idx % C::P, i = i0 + s;
    const bool vy = (i < ny) || (i > C::P - ny);
    const bool vx = (col < nx) || (col > C::P - nx);
    float2 h = make_float2(0.f, 0.f);
    if (i < C::P && vy && vx) h = rs_kernel_value(offx[col], offy[i], z, inv_lambda, k);
    row[idx] = h;
  }
  __syncthreads();

  const float2* twQ = tw_table(LOGQ);
  const float2* twP = tw_table(LOGQ + 1);
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = j + m * C::T;
    const float2 a = row[slot * C::P + n], b = row[slot * C::P + n + C::Q];
    v[m] = par ? cmul(csub(a, b), twP[n]) : cadd(a, b);
  }
  block_fft<LOGQ, 16, -1>(v, j, xch + (2 * slot + par) * C::XS, twQ);
  const int i = i0 + slot;
  if (i < C::P) {
    float2* dst = out + (long long)i * C::P + par * C::Q;
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[j + m * C::T] = v[m];
  }
}

// Transfer spectrum, step 2: P-point column transforms of the row spectra,
// times `scale`, stored in the blocked spectrum layout
// S[((tile*2 + parity)*Q + k)*W + w] for spectrum column tile*W + w.
template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::HCOL_THREADS)
    rs_hhat_cols(const float2* __restrict__ in, float scale, float2* __restrict__ out) {
  using C = RsCfg<LOGQ>;
  constexpr int WH = C::WH, PITCH = C::WH + 1;
  extern __shared__ float2 smem[];
  float2* tile = smem;                  // P x PITCH
  float2* xch = smem + C::P * PITCH;    // 2 WH x XS
  const int tid = threadIdx.x;
  const int w = tid / (2 * C::T);
  const int par = (tid / C::T) & 1;
  const int j = tid % C::T;
  const int c0 = blockIdx.x * WH;

  for (int idx = tid; idx < C::P * WH; idx += blockDim.x) {
    const int r = idx / WH, ww = idx % WH;
    tile[r * PITCH + ww] = in[(long long)r * C::P + c0 + ww];
  }
  __syncthreads();
  const float2* twQ = tw_table(LOGQ);
  const float2* twP = tw_table(LOGQ + 1);
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = j + m * C::T;
    const float2 a = tile[n * PITCH + w], b = tile[(n + C::Q) * PITCH + w];
    v[m] = par ? cmul(csub(a, b), twP[n]) : cadd(a, b);
  }
  block_fft<LOGQ, 16, -1>(v, j, xch + (2 * w + par) * C::XS, twQ);
  const int col = c0 + w;
  float2* dst = out + ((long long)(col / C::W) * 2 + par) * C::Q * C::W + (col % C::W);
#pragma unroll
  for (int m = 0; m < 16; ++m) dst[(long long)(j + m * C::T) * C::W] = cscale(v[m], scale);
}

// ---------------------------------------------------------------------------
struct RsLaunch {
  int B, cin, cout, ny, nx;
  const float2* in[3];
  long long ibs;
  float2* out[3];
  long long obs;
  const double* x;
  const double* y;
  const double* z;
  const float2* spec;
  long long sstride;
  const int* sidx;
  float2* work;
  XlProg pre, post;
  int adjoint;
};

// Row pass: prologue (Jones program; VRS Ez derived at load) and, per
// component, the even- and odd-frequency Q-point row spectra, stored in the
// blocked layout.  One thread group per row.
template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::ROW_THREADS, RsCfg<LOGQ>::ROW_MINB)
    rs_rows_fwd(const RsLaunch p) {
  using C = RsCfg<LOGQ>;
  extern __shared__ float2 smem[];
  const int ns = p.cin;                            // staged components
  float2* stage = smem;                            // RPC x ns x nx
  float2* xch = stage + C::RPC * ns * p.nx;        // RPC x XS
  float2* stw = xch + C::RPC * C::XS;              // TWR
  const int tid = threadIdx.x;
  const int slot = tid / C::TR;
  const int j = tid % C::TR;
  const int b = blockIdx.y;
  const int r0 = blockIdx.x * C::RPC;
  fill_pass_twiddles<LOGQ, C::ER>(stw);

  for (int idx = tid; idx < C::RPC * p.nx; idx += blockDim.x) {
    const int s = idx / p.nx, n = idx % p.nx, r = r0 + s;
    if (r >= p.ny) continue;
    const long long off = (long long)b * p.ibs + (long long)r * p.nx + n;
    float2 e[3];
    e[0] = p.in[0][off];
    e[1] = p.cin > 1 ? p.in[1][off] : make_float2(0.f, 0.f);
    e[2] = p.cin > 2 ? p.in[2][off] : make_float2(0.f, 0.f);
    PixelCtx px{r, n, (long long)r * p.nx + n, b};
    apply_prog(p.pre, e, px);
    stage[(s * ns) * p.nx + n] = e[0];
    if (ns > 1) stage[(s * ns + 1) * p.nx + n] = e[1];
    if (ns > 2) stage[(s * ns + 2) * p.nx + n] = e[2];
  }
  __syncthreads();

  const float2* twP = tw_table(LOGQ + 1);
  const int r = r0 + slot;
  const bool live = r < p.ny;
  const float zb = p.z ? (float)p.z[b] : 0.f;
  const float Y = (live && p.cout == 3) ? (float)p.y[r] : 0.f;
  const float2* st = stage + slot * ns * p.nx;
  float2* xb = xch + slot * C::XS;
  for (int c = 0; c < p.cout; ++c) {
    float2* plane = p.work + ((long long)b * p.cout + c) * p.ny * C::P;
    for (int par = 0; par < 2; ++par) {
      float2 v[C::ER];
#pragma unroll
      for (int m = 0; m < C::ER; ++m) {
        const int n = j + m * C::TR;
        float2 a = make_float2(0.f, 0.f);
        if (live && n < p.nx) {
          if (c < ns) {
            a = st[c * p.nx + n];
          } else {  // vectorized_optics.py:258-261, Ez = Ex X/r + Ey Y/r
            const float X = (float)p.x[n];
            const float inv = rsqrtf(X * X + Y * Y + zb * zb);
            a = cadd(cscale(st[n], X * inv), cscale(st[p.nx + n], Y * inv));
          }
        }
        v[m] = par ? cmul(a, twP[n]) : a;
      }
      block_fft_s<LOGQ, C::ER, -1>(v, j, xb, stw);
      if (live) {
#pragma unroll
        for (int m = 0; m < C::ER; ++m) plane[blk<LOGQ>(r, par * C::Q + j + m * C::TR, p.ny)] = v[m];
      }
    }
  }
}

// Column pass, in place on one tile of W spectrum columns: for each column,
// even chain FFT -> x S_even -> IFFT and odd chain (pre-twiddled) likewise,
// combined in registers; only the ny rows that survive the crop are kept.
// Lanes interleave the W columns so every warp access is 256 contiguous bytes.
// A component's tile (ny x W, contiguous in the blocked layout) is staged into
// shared memory by a TMA bulk copy; the next component's copy is issued once
// the odd chain has read the current tile, so it overlaps that chain's work.
__device__ unsigned int g_rs_timeouts;

template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::CONV_THREADS) rs_cols_conv(const RsLaunch p) {
  using C = RsCfg<LOGQ>;
  constexpr int W = C::W, LPW = 32 / W;
  extern __shared__ __align__(16) float2 smem[];
  float2* xch = smem;                // W x CXS
  float2* stw = smem + W * C::CXS;   // TWC
  float2* yb = stw + C::TWC;         // W x CYS: even-chain result, held across the odd chain
  float2* tb = smem + C::TBASE;      // ny x W: staged tile (TMA), 16-byte aligned
  unsigned long long* mbar = (unsigned long long*)(tb + (C::TMA ? p.ny * W : 0));
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int w = lane % W;
  const int j = (tid >> 5) * LPW + lane / W;
  const int t = blockIdx.x;
  const int b = blockIdx.y;
  const unsigned tile_bytes = (unsigned)(p.ny * W * sizeof(float2));
  auto tile_of = [&](int c) {
    return p.work + ((long long)b * p.cout + c) * p.ny * C::P + (long long)t * p.ny * W;
  };
  if (C::TMA && tid == 0) {
    mbar_init(mbar, 1);
    fence_mbar_init();
  }
  fill_pass_twiddles<LOGQ, C::EC>(stw);
  __syncthreads();
  if (C::TMA && tid == 0) bulk_g2s(tb, tile_of(0), tile_bytes, mbar);
  const float2* twP = tw_table(LOGQ + 1);
  const float2* spec = p.spec + (long long)(p.sidx ? p.sidx[b] : 0) * p.sstride + (long long)t * 2 * C::Q * W + w;
  float2* xb = xch + w * C::CXS;
  float2* y0 = yb + w * C::CYS;
  unsigned phase = 0;
  bool ok = true;

  for (int c = 0; c < p.cout; ++c) {
    float2* tileA = tile_of(c) + w;
    const float2* src = C::TMA ? (const float2*)(tb + w) : (const float2*)tileA;
    if (C::TMA) {
      if (!mbar_wait_bounded(mbar, phase)) ok = false;
      phase ^= 1u;
    }
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      float2 v[C::EC];
#pragma unroll
      for (int m = 0; m < C::EC; ++m) {
        const int n = j + m * C::TC;
        const float2 a = n < p.ny ? src[(long long)n * W] : make_float2(0.f, 0.f);
        v[m] = par ? cmul(a, twP[n]) : a;
      }
      if (C::TMA && par == 1) {
        __syncthreads();   // every thread has read the staged tile
        if (tid == 0 && c + 1 < p.cout) {
          fence_proxy_async();
          bulk_g2s(tb, tile_of(c + 1), tile_bytes, mbar);
        }
      }
      block_fft_s<LOGQ, C::EC, -1>(v, j, xb, stw);
      const float2* sp = spec + (long long)par * C::Q * W;
      if (p.adjoint) {
#pragma unroll
        for (int m = 0; m < C::EC; ++m) v[m] = cmulc(v[m], sp[(long long)(j + m * C::TC) * W]);
      } else {
#pragma unroll
        for (int m = 0; m < C::EC; ++m) v[m] = cmul(v[m], sp[(long long)(j + m * C::TC) * W]);
      }
      block_fft_s<LOGQ, C::EC, 1>(v, j, xb, stw);
      if (par == 0) {
#pragma unroll
        for (int m = 0; m < C::EC; ++m) y0[j + m * C::TC] = v[m];
      } else {
#pragma unroll
        for (int m = 0; m < C::EC; ++m) {
          const int n = j + m * C::TC;
          if (n < p.ny) tileA[(long long)n * W] = cadd(y0[n], cmulc(v[m], twP[n]));
        }
      }
    }
  }
  if (!ok) {
    atomicAdd(&g_rs_timeouts, 1u);
    if (tid == 0) mbar_wait_bounded(mbar, phase);   // a copy may still be in flight
  }
}

// Inverse row pass: inverse of both parity halves, combined in registers,
// cropped to nx columns; optional fused epilogue program; store.
template <int LOGQ>
__global__ void __launch_bounds__(RsCfg<LOGQ>::ROW_THREADS, RsCfg<LOGQ>::ROW_MINB)
    rs_rows_inv(const RsLaunch p) {
  using C = RsCfg<LOGQ>;
  extern __shared__ float2 smem[];
  const int nc = p.cout;
  const bool fold = p.adjoint && nc == 3;      // VRS adjoint: Ez gradient folded into Ex, Ey
  const bool epi = p.post.nops > 0 || fold;
  float2* xch = smem;                           // RPC x XS
  float2* stw = xch + C::RPC * C::XS;           // TWR
  float2* yb = stw + C::TWR;                    // RPC x Q: even-half result
  float2* stage = yb + C::RPC * C::Q;           // RPC x nc x nx (epilogue only)
  const int tid = threadIdx.x;
  const int slot = tid / C::TR;
  const int j = tid % C::TR;
  const int b = blockIdx.y;
  const int r0 = blockIdx.x * C::RPC;
  const int r = r0 + slot;
  const bool live = r < p.ny;
  const int rr = live ? r : 0;
  fill_pass_twiddles<LOGQ, C::ER>(stw);
  __syncthreads();
  const float2* twP = tw_table(LOGQ + 1);
  float2* xb = xch + slot * C::XS;
  float2* y0 = yb + slot * C::Q;

  for (int c = 0; c < nc; ++c) {
    const float2* plane = p.work + ((long long)b * nc + c) * p.ny * C::P;
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      float2 v[C::ER];
#pragma unroll
      for (int m = 0; m < C::ER; ++m) v[m] = plane[blk<LOGQ>(rr, par * C::Q + j + m * C::TR, p.ny)];
      block_fft_s<LOGQ, C::ER, 1>(v, j, xb, stw);
      if (par == 0) {
#pragma unroll
        for (int m = 0; m < C::ER; ++m) y0[j + m * C::TR] = v[m];
      } else if (live) {
#pragma unroll
        for (int m = 0; m < C::ER; ++m) {
          const int n = j + m * C::TR;
          if (n < p.nx) {
            const float2 o = cadd(y0[n], cmulc(v[m], twP[n]));
            if (epi) stage[(slot * nc + c) * p.nx + n] = o;
            else p.out[c][(long long)b * p.obs + (long long)r * p.nx + n] = o;
          }
        }
      }
    }
  }
  if (epi) {
    __syncthreads();
    for (int idx = tid; idx < C::RPC * p.nx; idx += blockDim.x) {
      const int s = idx / p.nx, n = idx % p.nx, ro = r0 + s;
      if (ro >= p.ny) continue;
      const float2 zero = make_float2(0.f, 0.f);
      float2 e[3] = {stage[(s * nc) * p.nx + n], nc > 1 ? stage[(s * nc + 1) * p.nx + n] : zero,
                     nc > 2 ? stage[(s * nc + 2) * p.nx + n] : zero};
      const long long o = (long long)b * p.obs + (long long)ro * p.nx + n;
      if (fold) {  // adjoint of Ez = Ex X/r + Ey Y/r (vectorized_optics.py:258-261)
        const float zb = (float)p.z[b];
        const float X = (float)p.x[n], Y = (float)p.y[ro];
        const float inv = rsqrtf(X * X + Y * Y + zb * zb);
        p.out[0][o] = cadd(e[0], cscale(e[2], X * inv));
        p.out[1][o] = cadd(e[1], cscale(e[2], Y * inv));
        continue;
      }
      PixelCtx px{ro, n, (long long)ro * p.nx + n, b};
      apply_prog(p.post, e, px);
      p.out[0][o] = e[0];
      if (nc > 1) p.out[1][o] = e[1];
      if (nc > 2) p.out[2][o] = e[2];
    }
  }
}

// ---------------------------------------------------------------------------
// Host side.

static int rs_logq(int ny, int nx) {
  const int n = ny > nx ? ny : nx;
  int l = ilog2_ceil(n);
  return l < 4 ? 4 : l;
}

template <int LOGQ>
static int launch_spectrum(cudaStream_t st, int ny, int nx, const double* offx, const double* offy,
                           double z, double wavelength, double scale, float2* spec, float2* work) {
  using C = RsCfg<LOGQ>;
  const size_t sm1 = (size_t)(C::HRPC * C::P + 2 * C::HRPC * C::XS) * sizeof(float2);
  cudaError_t e = allow_smem(rs_hhat_rows<LOGQ>, sm1);
  if (e != cudaSuccess) return cuda_fail(e, "rs_hhat_rows smem");
  const float k = (float)(2.0 * M_PI / wavelength);
  rs_hhat_rows<LOGQ><<<(C::P + C::HRPC - 1) / C::HRPC, C::HROW_THREADS, sm1, st>>>(
      ny, nx, offx, offy, z, 1.0 / wavelength, k, work);
  XL_CHECK_LAUNCH("rs_hhat_rows");
  const size_t sm2 = (size_t)(C::P * (C::WH + 1) + 2 * C::WH * C::XS) * sizeof(float2);
  e = allow_smem(rs_hhat_cols<LOGQ>, sm2);
  if (e != cudaSuccess) return cuda_fail(e, "rs_hhat_cols smem");
  rs_hhat_cols<LOGQ><<<C::P / C::WH, C::HCOL_THREADS, sm2, st>>>(work, (float)scale, spec);
  XL_CHECK_LAUNCH("rs_hhat_cols");
  return XL_OK;
}

template <int LOGQ>
static int launch_stage(cudaStream_t st, const RsLaunch& p, int stage) {
  using C = RsCfg<LOGQ>;
  const dim3 g_rows((p.ny + C::RPC - 1) / C::RPC, p.B);
  cudaError_t e;
  if (stage == 0) {
    const size_t sm = (size_t)(C::RPC * p.cin * p.nx + C::RPC * C::XS + C::TWR) * sizeof(float2);
    if ((e = allow_smem(rs_rows_fwd<LOGQ>, sm)) != cudaSuccess) return cuda_fail(e, "rs_rows_fwd smem");
    rs_rows_fwd<LOGQ><<<g_rows, C::ROW_THREADS, sm, st>>>(p);
    XL_CHECK_LAUNCH("rs_rows_fwd");
  } else if (stage == 1) {
    const size_t sm = (size_t)(C::TBASE + (C::TMA ? p.ny * C::W + 1 : 0)) * sizeof(float2);
    if ((e = allow_smem(rs_cols_conv<LOGQ>, sm)) != cudaSuccess) return cuda_fail(e, "rs_cols_conv smem");
    rs_cols_conv<LOGQ><<<dim3(C::P / C::W, p.B), C::CONV_THREADS, sm, st>>>(p);
    XL_CHECK_LAUNCH("rs_cols_conv");
  } else {
    const bool stage_out = p.post.nops || (p.adjoint && p.cout == 3);
    const size_t sm = (size_t)(C::RPC * C::XS + C::TWR + C::RPC * C::Q +
                               (stage_out ? C::RPC * p.cout * p.nx : 0)) * sizeof(float2);
    if ((e = allow_smem(rs_rows_inv<LOGQ>, sm)) != cudaSuccess) return cuda_fail(e, "rs_rows_inv smem");
    rs_rows_inv<LOGQ><<<g_rows, C::ROW_THREADS, sm, st>>>(p);
    XL_CHECK_LAUNCH("rs_rows_inv");
  }
  return XL_OK;
}

template <int LOGQ>
static int launch_propagate(cudaStream_t st, const RsLaunch& p, int stage) {
  if (stage >= 0) return launch_stage<LOGQ>(st, p, stage);
  for (int s = 0; s < 3; ++s)
    if (int rc = launch_stage<LOGQ>(st, p, s)) return rc;
  return XL_OK;
}

#define XL_RS_DISPATCH(LOGQ_VAR, CALL)          \
  switch (LOGQ_VAR) {                           \
    case 4: return CALL(4);                     \
    case 5: return CALL(5);                     \
    case 6: return CALL(6);                     \
    case 7: return CALL(7);                     \
    case 8: return CALL(8);                     \
    case 9: return CALL(9);                     \
    case 10: return CALL(10);                   \
    case 11: return CALL(11);                   \
    case 12: return CALL(12);                   \
    default: break;                             \
  }

cudaError_t rs_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

}  // namespace xl

using namespace xl;

extern "C" int xl_device_timeouts(unsigned int* count, int reset) {
  if (!count) {
    set_error("xl_device_timeouts: null output");
    return XL_EINVAL;
  }
  cudaError_t e = cudaMemcpyFromSymbol(count, g_rs_timeouts, sizeof(unsigned int));
  if (e != cudaSuccess) return cuda_fail(e, "xl_device_timeouts");
  if (reset) {
    const unsigned int zero = 0;
    e = cudaMemcpyToSymbol(g_rs_timeouts, &zero, sizeof(unsigned int));
    if (e != cudaSuccess) return cuda_fail(e, "xl_device_timeouts reset");
  }
  return XL_OK;
}

extern "C" size_t xl_rs_spectrum_bytes(int ny, int nx) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE) return 0;
  const size_t P = (size_t)2 << rs_logq(ny, nx);
  return P * P * sizeof(float2);
}

extern "C" size_t xl_rs_spectrum_work_bytes(int ny, int nx) { return xl_rs_spectrum_bytes(ny, nx); }

extern "C" size_t xl_rs_work_bytes(int batch, int comps, int ny, int nx) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE || batch < 1 || comps < 1) return 0;
  const size_t P = (size_t)2 << rs_logq(ny, nx);
  return (size_t)batch * comps * ny * P * sizeof(float2);
}

extern "C" int xl_rs_transfer_spectrum(void* stream, int ny, int nx, const double* offx,
                                       const double* offy, double z, double wavelength,
                                       double scale, void* spectrum, void* work) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE) {
    set_error("xl_rs_transfer_spectrum: field side out of range (2..%d): %d x %d", XL_MAX_SIDE, ny, nx);
    return XL_EINVAL;
  }
  if (!offx || !offy || !spectrum || !work) {
    set_error("xl_rs_transfer_spectrum: null pointer argument");
    return XL_EINVAL;
  }
  if (!(z != 0.0) || !(wavelength > 0.0)) {
    set_error("xl_rs_transfer_spectrum: need z != 0 and wavelength > 0 (got z=%g, wavelength=%g)", z,
              wavelength);
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int lq = rs_logq(ny, nx);
#define CALL(L) launch_spectrum<L>(st, ny, nx, offx, offy, z, wavelength, scale, (float2*)spectrum, \
                                   (float2*)work)
  XL_RS_DISPATCH(lq, CALL)
#undef CALL
  set_error("xl_rs_transfer_spectrum: unsupported size");
  return XL_EUNSUPPORTED;
}

static int rs_run(void* stream, const XlRsArgs* a, int stage) {
  if (!a) {
    set_error("xl_rs_propagate: null args");
    return XL_EINVAL;
  }
  if (a->ny < 2 || a->nx < 2 || a->ny > XL_MAX_SIDE || a->nx > XL_MAX_SIDE || a->batch < 1) {
    set_error("xl_rs_propagate: bad shape batch=%d ny=%d nx=%d", a->batch, a->ny, a->nx);
    return XL_EINVAL;
  }
  const bool scalar = a->comps_in == 1 && a->comps_out == 1;
  const bool vector = a->adjoint ? (a->comps_in == 3 && a->comps_out == 3)
                                 : (a->comps_in == 2 && a->comps_out == 3);
  if (!scalar && !vector) {
    set_error("xl_rs_propagate: comps_in/comps_out must be 1/1 (RS), 2/3 (VRS) or 3/3 (VRS adjoint), "
              "got %d/%d (adjoint=%d)", a->comps_in, a->comps_out, a->adjoint);
    return XL_EINVAL;
  }
  if (a->adjoint && (a->pre.nops || a->post.nops)) {
    set_error("xl_rs_propagate: the adjoint takes no fused programs");
    return XL_EINVAL;
  }
  const int nout = (a->adjoint && vector) ? 2 : a->comps_out;
  for (int c = 0; c < a->comps_in; ++c)
    if (!a->in[c]) { set_error("xl_rs_propagate: null input plane %d", c); return XL_EINVAL; }
  for (int c = 0; c < nout; ++c)
    if (!a->out[c]) { set_error("xl_rs_propagate: null output plane %d", c); return XL_EINVAL; }
  if (!a->spectrum || !a->work) {
    set_error("xl_rs_propagate: null spectrum or workspace");
    return XL_EINVAL;
  }
  if (vector && (!a->x || !a->y || !a->z)) {
    set_error("xl_rs_propagate: VRS needs x, y and z arrays");
    return XL_EINVAL;
  }
  if (a->pre.nops < 0 || a->pre.nops > XL_MAX_OPS || a->post.nops < 0 || a->post.nops > XL_MAX_OPS) {
    set_error("xl_rs_propagate: op program too long");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  RsLaunch p;
  p.B = a->batch; p.cin = a->comps_in; p.cout = a->comps_out; p.ny = a->ny; p.nx = a->nx;
  for (int c = 0; c < 3; ++c) {
    p.in[c] = (const float2*)a->in[c];
    p.out[c] = (float2*)a->out[c];
  }
  p.ibs = a->in_bstride; p.obs = a->out_bstride;
  p.x = a->x; p.y = a->y; p.z = a->z;
  p.spec = (const float2*)a->spectrum; p.sstride = a->spectrum_stride; p.sidx = a->spectrum_index;
  p.work = (float2*)a->work;
  p.pre = a->pre; p.post = a->post;
  p.adjoint = a->adjoint ? 1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  const int lq = rs_logq(a->ny, a->nx);
#define CALL(L) launch_propagate<L>(st, p, stage)
  XL_RS_DISPATCH(lq, CALL)
#undef CALL
  set_error("xl_rs_propagate: unsupported size");
  return XL_EUNSUPPORTED;
}

extern "C" int xl_rs_propagate(void* stream, const XlRsArgs* a) { return rs_run(stream, a, -1); }

extern "C" int xl_rs_stage(void* stream, const XlRsArgs* a, int stage) {
  if (stage < 0 || stage > 2) {
    set_error("xl_rs_stage: stage must be 0, 1 or 2 (got %d)", stage);
    return XL_EINVAL;
  }
  return rs_run(stream, a, stage);
}

// ---------------------------------------------------------------------------
// Allocation-free RS / VRS.
//
// Some callers of this library cannot call cudaMalloc.  Two examples: a host
// program that reserves all device memory for its own pool at start-up (a
// later cudaMalloc fails or fragments the pool), and a loop that drives
// optical hardware frame by frame, which cannot take the implicit device
// synchronisation and unbounded latency that cudaMalloc / cudaFree can cause.
// xl_rs_propagate_noalloc serves them.  It runs exactly the passes of
// xl_rs_propagate, but its workspace is the fixed device array below, so the
// caller passes only inputs (fields, transfer spectrum, coordinates) and
// outputs, and the call allocates no device memory.
//
// The array holds XL_RS_NOALLOC_MAX_WORK_BYTES on every GPU that loads the
// library, until the process exits.  All calls share it and it keeps the last
// call's contents; nothing in it needs clearing, because the first pass writes
// every element the later passes read.  Calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array.
static __device__ __align__(256) float2 g_rs_noalloc_scratch[XL_RS_NOALLOC_MAX_WORK_BYTES / sizeof(float2)];

static std::mutex g_noalloc_mu;
static float2* g_noalloc_ptr[256];

// Device address of the scratch array for the current device.  The array's
// name in host code is only a stand-in for the symbol, so the address is
// looked up once per device, with that device current.
static int noalloc_scratch(float2** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "xl_rs_propagate_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= 256) {
    set_error("xl_rs_propagate_noalloc: device index %d out of range", dev);
    return XL_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_rs_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "xl_rs_propagate_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = (float2*)p;
  }
  *out = g_noalloc_ptr[dev];
  return XL_OK;
}

extern "C" int xl_rs_propagate_noalloc(void* stream, const XlRsArgs* a) {
  if (!a) {
    set_error("xl_rs_propagate_noalloc: null args");
    return XL_EINVAL;
  }
  const size_t need = xl_rs_work_bytes(a->batch, a->comps_out, a->ny, a->nx);
  if (need == 0) {
    set_error("xl_rs_propagate_noalloc: bad shape batch=%d comps_out=%d ny=%d nx=%d", a->batch,
              a->comps_out, a->ny, a->nx);
    return XL_EINVAL;
  }
  if (need > (size_t)XL_RS_NOALLOC_MAX_WORK_BYTES) {
    set_error("xl_rs_propagate_noalloc: this call needs %zu bytes of scratch, the fixed limit is %llu "
              "(e.g. one 1024x1024 VRS field or one 2048x2048 scalar field); use xl_rs_propagate with a "
              "caller workspace for larger work",
              need, (unsigned long long)XL_RS_NOALLOC_MAX_WORK_BYTES);
    return XL_EINVAL;
  }
  float2* scratch = nullptr;
  if (int rc = noalloc_scratch(&scratch)) return rc;
  XlRsArgs b = *a;
  b.work = scratch;
  return rs_run(stream, &b, -1);
}
