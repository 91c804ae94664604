// Chirp-z (Bluestein) propagation for sm_103a: scalar CZT, vectorial VCZT and
// the high-NA objective-lens focus, forward and adjoint.
//
// The reference (wave_optics.py:333-460) runs Bluestein's algorithm along y
// and then along x, each as: multiply the input line by a pre-chirp,
// zero-pad to L = next_pow2(m+M-1), FFT, multiply by the spectrum of the
// inverse chirp, inverse FFT, keep entries [m, m+M) and multiply by a
// post-chirp.  The 2-D transform is separable, so here the x transform runs
// first over contiguous rows (czt_rows) and the y transform second over
// column tiles (czt_cols).  Each length-L transform is split into two
// Q-point chains (Q = L/2): even frequencies of (x[n] + x[n+Q]) and odd
// frequencies of (x[n] - x[n+Q]) w_L^n; one thread group runs both chains of
// a line, keeping the even result in shared memory, and combines them in
// registers for the output window.
//
// Fused into czt_rows: the Jones program (masks, high-NA lens), the VCZT
// Ez = (Ex X/r + Ey Y/r) z/r, and the input-plane transfer function F.
// Fused into czt_cols: the output-plane transfer function F0, the constant
// factor (z dx dy lambda, or -i sin^2(theta_max)/(f lambda)) and, for the
// VCZT adjoint, the fold of the Ez gradient into Ex, Ey.
// The intermediate (after the x transform) is stored in column tiles of W:
// element (row r, column l) at ((l / W) ny + r) W + l % W, planes of
// ny x mxp (mx rounded up to W).
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace xl {

struct CztLaunch {
  int B, cin, cout, ny, nx, my, mx, mxp;  // input plane ny x nx, output plane my x mx
  int mode;                               // XL_CZT_SCALAR / XL_CZT_VECTOR / XL_CZT_PLAIN
  int adjoint;                            // conjugate transpose of the forward transform
  int ioff_x, ooff_x, ioff_y, ooff_y;     // where input / output lines sit in the length-L line
  const float2* in[3];
  long long ibs;
  float2* out[3];
  long long obs;
  const double* x;
  const double* y;
  const double* xo;
  const double* yo;
  double z, inv_lambda;
  float k;
  float2 cte;
  const float2* pre_x;   // nx
  const float2* g_x;     // Lx, parity-split
  const float2* post_x;  // mx (includes 1/Lx)
  const float2* pre_y;   // ny
  const float2* g_y;     // Ly, parity-split
  const float2* post_y;  // my (includes 1/Ly)
  float2* work;          // B x cout x ny x mxp, column tiles of W
  XlProg pre;
};

#ifndef XL_CZT_ROW_E
#define XL_CZT_ROW_E 8
#endif

// Column-tile width of the intermediate, set by the y transform's length.
__host__ __device__ constexpr int czt_tile_w(int logqy) {
  return logqy >= 12 ? 2 : ((32 / ((1 << logqy) / 16)) > 4 ? (32 / ((1 << logqy) / 16)) : 4);
}

template <int LOGQ> struct CztCfg {
  static constexpr int Q = 1 << LOGQ;
  static constexpr int XS = Q + Q / 16;
  // x transform: one group of TR threads (ER elements) per row
  static constexpr int ER = XL_CZT_ROW_E;
  static constexpr int TR = Q / ER;
  static constexpr int TWR = FftTw<LOGQ, ER>::SIZE;
  static constexpr int RPC = (128 / TR) > 1 ? (128 / TR) : 1;
  static constexpr int ROW_THREADS = RPC * TR;
  static constexpr int ROW_MINB = (768 / ROW_THREADS) > 1 ? (768 / ROW_THREADS) : 1;
  // y transform: W groups of TC threads (16 elements), lanes interleaved over W columns
  static constexpr int EC = 16;
  static constexpr int TC = Q / EC;
  static constexpr int TWC = FftTw<LOGQ, EC>::SIZE;
  static constexpr int W = czt_tile_w(LOGQ);
  static constexpr int COL_THREADS = W * TC;
  static constexpr int CPAD = W >= 8 ? 0 : 4;
  static constexpr int CXS = XS + CPAD;
  static constexpr int CYS = Q + CPAD;
};

__device__ __forceinline__ long long tile_idx(int r, int l, int rows, int W) {
  return ((long long)(l / W) * rows + r) * W + (l % W);
}

template <int LOGQ, int E>
__device__ __forceinline__ void fill_czt_twiddles(float2* stw) {
  const float2* twQ = tw_table(LOGQ);
  for (int idx = threadIdx.x; idx < FftTw<LOGQ, E>::SIZE; idx += blockDim.x)
    stw[idx] = pass_twiddle_entry<LOGQ, E>(idx, twQ);
}

// Chain input for parity `par` at the thread's positions n = j + e T: the
// length-L line holds src(i) * pre[i] at position off + i (i < m);
// a_par[n] = (x[n] + (-1)^par x[n+Q]) w_L^(par n).
template <int LOGQ, int E, int T, class Src>
__device__ __forceinline__ void chain_load(float2 (&v)[E], int j, int par, const Src& src, int m, int off,
                                           const float2* __restrict__ pre) {
  const float2* twL = tw_table(LOGQ + 1);
  constexpr int Q = 1 << LOGQ;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int n = j + e * T;
    const int i1 = n - off, i2 = n + Q - off;
    const float2 a = (i1 >= 0 && i1 < m) ? cmul(src(i1), __ldg(pre + i1)) : make_float2(0.f, 0.f);
    const float2 b = (i2 >= 0 && i2 < m) ? cmul(src(i2), __ldg(pre + i2)) : make_float2(0.f, 0.f);
    v[e] = par ? cmul(csub(a, b), twL[n]) : cadd(a, b);
  }
}

// x transform over contiguous rows, with the prologue.
template <int LOGQ>
__global__ void __launch_bounds__(CztCfg<LOGQ>::ROW_THREADS, CztCfg<LOGQ>::ROW_MINB)
    czt_rows(const CztLaunch p, int wt) {
  using C = CztCfg<LOGQ>;
  constexpr int E = C::ER, T = C::TR;
  extern __shared__ float2 smem[];
  const int nc = p.cout;
  float2* stage = smem;                          // RPC x nc x nx
  float2* xch = stage + C::RPC * nc * p.nx;      // RPC x XS
  float2* stw = xch + C::RPC * C::XS;            // TWR
  float2* yb = stw + C::TWR;                     // RPC x Q
  const int tid = threadIdx.x;
  const int slot = tid / T;
  const int j = tid % T;
  const int b = blockIdx.y;
  const int r0 = blockIdx.x * C::RPC;
  const float zf = (float)p.z;
  fill_czt_twiddles<LOGQ, E>(stw);

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
    if (p.mode != XL_CZT_PLAIN) {
      if (p.mode == XL_CZT_VECTOR && !p.adjoint) {  // vectorized_optics.py:340-344
        const float X = (float)p.x[n], Y = (float)p.y[r];
        const float rr = sqrtf(X * X + Y * Y + zf * zf);
        e[2] = cscale(cadd(cscale(e[0], X / rr), cscale(e[1], Y / rr)), zf / rr);
      }
      // wave_optics.py:341 (F on the input plane); the adjoint applies conj(F0) here
      float2 F = rs_kernel_value(p.x[n], p.y[r], p.z, p.inv_lambda, p.k);
      if (p.adjoint) F = cconj(F);
      e[0] = cmul(e[0], F);
      e[1] = cmul(e[1], F);
      e[2] = cmul(e[2], F);
    }
    stage[(s * nc) * p.nx + n] = e[0];
    if (nc > 1) stage[(s * nc + 1) * p.nx + n] = e[1];
    if (nc > 2) stage[(s * nc + 2) * p.nx + n] = e[2];
  }
  __syncthreads();

  const int r = r0 + slot;
  const bool live = r < p.ny;
  const float2* twL = tw_table(LOGQ + 1);
  float2* xb = xch + slot * C::XS;
  float2* y0 = yb + slot * C::Q;
  for (int c = 0; c < nc; ++c) {
    const float2* src = stage + (slot * nc + c) * p.nx;
    auto rd = [src](int i) { return src[i]; };
    float2* plane = p.work + ((long long)b * nc + c) * p.ny * p.mxp;
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      float2 v[E];
      chain_load<LOGQ, E, T>(v, j, par, rd, live ? p.nx : 0, p.ioff_x, p.pre_x);
      block_fft_s<LOGQ, E, -1>(v, j, xb, stw);
      const float2* gp = p.g_x + par * C::Q;
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = cmul(v[e], __ldg(gp + j + e * T));
      block_fft_s<LOGQ, E, 1>(v, j, xb, stw);
      if (par == 0) {
#pragma unroll
        for (int e = 0; e < E; ++e) y0[j + e * T] = v[e];
      } else if (live) {
        // output window [ooff, ooff + mx) of the length-L line: indices i and i + Q
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int i = j + e * T;
          const float2 yo = cmulc(v[e], twL[i]);
          const float2 ye = y0[i];
          const int o1 = i - p.ooff_x, o2 = i + C::Q - p.ooff_x;
          if (o1 >= 0 && o1 < p.mx) plane[tile_idx(r, o1, p.ny, wt)] = cmul(cadd(ye, yo), __ldg(p.post_x + o1));
          if (o2 >= 0 && o2 < p.mx) plane[tile_idx(r, o2, p.ny, wt)] = cmul(csub(ye, yo), __ldg(p.post_x + o2));
        }
      }
    }
  }
}

// y transform over tiles of W columns, with the epilogue.  Lanes interleave
// the W columns of a tile, so every warp load of the intermediate is one
// contiguous run.
template <int LOGQ>
__global__ void __launch_bounds__(CztCfg<LOGQ>::COL_THREADS) czt_cols(const CztLaunch p) {
  using C = CztCfg<LOGQ>;
  constexpr int W = C::W, LPW = 32 / W, E = C::EC, T = C::TC;
  extern __shared__ float2 smem[];
  float2* xch = smem;                  // W x CXS
  float2* stw = smem + W * C::CXS;     // TWC
  float2* yb = stw + C::TWC;           // W x CYS
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int w = lane % W;
  const int j = (tid >> 5) * LPW + lane / W;
  const int t = blockIdx.x;
  const int b = blockIdx.y;
  const int col = t * W + w;
  const bool live = col < p.mx;
  fill_czt_twiddles<LOGQ, E>(stw);
  __syncthreads();
  const float2* twL = tw_table(LOGQ + 1);
  float2* xb = xch + w * C::CXS;
  float2* y0 = yb + w * C::CYS;
  const bool fold = p.adjoint && p.mode == XL_CZT_VECTOR;
  const float zf = (float)p.z;

  for (int c = 0; c < p.cout; ++c) {
    const float2* tileT = p.work + ((long long)b * p.cout + c) * p.ny * p.mxp + (long long)t * p.ny * W + w;
    auto rd = [tileT](int i) { return tileT[(long long)i * W]; };
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      float2 v[E];
      chain_load<LOGQ, E, T>(v, j, par, rd, live ? p.ny : 0, p.ioff_y, p.pre_y);
      block_fft_s<LOGQ, E, -1>(v, j, xb, stw);
      const float2* gp = p.g_y + par * C::Q;
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = cmul(v[e], __ldg(gp + j + e * T));
      block_fft_s<LOGQ, E, 1>(v, j, xb, stw);
      if (par == 0) {
#pragma unroll
        for (int e = 0; e < E; ++e) y0[j + e * T] = v[e];
      } else if (live) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int i = j + e * T;
          const float2 yo = cmulc(v[e], twL[i]);
          const float2 ye = y0[i];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int o = i + h * C::Q - p.ooff_y;
            if (o < 0 || o >= p.my) continue;
            float2 val = cmul(h ? csub(ye, yo) : cadd(ye, yo), __ldg(p.post_y + o));
            if (p.mode != XL_CZT_PLAIN) {  // wave_optics.py:340, 355: F0 * U (adjoint: conj F)
              const float2 F = rs_kernel_value(p.xo[col], p.yo[o], p.z, p.inv_lambda, p.k);
              val = p.adjoint ? cmulc(val, F) : cmul(val, F);
            }
            val = cmul(val, p.cte);
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
  }
}

// ---------------------------------------------------------------------------

template <int LOGQ>
static int launch_rows(cudaStream_t st, const CztLaunch& p, int wt) {
  using C = CztCfg<LOGQ>;
  const size_t sm = (size_t)(C::RPC * p.cout * p.nx + C::RPC * C::XS + C::TWR + C::RPC * C::Q) * sizeof(float2);
  if (sm > 227 * 1024) {
    set_error("czt: input row too long for shared memory (%zu bytes)", sm);
    return XL_EUNSUPPORTED;
  }
  cudaError_t e = allow_smem(czt_rows<LOGQ>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "czt_rows smem");
  czt_rows<LOGQ><<<dim3((p.ny + C::RPC - 1) / C::RPC, p.B), C::ROW_THREADS, sm, st>>>(p, wt);
  XL_CHECK_LAUNCH("czt_rows");
  return XL_OK;
}

template <int LOGQ>
static int launch_cols(cudaStream_t st, const CztLaunch& p) {
  using C = CztCfg<LOGQ>;
  const size_t sm = (size_t)(C::W * C::CXS + C::TWC + C::W * C::CYS) * sizeof(float2);
  cudaError_t e = allow_smem(czt_cols<LOGQ>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "czt_cols smem");
  czt_cols<LOGQ><<<dim3((p.mx + C::W - 1) / C::W, p.B), C::COL_THREADS, sm, st>>>(p);
  XL_CHECK_LAUNCH("czt_cols");
  return XL_OK;
}

#define XL_CZT_DISPATCH(LQ, FN, ...)          \
  switch (LQ) {                               \
    case 4: return FN<4>(__VA_ARGS__);        \
    case 5: return FN<5>(__VA_ARGS__);        \
    case 6: return FN<6>(__VA_ARGS__);        \
    case 7: return FN<7>(__VA_ARGS__);        \
    case 8: return FN<8>(__VA_ARGS__);        \
    case 9: return FN<9>(__VA_ARGS__);        \
    case 10: return FN<10>(__VA_ARGS__);      \
    case 11: return FN<11>(__VA_ARGS__);      \
    case 12: return FN<12>(__VA_ARGS__);      \
    default: break;                           \
  }

static int dispatch_rows(cudaStream_t st, const CztLaunch& p, int lq, int wt) {
  XL_CZT_DISPATCH(lq, launch_rows, st, p, wt)
  set_error("czt: unsupported Bluestein length 2^%d", lq + 1);
  return XL_EUNSUPPORTED;
}

static int dispatch_cols(cudaStream_t st, const CztLaunch& p, int lq) {
  XL_CZT_DISPATCH(lq, launch_cols, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", lq + 1);
  return XL_EUNSUPPORTED;
}

static cudaError_t czt_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

static const bool czt_registered = register_device_tables(&czt_upload_twiddles, nullptr);

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
  const int lqx = a->log2_lx - 1, lqy = a->log2_ly - 1;
  if (lqx < 4 || lqx > 12 || lqy < 4 || lqy > 12 || (1 << a->log2_lx) < a->nx + a->mx ||
      (1 << a->log2_ly) < a->ny + a->my) {
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
  const int wt = czt_tile_w(lqy);
  p.mxp = (a->mx + wt - 1) / wt * wt;
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
    if (int rc = dispatch_rows(st, p, lqx, wt)) return rc;
  if (stage < 0 || stage == 1)
    if (int rc = dispatch_cols(st, p, lqy)) return rc;
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
