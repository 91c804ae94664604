// Chirp-z (Bluestein) propagation for sm_103a: scalar CZT, vectorial VCZT and
// the high-NA objective-lens focus.
//
// The reference (wave_optics.py:333-460) runs Bluestein's algorithm along y
// and then along x, each as: multiply the input column by a pre-chirp,
// zero-pad to L = next_pow2(m+M-1), FFT, multiply by the spectrum of the
// inverse chirp, inverse FFT, keep entries [m, m+M) and multiply by a
// post-chirp.  The 2-D transform is separable, so here the x transform runs
// first over contiguous rows (czt_rows) and the y transform second over
// column tiles (czt_cols).  Each length-L transform is split into two
// Q-point chains (Q = L/2): even frequencies of (x[n] + x[n+Q]) and odd
// frequencies of (x[n] - x[n+Q]) w_L^n.
//
// Fused into czt_rows: the Jones program (masks, high-NA lens), the VCZT
// Ez = (Ex X/r + Ey Y/r) z/r, and the input-plane transfer function F.
// Fused into czt_cols: the output-plane transfer function F0 and the
// constant factor (z dx dy lambda, or -i sin^2(theta_max)/(f lambda)).
// Chirp vectors are computed in float64 on the host, as the reference does.
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace xl {

struct CztLaunch {
  int B, cin, cout, ny, nx, my, mx;  // input plane ny x nx, output plane my x mx
  int mode;                          // XL_CZT_SCALAR / XL_CZT_VECTOR / XL_CZT_PLAIN
  int adjoint;                       // transpose-conjugate of the forward transform
  int ioff_x, ooff_x, ioff_y, ooff_y;  // where the input / output lines sit in the length-L line
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
  float2* work;          // B x cout x ny x mx
  XlProg pre;
};

template <int LOGQ> struct CztCfg {
  using S = FftShape<LOGQ>;
  static constexpr int Q = S::N;
  static constexpr int T = S::T;
  static constexpr int XS = S::SMEM;
  static constexpr int RPC = (256 / (2 * T)) > 1 ? (256 / (2 * T)) : 1;
  static constexpr int W = (256 / T) < 1 ? 1 : ((256 / T) > 32 ? 32 : (256 / T));
  static constexpr int ROW_THREADS = 2 * RPC * T;
  static constexpr int COL_THREADS = 2 * W * T;
};

// One Bluestein chain pair on registers: v holds the parity-`par` input
// a_par[n], n = j + m*T.  On return the group's exchange buffer holds
// Ye[i] (par 0) or w_L^{-i} Yo[i] (par 1) at smpad(i).
template <int LOGQ>
__device__ __forceinline__ void bluestein_chain(float2 (&v)[16], int j, int par, float2* xb,
                                                const float2* __restrict__ g) {
  using C = CztCfg<LOGQ>;
  const float2* twQ = tw_table(LOGQ);
  const float2* twL = tw_table(LOGQ + 1);
  block_fft<LOGQ, 16, -1>(v, j, xb, twQ);
  const float2* gp = g + par * C::Q;
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], gp[j + m * C::T]);
  block_fft<LOGQ, 16, 1>(v, j, xb, twQ);
  // block_fft ends with all gathers done; the buffer may be overwritten.
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int i = j + m * C::T;
    xb[smpad(i)] = par ? cmulc(v[m], twL[i]) : v[m];
  }
}

// Chain input for parity `par`: the length-L line holds src[i] * pre[i] at
// position off + i (i < m) and zeros elsewhere; a_par[n] = (x[n] +- x[n+Q]) w_L^(par n).
template <int LOGQ>
__device__ __forceinline__ void bluestein_load(float2 (&v)[16], int j, int par, const float2* src,
                                               int stride, int m, int off, const float2* __restrict__ pre) {
  using C = CztCfg<LOGQ>;
  const float2* twL = tw_table(LOGQ + 1);
#pragma unroll
  for (int mm = 0; mm < 16; ++mm) {
    const int n = j + mm * C::T;
    const int i1 = n - off, i2 = n + C::Q - off;
    const float2 a = (i1 >= 0 && i1 < m) ? cmul(src[i1 * stride], pre[i1]) : make_float2(0.f, 0.f);
    const float2 b = (i2 >= 0 && i2 < m) ? cmul(src[i2 * stride], pre[i2]) : make_float2(0.f, 0.f);
    v[mm] = par ? cmul(csub(a, b), twL[n]) : cadd(a, b);
  }
}

// x transform over contiguous rows, with the prologue.
template <int LOGQ>
__global__ void __launch_bounds__(CztCfg<LOGQ>::ROW_THREADS) czt_rows(const CztLaunch p) {
  using C = CztCfg<LOGQ>;
  extern __shared__ float2 smem[];
  const int nc = p.cout;
  float2* stage = smem;                          // RPC x nc x nx
  float2* xch = smem + C::RPC * nc * p.nx;       // 2 RPC x XS
  const int tid = threadIdx.x;
  const int slot = tid / (2 * C::T);
  const int par = (tid / C::T) & 1;
  const int j = tid % C::T;
  const int b = blockIdx.y;
  const int r0 = blockIdx.x * C::RPC;
  const float zf = (float)p.z;

  for (int idx = tid; idx < C::RPC * p.nx; idx += blockDim.x) {
    const int s = idx / p.nx, n = idx % p.nx, r = r0 + s;
    if (r >= p.ny) continue;
    const long long off = (long long)b * p.ibs + (long long)r * p.nx + n;
    float2 e[3];
    e[0] = p.in[0][off];
    e[1] = p.cin > 1 ? p.in[1][off] : make_float2(0.f, 0.f);
    e[2] = make_float2(0.f, 0.f);
    if (p.cin > 2) e[2] = p.in[2][off];
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
  float2* xb = xch + (2 * slot + par) * C::XS;
  const float2* xe = xch + (2 * slot) * C::XS;
  const float2* xo = xch + (2 * slot + 1) * C::XS;
  for (int c = 0; c < nc; ++c) {
    float2 v[16];
    bluestein_load<LOGQ>(v, j, par, stage + (slot * nc + c) * p.nx, 1, r < p.ny ? p.nx : 0, p.ioff_x,
                         p.pre_x);
    bluestein_chain<LOGQ>(v, j, par, xb, p.g_x);
    __syncthreads();
    if (r < p.ny) {
      float2* dst = p.work + (((long long)b * nc + c) * p.ny + r) * p.mx;
      for (int o = par * C::T + j; o < p.mx; o += 2 * C::T) {
        const int n2 = p.ooff_x + o;
        const int i = n2 & (C::Q - 1);
        const float2 t = (n2 >> LOGQ) & 1 ? csub(xe[smpad(i)], xo[smpad(i)]) : cadd(xe[smpad(i)], xo[smpad(i)]);
        dst[o] = cmul(t, p.post_x[o]);
      }
    }
    __syncthreads();
  }
}

// y transform over tiles of W columns, with the epilogue.
template <int LOGQ>
__global__ void __launch_bounds__(CztCfg<LOGQ>::COL_THREADS) czt_cols(const CztLaunch p) {
  using C = CztCfg<LOGQ>;
  constexpr int W = C::W, PITCH = C::W + 1;
  extern __shared__ float2 smem[];
  const int rows = p.ny > p.my ? p.ny : p.my;
  float2* tile = smem;                   // rows x PITCH
  float2* xch = smem + rows * PITCH;     // 2W x XS
  const int tid = threadIdx.x;
  const int w = tid / (2 * C::T);
  const int par = (tid / C::T) & 1;
  const int j = tid % C::T;
  const int b = blockIdx.y;
  const int c0 = blockIdx.x * W;
  const int nc = p.cout;
  float2* xb = xch + (2 * w + par) * C::XS;

  for (int c = 0; c < nc; ++c) {
    const float2* plane = p.work + ((long long)b * nc + c) * p.ny * p.mx;
    for (int idx = tid; idx < p.ny * W; idx += blockDim.x) {
      const int r = idx / W, ww = idx % W;
      tile[r * PITCH + ww] = (c0 + ww < p.mx) ? plane[(long long)r * p.mx + c0 + ww] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 v[16];
    bluestein_load<LOGQ>(v, j, par, tile + w, PITCH, p.ny, p.ioff_y, p.pre_y);
    bluestein_chain<LOGQ>(v, j, par, xb, p.g_y);
    __syncthreads();
    // combine: output rows o in [0, my) of the W columns, into the tile
    for (int idx = tid; idx < p.my * W; idx += blockDim.x) {
      const int o = idx / W, ww = idx % W;
      const float2* e0 = xch + (2 * ww) * C::XS;
      const float2* e1 = xch + (2 * ww + 1) * C::XS;
      const int n2 = p.ooff_y + o;
      const int i = n2 & (C::Q - 1);
      float2 t = (n2 >> LOGQ) & 1 ? csub(e0[smpad(i)], e1[smpad(i)]) : cadd(e0[smpad(i)], e1[smpad(i)]);
      t = cmul(t, p.post_y[o]);
      const int col = c0 + ww;
      if (p.mode != XL_CZT_PLAIN && col < p.mx) {  // wave_optics.py:340, 355: F0 * U (adjoint: conj F)
        const float2 F = rs_kernel_value(p.xo[col], p.yo[o], p.z, p.inv_lambda, p.k);
        t = p.adjoint ? cmulc(t, F) : cmul(t, F);
      }
      tile[o * PITCH + ww] = cmul(t, p.cte);
    }
    __syncthreads();
    const bool fold = p.adjoint && p.mode == XL_CZT_VECTOR;
    for (int idx = tid; idx < p.my * W; idx += blockDim.x) {
      const int o = idx / W, ww = idx % W;
      const int col = c0 + ww;
      if (col >= p.mx) continue;
      const long long pix = (long long)b * p.obs + (long long)o * p.mx + col;
      if (fold && c == 2) {  // adjoint of Ez = (Ex X/r + Ey Y/r) z/r, vectorized_optics.py:341-344
        const float zf = (float)p.z;
        const float X = (float)p.xo[col], Y = (float)p.yo[o];
        const float r2 = X * X + Y * Y + zf * zf;
        const float2 gz = tile[o * PITCH + ww];
        p.out[0][pix] = cadd(p.out[0][pix], cscale(gz, X * zf / r2));
        p.out[1][pix] = cadd(p.out[1][pix], cscale(gz, Y * zf / r2));
      } else {
        p.out[c][pix] = tile[o * PITCH + ww];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------

template <int LOGQ>
static int launch_rows(cudaStream_t st, const CztLaunch& p) {
  using C = CztCfg<LOGQ>;
  const size_t sm = (size_t)(C::RPC * p.cout * p.nx + 2 * C::RPC * C::XS) * sizeof(float2);
  if (sm > 227 * 1024) {
    set_error("czt: input row too long for shared memory (%zu bytes)", sm);
    return XL_EUNSUPPORTED;
  }
  cudaError_t e = allow_smem(czt_rows<LOGQ>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "czt_rows smem");
  czt_rows<LOGQ><<<dim3((p.ny + C::RPC - 1) / C::RPC, p.B), C::ROW_THREADS, sm, st>>>(p);
  XL_CHECK_LAUNCH("czt_rows");
  return XL_OK;
}

template <int LOGQ>
static int launch_cols(cudaStream_t st, const CztLaunch& p) {
  using C = CztCfg<LOGQ>;
  const int rows = p.ny > p.my ? p.ny : p.my;
  const size_t sm = (size_t)(rows * (C::W + 1) + 2 * C::W * C::XS) * sizeof(float2);
  if (sm > 227 * 1024) {
    set_error("czt: column tile too large for shared memory (%zu bytes)", sm);
    return XL_EUNSUPPORTED;
  }
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

static int dispatch_rows(cudaStream_t st, const CztLaunch& p, int lq) {
  XL_CZT_DISPATCH(lq, launch_rows, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", lq + 1);
  return XL_EUNSUPPORTED;
}

static int dispatch_cols(cudaStream_t st, const CztLaunch& p, int lq) {
  XL_CZT_DISPATCH(lq, launch_cols, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", lq + 1);
  return XL_EUNSUPPORTED;
}

cudaError_t czt_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

}  // namespace xl

using namespace xl;

extern "C" size_t xl_czt_work_bytes(int batch, int comps, int ny, int mx) {
  if (batch < 1 || comps < 1 || ny < 1 || mx < 1) return 0;
  return (size_t)batch * comps * ny * mx * sizeof(float2);
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
    if (int rc = dispatch_rows(st, p, lqx)) return rc;
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
