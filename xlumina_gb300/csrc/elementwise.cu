// Stand-alone per-pixel kernels: a Jones program applied outside a
// propagator (masks whose result the caller reads directly).
#include <initializer_list>

#include "common.cuh"
#include "internal.h"

namespace xl {

struct ElemLaunch {
  int B, C, ny, nx;
  const float2* in[3];
  long long ibs;
  float2* out[3];
  long long obs;
  XlProg prog;
};

__global__ void apply_ops_kernel(const ElemLaunch p) {
  const long long npix = (long long)p.ny * p.nx;
  const int b = blockIdx.y;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    float2 e[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const long long off = (long long)b * p.ibs + i;
    e[0] = p.in[0][off];
    if (p.C > 1) e[1] = p.in[1][off];
    if (p.C > 2) e[2] = p.in[2][off];
    const int row = (int)((unsigned)i / (unsigned)p.nx), col = (int)i - row * p.nx;
    PixelCtx px{row, col, i, b};
    apply_prog(p.prog, e, px);
    const long long o = (long long)b * p.obs + i;
    p.out[0][o] = e[0];
    if (p.C > 1) p.out[1][o] = e[1];
    if (p.C > 2) p.out[2][o] = e[2];
  }
}

struct OpsBwdLaunch {
  int B, C, ny, nx;
  const float2* in[3];
  long long ibs;
  const float2* gout[3];
  long long gbs;
  float2* gin[3];
  long long ginbs;
  XlProg prog;
  void* pgrad[XL_MAX_OPS * 4];
};

// One thread per pixel and batch entry, or (when a per-pixel parameter shared
// by the whole batch needs its gradient) one thread per pixel looping over
// the batch, so that the batch sum runs in a fixed order.  The op loops are
// unrolled to KMAX so the per-op intermediates stay in registers.  Dynamic
// shared memory holds, [slot][thread] so that a warp's accesses fall in
// distinct banks: the scalar-parameter partial sums (when any scalar
// gradient is asked for), then the shared-plane batch sums (when needed).
//
// FK: the program's op kinds fixed at compile time (FixedKinds<...>, for the
// programs the tables run), so that the per-op switches fold and the trig
// stays in registers; FixedKinds<> reads them from the program.

template <int KMAX, class FK = FixedKinds<>>
__global__ void __launch_bounds__(128) ops_backward_kernel(const OpsBwdLaunch p, int scalar_acc, int plane_acc) {
  constexpr int NS = XL_MAX_OPS * 4;
  constexpr int NT = 128;
  constexpr bool FIXED = FK::n > 0;
  static_assert(!FIXED || FK::n == KMAX, "a fixed program unrolls to its length");
  extern __shared__ float accm[];
  // the trig of every op the forward recompute applies, for its backward
  // (thread-private slots, so no barrier): evaluated once per pixel and entry.
  // A fixed program keeps it in registers instead.
  __shared__ float4 trig_s[FIXED ? 1 : KMAX - 1][NT];
  float* acc_s = accm;                              // NS x NT, when scalar_acc
  float* acc_p = accm + (scalar_acc ? NS * NT : 0); // NS x NT, when plane_acc
  const long long npix = (long long)p.ny * p.nx;
  const int K = FIXED ? FK::n : p.prog.nops;
  auto kind = [&](int k) { return FIXED ? FK::at(k) : p.prog.ops[k].kind; };
  const int tid = threadIdx.x;
  const int b_lo = gridDim.y > 1 ? blockIdx.y : 0;
  const int b_hi = gridDim.y > 1 ? blockIdx.y + 1 : p.B;
  if (scalar_acc)
    for (int q = 0; q < NS; ++q) acc_s[q * NT + tid] = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const int row = (int)((unsigned)i / (unsigned)p.nx), col = (int)i - row * p.nx;
    if (plane_acc)
      for (int q = 0; q < 4 * K; ++q) acc_p[q * NT + tid] = 0.f;
    // the high-NA lens depends on the pixel only: its coefficients are hoisted out of the batch loop
    float kc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int hk = -1;
    {
      PixelCtx px0{row, col, i, 0};
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K && hk < 0 && (kind(k) == XL_OP_HIGHNA || kind(k) == XL_OP_HIGHNA_EZ)) {
          highna_coeffs(p.prog.ops[k], px0, kc);
          hk = k;
        }
    }
    for (int b = b_lo; b < b_hi; ++b) {
      PixelCtx px{row, col, i, b};
      float2 st[KMAX][3];
      float4 trig_r[KMAX];
      float2 e[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      const long long off = (long long)b * p.ibs + i;
      e[0] = p.in[0][off];
      if (p.C > 1 && p.in[1]) e[1] = p.in[1][off];
      if (p.C > 2 && p.in[2]) e[2] = p.in[2][off];
      // forward recompute: the input of every op (the last op's output is not needed)
#pragma unroll
      for (int k = 0; k < KMAX; ++k) {
        if (k < K) {
          st[k][0] = e[0]; st[k][1] = e[1]; st[k][2] = e[2];
          if (k + 1 < K) {
            if (k == hk) {
              if (kind(k) == XL_OP_HIGHNA) apply_highna(kc, e);
              else apply_highna_ez(kc, e);
            } else if (k < KMAX - 1) {
              const float4 t = op_trig(kind(k), p.prog.ops[k], px);
              if constexpr (FIXED) trig_r[k] = t;
              else trig_s[FIXED ? 0 : k][tid] = t;
              apply_op_t(kind(k), p.prog.ops[k], t, e, px);
            }
          }
        }
      }
      float2 g[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      const long long go = (long long)b * p.gbs + i;
      g[0] = p.gout[0][go];
      if (p.C > 1 && p.gout[1]) g[1] = p.gout[1][go];
      if (p.C > 2 && p.gout[2]) g[2] = p.gout[2][go];
#pragma unroll
      for (int k = KMAX - 1; k >= 0; --k) {
        if (k < K) {
          const XlOp& op = p.prog.ops[k];
          float pg[4] = {0.f, 0.f, 0.f, 0.f};
          const float2 ek[3] = {st[k][0], st[k][1], st[k][2]};
          if (k == hk) {
            if (kind(k) == XL_OP_HIGHNA) apply_highna_bwd(kc, g);
            else apply_highna_ez_bwd(kc, g);
          }
          else if (k + 1 < K && k < KMAX - 1)
            apply_op_bwd_t(kind(k), op, FIXED ? trig_r[k] : trig_s[FIXED ? 0 : k][tid], ek, g, px, pg);
          else apply_op_bwd(kind(k), op, ek, g, px, pg);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            void* dst = p.pgrad[k * 4 + q];
            if (!dst) continue;
            if (op.pmask & (1 << q)) {
              if (op.pbstride) ((float*)dst)[(long long)b * op.pbstride + i] = pg[q];
              else acc_p[(k * 4 + q) * NT + tid] += pg[q];
            } else {
              acc_s[(k * 4 + q) * NT + tid] += pg[q];
            }
          }
        }
      }
      const long long gi = (long long)b * p.ginbs + i;
      if (p.gin[0]) p.gin[0][gi] = g[0];
      if (p.C > 1 && p.gin[1]) p.gin[1][gi] = g[1];
      if (p.C > 2 && p.gin[2]) p.gin[2][gi] = g[2];
    }
    if (plane_acc)
      for (int k = 0; k < K; ++k)
        for (int q = 0; q < 4; ++q) {
          const XlOp& op = p.prog.ops[k];
          if (p.pgrad[k * 4 + q] && (op.pmask & (1 << q)) && !op.pbstride)
            ((float*)p.pgrad[k * 4 + q])[i] = acc_p[(k * 4 + q) * NT + tid];
        }
  }
  if (!scalar_acc) return;
  // scalar parameters: block reduction, one float64 atomic per block and slot
  __shared__ float red[8];
  const int lane = tid & 31, warp = tid >> 5;
  for (int k = 0; k < K; ++k)
    for (int q = 0; q < 4; ++q) {
      const XlOp& op = p.prog.ops[k];
      if (!p.pgrad[k * 4 + q] || (op.pmask & (1 << q))) continue;
      float v = acc_s[(k * 4 + q) * NT + tid];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp] = v;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd((double*)p.pgrad[k * 4 + q], t);
      }
      __syncthreads();
    }
}

__global__ void highna_plane_kernel(int ny, int nx, XlOp op, float* out) {
  const long long npix = (long long)ny * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const int row = (int)((unsigned)i / (unsigned)nx);
    PixelCtx px{row, (int)i - row * nx, i, 0};
    float kc[6];
    highna_coeffs(op, px, kc);
#pragma unroll
    for (int q = 0; q < 6; ++q) out[q * npix + i] = kc[q];
  }
}

// ---- intensity MSE (loss_functions.py:137-149) ----
// loss[p] = sum_i (|a_i|^2 - |b_i|^2)^2 / npix for plane p; the sum runs in two
// fixed-order stages (per-block float partials in float64, then per plane),
// so the result does not depend on scheduling.
constexpr int MSE_THREADS = 256;

// Per-plane reductions of a pixel function f(a_i, b_i): KIND 0 the intensity
// MSE term (|a|^2 - |b|^2)^2, KIND 1 the real inner product Re(conj(a) b),
// KIND 2 the amplitude term (|a| - |b|)^2, KIND 3 the phase term
// (arg a - arg b)^2 (loss_functions.py:109-135).
template <int KIND>
__global__ void __launch_bounds__(MSE_THREADS) plane_sum_partial(const float2* __restrict__ a, long long aps,
                                                                 const float2* __restrict__ b, long long bps,
                                                                 long long npix, double* __restrict__ partial) {
  const int plane = blockIdx.y;
  a += (long long)plane * aps;
  b += (long long)plane * bps;
  float acc = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 u = a[i], v = b[i];
    if (KIND == 0) {
      const float d = (u.x * u.x + u.y * u.y) - (v.x * v.x + v.y * v.y);
      acc = fmaf(d, d, acc);
    } else if (KIND == 1) {
      acc = fmaf(u.x, v.x, fmaf(u.y, v.y, acc));
    } else if (KIND == 2) {
      const float d = hypotf(u.x, u.y) - hypotf(v.x, v.y);
      acc = fmaf(d, d, acc);
    } else {
      const float d = atan2f(u.y, u.x) - atan2f(v.y, v.x);
      acc = fmaf(d, d, acc);
    }
  }
  __shared__ float red[MSE_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < MSE_THREADS / 32; ++w) t += red[w];
    partial[(long long)plane * gridDim.x + blockIdx.x] = t;
  }
}

// One warp per plane: lane l sums partials l, l + 32, ... in order, then a
// fixed shuffle tree (the same order on every call).
__global__ void mse_int_finish(const double* __restrict__ partial, int nblk, int planes, double inv_n,
                               float* __restrict__ out) {
  const int plane = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (plane >= planes) return;
  double t = 0.0;
  for (int k = lane; k < nblk; k += 32) t += partial[(long long)plane * nblk + k];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[plane] = (float)(t * inv_n);
}

// Gradients of loss[p] with upstream gradient g[p] (torch's convention for
// complex tensors, 2 dL/d conj): ga = 4 g (|a|^2 - |b|^2) a / npix and
// gb = -4 g (|a|^2 - |b|^2) b / npix (either may be NULL).
__global__ void mse_int_grad(const float2* __restrict__ a, long long aps, const float2* __restrict__ b,
                             long long bps, long long npix, const float* __restrict__ g, float four_inv_n,
                             float2* __restrict__ ga, float2* __restrict__ gb) {
  const int plane = blockIdx.y;
  a += (long long)plane * aps;
  b += (long long)plane * bps;
  const float s = g[plane] * four_inv_n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 u = a[i], v = b[i];
    const float d = s * ((u.x * u.x + u.y * u.y) - (v.x * v.x + v.y * v.y));
    if (ga) ga[(long long)plane * npix + i] = make_float2(d * u.x, d * u.y);
    if (gb) gb[(long long)plane * npix + i] = make_float2(-d * v.x, -d * v.y);
  }
}

// Gradients of the amplitude (KIND 2) and phase (KIND 3) MSE per plane with
// upstream gradient g[p] (torch's convention, 2 dL/d conj):
// amplitude: ga = 2 g (|a| - |b|) a / (|a| npix), gb = -2 g (|a| - |b|) b / (|b| npix);
// phase: ga = 2 g (arg a - arg b) i a / (|a|^2 npix), gb the same with -i b / |b|^2;
// zero where |a| (|b|) is zero, as torch's abs and angle give.
template <int KIND>
__global__ void amp_phase_grad(const float2* __restrict__ a, long long aps, const float2* __restrict__ b,
                               long long bps, long long npix, const float* __restrict__ g, float two_inv_n,
                               float2* __restrict__ ga, float2* __restrict__ gb) {
  const int plane = blockIdx.y;
  a += (long long)plane * aps;
  b += (long long)plane * bps;
  const float s = g[plane] * two_inv_n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 u = a[i], v = b[i];
    float2 ru, rv;
    if (KIND == 2) {
      const float au = hypotf(u.x, u.y), av = hypotf(v.x, v.y);
      const float d = s * (au - av);
      const float fu = au > 0.f ? d / au : 0.f, fv = av > 0.f ? -d / av : 0.f;
      ru = make_float2(fu * u.x, fu * u.y);
      rv = make_float2(fv * v.x, fv * v.y);
    } else {
      const float d = s * (atan2f(u.y, u.x) - atan2f(v.y, v.x));
      const float nu = u.x * u.x + u.y * u.y, nv = v.x * v.x + v.y * v.y;
      const float fu = nu > 0.f ? d / nu : 0.f, fv = nv > 0.f ? -d / nv : 0.f;
      ru = make_float2(-fu * u.y, fu * u.x);
      rv = make_float2(-fv * v.y, fv * v.x);
    }
    if (ga) ga[(long long)plane * npix + i] = ru;
    if (gb) gb[(long long)plane * npix + i] = rv;
  }
}

// The z-derivative of the VRS Ez derivation, reduced against the Ez gradient:
// per batch entry b, sum_i Re(conj(g_i) dEz_i/dz) with
// dEz/dz = -(Ex X + Ey Y) z / r^3, r^2 = X^2 + Y^2 + z^2 (vectorized_optics.py:258-261).
__global__ void __launch_bounds__(MSE_THREADS) vrs_dz_ez_partial(const float2* __restrict__ ex,
                                                                 const float2* __restrict__ ey, long long ebs,
                                                                 const float2* __restrict__ g, long long gbs,
                                                                 int ny, int nx, const double* __restrict__ x,
                                                                 const double* __restrict__ y,
                                                                 const double* __restrict__ z,
                                                                 double* __restrict__ partial) {
  const int b = blockIdx.y;
  const long long npix = (long long)ny * nx;
  ex += (long long)b * ebs;
  ey += (long long)b * ebs;
  g += (long long)b * gbs;
  const float zf = (float)z[b];
  float acc = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const int row = (int)((unsigned)i / (unsigned)nx), col = (int)i - row * nx;
    const float X = (float)x[col], Y = (float)y[row];
    const float ir = rsqrtf(X * X + Y * Y + zf * zf);
    const float w = -zf * ir * ir * ir;
    const float2 u = ex[i], v = ey[i], gg = g[i];
    const float2 d = make_float2(w * (u.x * X + v.x * Y), w * (u.y * X + v.y * Y));
    acc = fmaf(gg.x, d.x, fmaf(gg.y, d.y, acc));
  }
  __shared__ float red[MSE_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w2 = 0; w2 < MSE_THREADS / 32; ++w2) t += red[w2];
    partial[(long long)b * gridDim.x + blockIdx.x] = t;
  }
}

// The whole distance gradient of one RS / VRS call per batch entry b:
// sum_c sum_i Re(conj(g_c) d_c) over the propagated components (d: the
// propagation through the dH/dz spectrum) plus, for VRS, sum_i Re(conj(gez)
// dEz/dz) of the input-plane Ez derivation -- one pass instead of a reduction
// per component.
struct ZGradArgs {
  const float2* g[3];
  const float2* d[3];
  long long bs;          // batch stride of g and d (elements)
  int ncomp;
  const float2* ex;      // VRS: the Jones program's output (NULL: scalar RS)
  const float2* ey;
  long long ebs;
  const float2* gez;     // VRS: the propagated Ez gradient before its fold
  const double* x;
  const double* y;
  const double* z;       // one per batch entry
  int ny, nx;
};

__global__ void __launch_bounds__(MSE_THREADS) rs_zgrad_partial(ZGradArgs p, double* __restrict__ partial) {
  const int b = blockIdx.y;
  const long long npix = (long long)p.ny * p.nx;
  const long long o = (long long)b * p.bs;
  float acc = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    for (int c = 0; c < p.ncomp; ++c) {
      const float2 u = p.g[c][o + i], v = p.d[c][o + i];
      acc = fmaf(u.x, v.x, fmaf(u.y, v.y, acc));
    }
    if (p.ex) {
      const int row = (int)((unsigned)i / (unsigned)p.nx), col = (int)i - row * p.nx;
      const float X = (float)p.x[col], Y = (float)p.y[row], zf = (float)p.z[b];
      const float ir = rsqrtf(X * X + Y * Y + zf * zf);
      const float w = -zf * ir * ir * ir;
      const float2 u = p.ex[(long long)b * p.ebs + i], v = p.ey[(long long)b * p.ebs + i], gg = p.gez[o + i];
      acc = fmaf(gg.x, w * (u.x * X + v.x * Y), fmaf(gg.y, w * (u.y * X + v.y * Y), acc));
    }
  }
  __shared__ float red[MSE_THREADS / 32];
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < MSE_THREADS / 32; ++w) t += red[w];
    partial[(long long)b * gridDim.x + blockIdx.x] = t;
  }
}

static int mse_blocks(long long npix) {
  long long nb = (npix + MSE_THREADS * 8 - 1) / (MSE_THREADS * 8);
  if (nb > 152 * 4) nb = 152 * 4;
  return nb < 1 ? 1 : (int)nb;
}

static cudaError_t elem_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

static const bool elem_registered = register_device_tables(&elem_upload_twiddles, nullptr);

}  // namespace xl

using namespace xl;

extern "C" int xl_ops_backward(void* stream, int batch, int comps, int ny, int nx, const void* const* in,
                               long long in_bstride, const void* const* gout, long long gout_bstride,
                               void* const* gin, long long gin_bstride, const XlProg* prog,
                               void* const* pgrad) {
  if (batch < 1 || comps < 1 || comps > 3 || ny < 1 || nx < 1 || !in || !gout || !gin || !prog) {
    set_error("xl_ops_backward: bad arguments");
    return XL_EINVAL;
  }
  if (prog->nops < 0 || prog->nops > XL_MAX_OPS) {
    set_error("xl_ops_backward: op program too long");
    return XL_EINVAL;
  }
  OpsBwdLaunch p;
  p.B = batch; p.C = comps; p.ny = ny; p.nx = nx;
  p.ibs = in_bstride; p.gbs = gout_bstride; p.ginbs = gin_bstride;
  for (int c = 0; c < 3; ++c) {
    p.in[c] = c < comps ? (const float2*)in[c] : nullptr;
    p.gout[c] = c < comps ? (const float2*)gout[c] : nullptr;
    p.gin[c] = c < comps ? (float2*)gin[c] : nullptr;
    if (c == 0 && (!p.in[0] || !p.gout[0])) {
      set_error("xl_ops_backward: null plane %d", c);
      return XL_EINVAL;
    }
  }
  p.prog = *prog;
  for (int q = 0; q < XL_MAX_OPS * 4; ++q) p.pgrad[q] = pgrad ? pgrad[q] : nullptr;
  // which gradients need accumulation: scalar parameters (summed over all
  // pixels) and per-pixel parameters shared by the batch (summed over it)
  int scalar_acc = 0, plane_acc = 0;
  for (int k = 0; k < prog->nops; ++k)
    for (int q = 0; q < 4; ++q) {
      if (!p.pgrad[k * 4 + q]) continue;
      const XlOp& op = prog->ops[k];
      if (!(op.pmask & (1 << q))) scalar_acc = 1;
      else if (!op.pbstride) plane_acc = 1;
    }
  const long long npix = (long long)ny * nx;
  if (npix > 0x7fffffffLL) {
    set_error("xl_ops_backward: plane too large");
    return XL_EINVAL;
  }
  const long long need = (npix + 127) / 128;
  // without batch sums, one thread per pixel and batch entry (grid.y = batch)
  const int gy = (plane_acc || batch > 65535) ? 1 : batch;
  const size_t sm = (size_t)(scalar_acc + plane_acc) * XL_MAX_OPS * 4 * 128 * sizeof(float);
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 152;
  // one wave: the CTAs that fit on the device at once (the pixel loop strides
  // over the rest), so that no second, partly empty wave follows
  auto grid_for = [&](auto kernel) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, sm) != cudaSuccess || per_sm < 1)
      per_sm = 4;
    long long bx = ((long long)per_sm * sms + gy - 1) / gy;
    if (bx > need) bx = need;
    if (bx < 1) bx = 1;
    return dim3((unsigned)bx, gy);
  };
  // programs the tables and the benchmarks run get a kernel with their op
  // kinds fixed (the high-NA table's LCD-sSLM-lens, the VRS benchmark's
  // LCD-polarizer, the 4f table's phase SLM and thin lens); any other
  // program takes the generic one
  auto is = [&](std::initializer_list<int> ks) {
    if ((int)ks.size() != prog->nops) return false;
    int k = 0;
    for (int v : ks)
      if (prog->ops[k++].kind != v) return false;
    return true;
  };
  cudaStream_t s = (cudaStream_t)stream;
  auto run = [&](auto kernel) { kernel<<<grid_for(kernel), 128, sm, s>>>(p, scalar_acc, plane_acc); };
  if (is({XL_OP_LCD, XL_OP_SSLM, XL_OP_HIGHNA_EZ}))
    run(ops_backward_kernel<3, FixedKinds<XL_OP_LCD, XL_OP_SSLM, XL_OP_HIGHNA_EZ>>);
  else if (is({XL_OP_LCD, XL_OP_SSLM, XL_OP_HIGHNA}))
    run(ops_backward_kernel<3, FixedKinds<XL_OP_LCD, XL_OP_SSLM, XL_OP_HIGHNA>>);
  else if (is({XL_OP_LCD, XL_OP_LP}))
    run(ops_backward_kernel<2, FixedKinds<XL_OP_LCD, XL_OP_LP>>);
  else if (is({XL_OP_PHASE}))
    run(ops_backward_kernel<1, FixedKinds<XL_OP_PHASE>>);
  else if (is({XL_OP_SEPMASK}))
    run(ops_backward_kernel<1, FixedKinds<XL_OP_SEPMASK>>);
  else if (prog->nops <= 4)
    run(ops_backward_kernel<4>);
  else
    run(ops_backward_kernel<XL_MAX_OPS>);
  XL_CHECK_LAUNCH("ops_backward_kernel");
  return XL_OK;
}

namespace xl {
// The transfer function of the chirp-z prologue and epilogue on a whole grid,
// evaluated by the same device function (rs_kernel_value) as the kernels.
__global__ void __launch_bounds__(256) czt_transfer_plane_kernel(int ny, int nx, const double* __restrict__ x,
                                                                 const double* __restrict__ y, double z,
                                                                 double inv_lambda, float k, float2* out) {
  const long long n = (long long)ny * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / nx), c = (int)(i - (long long)r * nx);
    out[i] = rs_kernel_value(x[c], y[r], z, inv_lambda, k);
  }
}
}  // namespace xl

extern "C" int xl_czt_transfer_plane(void* stream, int ny, int nx, const double* x, const double* y, double z,
                                     double wavelength, void* out) {
  if (ny < 1 || nx < 1 || !x || !y || !out || !(wavelength > 0)) {
    set_error("xl_czt_transfer_plane: bad arguments");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  const long long n = (long long)ny * nx;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  czt_transfer_plane_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      ny, nx, x, y, z, 1.0 / wavelength, (float)(2.0 * M_PI / wavelength), (float2*)out);
  XL_CHECK_LAUNCH("czt_transfer_plane_kernel");
  return XL_OK;
}

extern "C" int xl_highna_coefficients(void* stream, int ny, int nx, const double* x, const double* y,
                                      double radius, double f, void* out) {
  if (ny < 1 || nx < 1 || !x || !y || !out || !(radius > 0) || !(f > 0)) {
    set_error("xl_highna_coefficients: bad arguments");
    return XL_EINVAL;
  }
  XlOp op = {};
  op.kind = XL_OP_HIGHNA;
  op.ptr[0] = x;
  op.ptr[1] = y;
  op.dval[0] = radius;
  op.dval[1] = f;
  op.dval[2] = radius / sqrt(radius * radius + f * f);
  op.dval[3] = 1.0 / (radius * radius);
  const long long npix = (long long)ny * nx;
  int blocks = (int)((npix + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  highna_plane_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(ny, nx, op, (float*)out);
  XL_CHECK_LAUNCH("highna_plane_kernel");
  return XL_OK;
}

extern "C" int xl_apply_ops(void* stream, int batch, int comps, int ny, int nx, const void* const* in,
                            long long in_bstride, void* const* out, long long out_bstride,
                            const XlProg* prog) {
  if (batch < 1 || comps < 1 || comps > 3 || ny < 1 || nx < 1 || !in || !out || !prog) {
    set_error("xl_apply_ops: bad arguments");
    return XL_EINVAL;
  }
  if (prog->nops < 0 || prog->nops > XL_MAX_OPS) {
    set_error("xl_apply_ops: op program too long");
    return XL_EINVAL;
  }
  ElemLaunch p;
  p.B = batch; p.C = comps; p.ny = ny; p.nx = nx; p.ibs = in_bstride; p.obs = out_bstride;
  for (int c = 0; c < 3; ++c) {
    p.in[c] = c < comps ? (const float2*)in[c] : nullptr;
    p.out[c] = c < comps ? (float2*)out[c] : nullptr;
    if (c < comps && (!p.in[c] || !p.out[c])) {
      set_error("xl_apply_ops: null plane %d", c);
      return XL_EINVAL;
    }
  }
  p.prog = *prog;
  const long long npix = (long long)ny * nx;
  int blocks = (int)((npix + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  apply_ops_kernel<<<dim3(blocks, batch), 256, 0, (cudaStream_t)stream>>>(p);
  XL_CHECK_LAUNCH("apply_ops_kernel");
  return XL_OK;
}

extern "C" size_t xl_mse_intensity_work_bytes(int planes, long long npix) {
  if (planes < 1 || npix < 1) return 0;
  return (size_t)planes * mse_blocks(npix) * sizeof(double);
}

extern "C" int xl_mse_intensity(void* stream, int planes, long long npix, const void* a, long long a_pstride,
                                const void* b, long long b_pstride, void* work, void* out) {
  if (planes < 1 || planes > 65535 || npix < 1 || !a || !b || !work || !out) {
    set_error("xl_mse_intensity: bad arguments");
    return XL_EINVAL;
  }
  const int nb = mse_blocks(npix);
  cudaStream_t st = (cudaStream_t)stream;
  plane_sum_partial<0><<<dim3(nb, planes), MSE_THREADS, 0, st>>>((const float2*)a, a_pstride, (const float2*)b,
                                                                  b_pstride, npix, (double*)work);
  XL_CHECK_LAUNCH("plane_sum_partial");
  mse_int_finish<<<(planes + 3) / 4, 128, 0, st>>>((const double*)work, nb, planes, 1.0 / (double)npix,
                                                    (float*)out);
  XL_CHECK_LAUNCH("mse_int_finish");
  return XL_OK;
}

extern "C" int xl_mse_intensity_grad(void* stream, int planes, long long npix, const void* a, long long a_pstride,
                                     const void* b, long long b_pstride, const void* gloss, void* ga, void* gb) {
  if (planes < 1 || planes > 65535 || npix < 1 || !a || !b || !gloss || (!ga && !gb)) {
    set_error("xl_mse_intensity_grad: bad arguments");
    return XL_EINVAL;
  }
  long long nblk = (npix + 255) / 256;
  if (nblk > 152 * 8) nblk = 152 * 8;
  mse_int_grad<<<dim3((unsigned)nblk, planes), 256, 0, (cudaStream_t)stream>>>(
      (const float2*)a, a_pstride, (const float2*)b, b_pstride, npix, (const float*)gloss,
      (float)(4.0 / (double)npix), (float2*)ga, (float2*)gb);
  XL_CHECK_LAUNCH("mse_int_grad");
  return XL_OK;
}

extern "C" int xl_plane_mse(void* stream, int kind, int planes, long long npix, const void* a, long long a_pstride,
                            const void* b, long long b_pstride, void* work, void* out) {
  if (kind < 0 || kind > 2) {
    set_error("xl_plane_mse: kind must be 0 (intensity), 1 (amplitude) or 2 (phase), got %d", kind);
    return XL_EINVAL;
  }
  if (kind == 0) return xl_mse_intensity(stream, planes, npix, a, a_pstride, b, b_pstride, work, out);
  if (planes < 1 || planes > 65535 || npix < 1 || !a || !b || !work || !out) {
    set_error("xl_plane_mse: bad arguments");
    return XL_EINVAL;
  }
  const int nb = mse_blocks(npix);
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 1)
    plane_sum_partial<2><<<dim3(nb, planes), MSE_THREADS, 0, st>>>((const float2*)a, a_pstride, (const float2*)b,
                                                                    b_pstride, npix, (double*)work);
  else
    plane_sum_partial<3><<<dim3(nb, planes), MSE_THREADS, 0, st>>>((const float2*)a, a_pstride, (const float2*)b,
                                                                    b_pstride, npix, (double*)work);
  XL_CHECK_LAUNCH("plane_sum_partial");
  mse_int_finish<<<(planes + 3) / 4, 128, 0, st>>>((const double*)work, nb, planes, 1.0 / (double)npix,
                                                    (float*)out);
  XL_CHECK_LAUNCH("mse_int_finish");
  return XL_OK;
}

extern "C" int xl_plane_mse_grad(void* stream, int kind, int planes, long long npix, const void* a,
                                 long long a_pstride, const void* b, long long b_pstride, const void* gloss, void* ga,
                                 void* gb) {
  if (kind < 0 || kind > 2) {
    set_error("xl_plane_mse_grad: kind must be 0 (intensity), 1 (amplitude) or 2 (phase), got %d", kind);
    return XL_EINVAL;
  }
  if (kind == 0) return xl_mse_intensity_grad(stream, planes, npix, a, a_pstride, b, b_pstride, gloss, ga, gb);
  if (planes < 1 || planes > 65535 || npix < 1 || !a || !b || !gloss || (!ga && !gb)) {
    set_error("xl_plane_mse_grad: bad arguments");
    return XL_EINVAL;
  }
  long long nblk = (npix + 255) / 256;
  if (nblk > 152 * 8) nblk = 152 * 8;
  const dim3 grid((unsigned)nblk, planes);
  const float tn = (float)(2.0 / (double)npix);
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 1)
    amp_phase_grad<2><<<grid, 256, 0, st>>>((const float2*)a, a_pstride, (const float2*)b, b_pstride, npix,
                                            (const float*)gloss, tn, (float2*)ga, (float2*)gb);
  else
    amp_phase_grad<3><<<grid, 256, 0, st>>>((const float2*)a, a_pstride, (const float2*)b, b_pstride, npix,
                                            (const float*)gloss, tn, (float2*)ga, (float2*)gb);
  XL_CHECK_LAUNCH("amp_phase_grad");
  return XL_OK;
}

extern "C" int xl_re_inner(void* stream, int planes, long long npix, const void* a, long long a_pstride,
                           const void* b, long long b_pstride, void* work, void* out) {
  if (planes < 1 || planes > 65535 || npix < 1 || !a || !b || !work || !out) {
    set_error("xl_re_inner: bad arguments");
    return XL_EINVAL;
  }
  const int nb = mse_blocks(npix);
  cudaStream_t st = (cudaStream_t)stream;
  plane_sum_partial<1><<<dim3(nb, planes), MSE_THREADS, 0, st>>>((const float2*)a, a_pstride, (const float2*)b,
                                                                  b_pstride, npix, (double*)work);
  XL_CHECK_LAUNCH("plane_sum_partial");
  mse_int_finish<<<(planes + 3) / 4, 128, 0, st>>>((const double*)work, nb, planes, 1.0, (float*)out);
  XL_CHECK_LAUNCH("mse_int_finish");
  return XL_OK;
}

extern "C" int xl_vrs_dz_ez(void* stream, int batch, int ny, int nx, const void* ex, const void* ey,
                            long long e_bstride, const void* gez, long long g_bstride, const double* x,
                            const double* y, const double* z, void* work, void* out) {
  if (batch < 1 || batch > 65535 || ny < 1 || nx < 1 || (long long)ny * nx > 0x7fffffffLL || !ex || !ey || !gez ||
      !x || !y || !z || !work || !out) {
    set_error("xl_vrs_dz_ez: bad arguments");
    return XL_EINVAL;
  }
  const long long npix = (long long)ny * nx;
  const int nb = mse_blocks(npix);
  cudaStream_t st = (cudaStream_t)stream;
  vrs_dz_ez_partial<<<dim3(nb, batch), MSE_THREADS, 0, st>>>((const float2*)ex, (const float2*)ey, e_bstride,
                                                             (const float2*)gez, g_bstride, ny, nx, x, y, z,
                                                             (double*)work);
  XL_CHECK_LAUNCH("vrs_dz_ez_partial");
  mse_int_finish<<<(batch + 3) / 4, 128, 0, st>>>((const double*)work, nb, batch, 1.0, (float*)out);
  XL_CHECK_LAUNCH("mse_int_finish");
  return XL_OK;
}

extern "C" int xl_rs_z_gradient(void* stream, int batch, int ny, int nx, int comps, const void* const* g,
                                const void* const* d, long long bstride, const void* ex, const void* ey,
                                long long e_bstride, const void* gez, const double* x, const double* y,
                                const double* z, void* work, void* out) {
  if (batch < 1 || batch > 65535 || ny < 1 || nx < 1 || (long long)ny * nx > 0x7fffffffLL || comps < 1 ||
      comps > 3 || !g || !d || !work || !out || (ex && (!ey || !gez || !x || !y || !z))) {
    set_error("xl_rs_z_gradient: bad arguments");
    return XL_EINVAL;
  }
  ZGradArgs p;
  for (int c = 0; c < 3; ++c) {
    p.g[c] = c < comps ? (const float2*)g[c] : nullptr;
    p.d[c] = c < comps ? (const float2*)d[c] : nullptr;
    if (c < comps && (!p.g[c] || !p.d[c])) {
      set_error("xl_rs_z_gradient: null plane %d", c);
      return XL_EINVAL;
    }
  }
  p.bs = bstride;
  p.ncomp = comps;
  p.ex = (const float2*)ex;
  p.ey = (const float2*)ey;
  p.ebs = e_bstride;
  p.gez = (const float2*)gez;
  p.x = x;
  p.y = y;
  p.z = z;
  p.ny = ny;
  p.nx = nx;
  const int nb = mse_blocks((long long)ny * nx);
  cudaStream_t st = (cudaStream_t)stream;
  rs_zgrad_partial<<<dim3(nb, batch), MSE_THREADS, 0, st>>>(p, (double*)work);
  XL_CHECK_LAUNCH("rs_zgrad_partial");
  mse_int_finish<<<(batch + 3) / 4, 128, 0, st>>>((const double*)work, nb, batch, 1.0, (float*)out);
  XL_CHECK_LAUNCH("mse_int_finish");
  return XL_OK;
}
