// Beam splitters: the two-port mixing of optical_elements.py:334-512.
//
// BS_symmetric (:334-391), BS_symmetric_SI (:393-460, one input port) and the
// lossless BS (:462-512) are all one complex 2x2 matrix M applied to the
// (Ex, Ey) planes of the input ports a, b:
//   c = M00 a + M01 b,   d = M10 a + M11 b     (Ez of c, d is zero).
// M is read from device memory (per batch entry, or one for the batch), or,
// for the lossy splitters, computed in each CTA from the splitting angle in
// device memory: a differentiable angle is never read back to the host and
// needs no separate kernels to build M or to take dL/dtheta.
//
// The backward runs in one pass over the output gradients gc, gd and the
// forward inputs: the input gradients (M^H applied to the output gradients)
// and, for the gradient of M, S_ij = sum over pixels and components of
// conj(g_i) in_j, per batch entry in fixed-order float64 partial sums.
#include "fft_core.cuh"
#include "internal.h"
#include "xlgb.h"

namespace xl {

constexpr int BS_THREADS = 256;

struct BsKernelArgs {
  const float2* in[2][2];   // [port][component]
  long long ibs[2];
  float2* out[2][2];
  long long obs;
  const float2* m;
  long long mbs;
  const double* theta;      // splitter angle (kind > 0), per batch entry when tbs = 1
  long long tbs;
  int kind;
  int npix;
};

// R and T of the lossy symmetric splitter (optical_elements.py:376-383):
// R = |sin t| - 0.01 |cos t|, T = 0.99 |cos t|, and their derivatives
// (d|u| = sign(u) du, sign(0) = 0, as torch's and jax's abs).
__host__ __device__ __forceinline__ void bs_rt(double t, double* R, double* T, double* dR, double* dT) {
  const double s = sin(t), c = cos(t);
  const double ss = (s > 0) - (s < 0), sc = (c > 0) - (c < 0);
  *R = fabs(s) - 0.01 * fabs(c);
  *T = 0.99 * fabs(c);
  *dR = ss * c + 0.01 * sc * s;
  *dT = -0.99 * sc * s;
}

// The splitter matrix of batch entry b: given (kind 0), or from the angle.
__device__ __forceinline__ void bs_matrix(const BsKernelArgs& p, int b, float2 (&m)[4]) {
  if (p.kind == XL_BS_MATRIX) {
    const float2* q = p.m + (long long)b * p.mbs;
    for (int i = 0; i < 4; ++i) m[i] = q[i];
    return;
  }
  double R, T, dR, dT;
  bs_rt(p.theta[(long long)b * p.tbs], &R, &T, &dR, &dT);
  const float2 r = make_float2((float)R, 0.f), it = make_float2(0.f, (float)T), z = make_float2(0.f, 0.f);
  if (p.kind == XL_BS_SYMMETRIC) {          // c = R a + iT b, d = iT a + R b
    m[0] = r; m[1] = it; m[2] = it; m[3] = r;
  } else if (p.kind == XL_BS_SINGLE_PORT0) { // c = R a, d = iT a
    m[0] = r; m[1] = z; m[2] = it; m[3] = z;
  } else {                                  // port 1: c = iT a, d = R a
    m[0] = it; m[1] = z; m[2] = r; m[3] = z;
  }
}

__device__ __forceinline__ float2 ld_or_zero(const float2* p, long long i) {
  return p ? p[i] : make_float2(0.f, 0.f);
}

__global__ void __launch_bounds__(BS_THREADS) bs_apply_kernel(BsKernelArgs p) {
  const int b = blockIdx.y;
  float2 m[4];
  bs_matrix(p, b, m);
  const float2 m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
  const long long ib0 = (long long)b * p.ibs[0], ib1 = (long long)b * p.ibs[1], ob = (long long)b * p.obs;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.npix; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float2 u = ld_or_zero(p.in[0][c], ib0 + i);
      const float2 v = ld_or_zero(p.in[1][c], ib1 + i);
      if (p.out[0][c]) p.out[0][c][ob + i] = cadd(cmul(m00, u), cmul(m01, v));
      if (p.out[1][c]) p.out[1][c][ob + i] = cadd(cmul(m10, u), cmul(m11, v));
    }
  }
}

struct BsBackArgs {
  BsKernelArgs f;            // forward inputs and M (f.out unused)
  const float2* g[2][2];     // output gradients [port][component]
  long long gbs;
  float2* gin[2][2];         // input gradients [port][component], NULL skips
  long long ginbs;
  double* partial;           // [batch][8][blocks] or NULL
};

// gin_j = sum_i conj(M_ij) g_i; S_ij = sum conj(g_i) in_j, accumulated as
// (Re S00, Im S00, Re S01, Im S01, Re S10, Im S10, Re S11, Im S11).
__global__ void __launch_bounds__(BS_THREADS) bs_backward_kernel(BsBackArgs p) {
  const int b = blockIdx.y;
  float2 m[4];
  bs_matrix(p.f, b, m);
  const float2 m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
  const long long ib0 = (long long)b * p.f.ibs[0], ib1 = (long long)b * p.f.ibs[1];
  const long long gb = (long long)b * p.gbs, ob = (long long)b * p.ginbs;
  float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.f.npix; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float2 g0 = ld_or_zero(p.g[0][c], gb + i);
      const float2 g1 = ld_or_zero(p.g[1][c], gb + i);
      if (p.gin[0][c]) p.gin[0][c][ob + i] = cadd(cmulc(g0, m00), cmulc(g1, m10));
      if (p.gin[1][c]) p.gin[1][c][ob + i] = cadd(cmulc(g0, m01), cmulc(g1, m11));
      if (p.partial) {
        const float2 u = ld_or_zero(p.f.in[0][c], ib0 + i);
        const float2 v = ld_or_zero(p.f.in[1][c], ib1 + i);
        const float2 a = cmulc(u, g0), bb = cmulc(v, g0), cc = cmulc(u, g1), d = cmulc(v, g1);
        s[0] += a.x; s[1] += a.y; s[2] += bb.x; s[3] += bb.y;
        s[4] += cc.x; s[5] += cc.y; s[6] += d.x; s[7] += d.y;
      }
    }
  }
  if (!p.partial) return;
  __shared__ float red[8][BS_THREADS / 32];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    float t = s[q];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    double t = 0.0;
    for (int w = 0; w < BS_THREADS / 32; ++w) t += red[threadIdx.x][w];
    p.partial[((long long)b * 8 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
}

// One warp per (batch entry, component of S): lane l sums partials l, l + 32,
// ... in order, then a fixed shuffle tree.
__global__ void bs_finish_kernel(const double* __restrict__ partial, int nblk, int rows, float* __restrict__ out) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  double t = 0.0;
  for (int k = lane; k < nblk; k += 32) t += partial[(long long)row * nblk + k];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[row] = (float)t;
}

// dL/dtheta per batch entry from S_ij = sum conj(g_i) in_j: sum_ij Re(dM_ij/dtheta S_ij).
__global__ void bs_dtheta_kernel(const float2* __restrict__ S, const double* __restrict__ theta, long long tbs,
                                 int kind, int batch, double* __restrict__ dtheta) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  double R, T, dR, dT;
  bs_rt(theta[(long long)b * tbs], &R, &T, &dR, &dT);
  const float2* s = S + 4 * (long long)b;
  double g;
  if (kind == XL_BS_SYMMETRIC)
    g = dR * ((double)s[0].x + s[3].x) - dT * ((double)s[1].y + s[2].y);
  else if (kind == XL_BS_SINGLE_PORT0)
    g = dR * s[0].x - dT * s[2].y;
  else
    g = -dT * s[0].y + dR * s[2].x;
  dtheta[b] = g;
}

static int bs_blocks(int npix) {
  int nb = (npix + BS_THREADS * 4 - 1) / (BS_THREADS * 4);
  if (nb > 152 * 4) nb = 152 * 4;
  return nb < 1 ? 1 : nb;
}

static int bs_check(const XlBsArgs* a, const char* where) {
  if (!a || a->batch < 1 || a->batch > 65535 || a->ny < 1 || a->nx < 1 ||
      (long long)a->ny * a->nx > 0x7fffffffLL || a->kind < XL_BS_MATRIX || a->kind > XL_BS_SINGLE_PORT1 ||
      (a->kind == XL_BS_MATRIX && !a->m) || (a->kind != XL_BS_MATRIX && !a->theta) ||
      (a->theta_bstride != 0 && a->theta_bstride != 1) || !a->in[0][0] || !a->in[0][1] ||
      (!a->in[1][0]) != (!a->in[1][1]) || a->in_bstride[0] < 0 || a->in_bstride[1] < 0 ||
      a->out_bstride < 0 || (a->m_bstride != 0 && a->m_bstride != 4)) {
    set_error("%s: bad arguments", where);
    return XL_EINVAL;
  }
  return XL_OK;
}

static BsKernelArgs bs_kernel_args(const XlBsArgs* a) {
  BsKernelArgs k;
  for (int j = 0; j < 2; ++j)
    for (int c = 0; c < 2; ++c) {
      k.in[j][c] = (const float2*)a->in[j][c];
      k.out[j][c] = (float2*)a->out[j][c];
    }
  k.ibs[0] = a->in_bstride[0];
  k.ibs[1] = a->in_bstride[1];
  k.obs = a->out_bstride;
  k.m = (const float2*)a->m;
  k.mbs = a->m_bstride;
  k.theta = a->theta;
  k.tbs = a->theta_bstride;
  k.kind = a->kind;
  k.npix = a->ny * a->nx;
  return k;
}

}  // namespace xl

using namespace xl;

extern "C" int xl_beam_splitter(void* stream, const XlBsArgs* a) {
  if (int rc = bs_check(a, "xl_beam_splitter")) return rc;
  const BsKernelArgs k = bs_kernel_args(a);
  bs_apply_kernel<<<dim3(bs_blocks(k.npix), a->batch), BS_THREADS, 0, (cudaStream_t)stream>>>(k);
  XL_CHECK_LAUNCH("bs_apply_kernel");
  return XL_OK;
}

extern "C" size_t xl_beam_splitter_work_bytes(int batch, int ny, int nx) {
  if (batch < 1 || ny < 1 || nx < 1) return 0;
  return (size_t)batch * 8 * bs_blocks(ny * nx) * sizeof(double);
}

extern "C" int xl_beam_splitter_backward(void* stream, const XlBsArgs* a, const void* const* gout,
                                         long long gout_bstride, void* const* gin, long long gin_bstride,
                                         void* s, void* work, void* dtheta) {
  if (int rc = bs_check(a, "xl_beam_splitter_backward")) return rc;
  if (!gout || (s && !work) || gout_bstride < 0 || gin_bstride < 0 ||
      (dtheta && (!s || a->kind == XL_BS_MATRIX))) {
    set_error("xl_beam_splitter_backward: bad arguments");
    return XL_EINVAL;
  }
  BsBackArgs p;
  p.f = bs_kernel_args(a);
  for (int i = 0; i < 2; ++i)
    for (int c = 0; c < 2; ++c) {
      p.g[i][c] = (const float2*)gout[2 * i + c];
      p.gin[i][c] = gin ? (float2*)gin[2 * i + c] : nullptr;
    }
  if (!p.g[0][0] && !p.g[0][1] && !p.g[1][0] && !p.g[1][1]) {
    set_error("xl_beam_splitter_backward: no output gradient");
    return XL_EINVAL;
  }
  p.gbs = gout_bstride;
  p.ginbs = gin_bstride;
  p.partial = s ? (double*)work : nullptr;
  const int nb = bs_blocks(p.f.npix);
  cudaStream_t st = (cudaStream_t)stream;
  bs_backward_kernel<<<dim3(nb, a->batch), BS_THREADS, 0, st>>>(p);
  XL_CHECK_LAUNCH("bs_backward_kernel");
  if (s) {
    const int rows = a->batch * 8;
    bs_finish_kernel<<<(rows + 3) / 4, 128, 0, st>>>((const double*)work, nb, rows, (float*)s);
    XL_CHECK_LAUNCH("bs_finish_kernel");
  }
  if (dtheta) {
    bs_dtheta_kernel<<<(a->batch + 127) / 128, 128, 0, st>>>((const float2*)s, a->theta, a->theta_bstride,
                                                             a->kind, a->batch, (double*)dtheta);
    XL_CHECK_LAUNCH("bs_dtheta_kernel");
  }
  return XL_OK;
}
