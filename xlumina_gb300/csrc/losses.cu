// Fused loss epilogues of the optimisation tables, forward and gradient, on
// complex fields (the intensity |u|^2 formed in the kernel) or on real
// intensities:
//
//   area loss, small_area_hybrid (loss_functions.py:24-40) per plane:
//     In = I / (sum I + 1e-8), mask = In > 0.7 max In,
//     L = sum(mask) / (sum(mask In) + 1e-8);
//   normalised intensity MSE (experiments/four_f_optical_table.py:129-141):
//     In = I / sum I, L = sum((In - T)^2) / npix.
//
// Each is two reduction passes (the plane sum and maximum, then the masked or
// squared sums) with block partials in float64, summed in a fixed order (the
// same result on every call), and one elementwise gradient pass seeded by the
// upstream gradient per plane.  The statistics of the forward (sum, threshold,
// the second-pass sums) stay in the caller's work buffer for the gradient.
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace xl {

constexpr int LOSS_THREADS = 256;
constexpr int LOSS_STATS = 8;   // doubles per plane at the start of the work buffer

static int loss_blocks(long long npix) {
  long long b = (npix + 4LL * LOSS_THREADS - 1) / (4LL * LOSS_THREADS);
  return (int)(b < 1 ? 1 : (b > 96 ? 96 : b));
}

struct LossIn {
  const void* p;
  long long ps;      // plane stride (elements)
  int cplx;          // 1: complex64 field, 0: float32 intensity
  __device__ __forceinline__ float I(int plane, long long i) const {
    if (cplx) {
      const float2 u = ((const float2*)p)[(long long)plane * ps + i];
      return u.x * u.x + u.y * u.y;
    }
    return ((const float*)p)[(long long)plane * ps + i];
  }
};

// Block reduction of a float sum (to double) and, optionally, a float max.
__device__ __forceinline__ void block_reduce(float s, float m, double* out_s, float* out_m) {
  __shared__ float rs[LOSS_THREADS / 32], rm[LOSS_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  if ((threadIdx.x & 31) == 0) {
    rs[threadIdx.x >> 5] = s;
    rm[threadIdx.x >> 5] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    float mm = rm[0];
    for (int w = 0; w < LOSS_THREADS / 32; ++w) {
      t += rs[w];
      mm = fmaxf(mm, rm[w]);
    }
    *out_s = t;
    if (out_m) *out_m = mm;
  }
}

// Pass 1: per block, the sum and the maximum of the plane's intensities.
__global__ void __launch_bounds__(LOSS_THREADS) loss_pass1(LossIn in, long long npix, double* __restrict__ psum,
                                                           float* __restrict__ pmax) {
  const int plane = blockIdx.y;
  float s = 0.f, m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const float v = in.I(plane, i);
    s += v;
    m = fmaxf(m, v);
  }
  block_reduce(s, m, psum + (long long)plane * gridDim.x + blockIdx.x,
               pmax + (long long)plane * gridDim.x + blockIdx.x);
}

// Finish 1, one warp per plane: stats[0] = S, stats[1] = 1 / (S + eps),
// stats[2] = the area threshold 0.7 max(In) (area loss only).
__global__ void loss_finish1(const double* __restrict__ psum, const float* __restrict__ pmax, int nb, int planes,
                             double eps, double* __restrict__ stats) {
  const int plane = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (plane >= planes) return;
  double t = 0.0;
  float m = 0.f;
  for (int k = lane; k < nb; k += 32) {
    t += psum[(long long)plane * nb + k];
    m = fmaxf(m, pmax[(long long)plane * nb + k]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_xor_sync(0xffffffffu, t, o);
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  if (lane == 0) {
    double* st = stats + (long long)plane * LOSS_STATS;
    const double inv = 1.0 / (t + eps);
    st[0] = t;
    st[1] = inv;
    st[2] = 0.7 * ((double)m * inv);
  }
}

// Pass 2.  AREA: sums of mask and of mask * In; NMSE: sums of (In - T)^2 and
// of (In - T) In.
template <bool AREA>
__global__ void __launch_bounds__(LOSS_THREADS) loss_pass2(LossIn in, const float* __restrict__ tgt, long long tps,
                                                           long long npix, const double* __restrict__ stats,
                                                           double* __restrict__ pa, double* __restrict__ pb) {
  const int plane = blockIdx.y;
  const double* st = stats + (long long)plane * LOSS_STATS;
  const float inv = (float)st[1], thr = (float)st[2];
  float a = 0.f, c = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const float In = in.I(plane, i) * inv;
    if (AREA) {
      if (In > thr) {
        a += 1.f;
        c += In;
      }
    } else {
      const float d = In - tgt[(long long)plane * tps + i];
      a = fmaf(d, d, a);
      c = fmaf(d, In, c);
    }
  }
  const long long slot = (long long)plane * gridDim.x + blockIdx.x;
  block_reduce(a, 0.f, pa + slot, nullptr);
  __syncthreads();
  block_reduce(c, 0.f, pb + slot, nullptr);
}

// Finish 2: stats[3], stats[4] = the two sums, and the plane's loss.
template <bool AREA>
__global__ void loss_finish2(const double* __restrict__ pa, const double* __restrict__ pb, int nb, int planes,
                             double inv_npix, double* __restrict__ stats, float* __restrict__ loss) {
  const int plane = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (plane >= planes) return;
  double a = 0.0, c = 0.0;
  for (int k = lane; k < nb; k += 32) {
    a += pa[(long long)plane * nb + k];
    c += pb[(long long)plane * nb + k];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (lane == 0) {
    double* st = stats + (long long)plane * LOSS_STATS;
    st[3] = a;
    st[4] = c;
    loss[plane] = (float)(AREA ? a / (c + 1e-8) : a * inv_npix);
  }
}

// Gradient.  dL/dI_j: AREA -A / (E + eps)^2 (mask_j - E) / (S + eps);
// NMSE 2 / (npix S) ((In_j - T_j) - C).  A complex input gets 2 g dL/dI u_j
// (torch's convention for complex tensors), a real one g dL/dI_j.
template <bool AREA>
__global__ void __launch_bounds__(LOSS_THREADS) loss_grad(LossIn in, const float* __restrict__ tgt, long long tps,
                                                          long long npix, const double* __restrict__ stats,
                                                          const float* __restrict__ gloss, void* gin, long long gps) {
  const int plane = blockIdx.y;
  const double* st = stats + (long long)plane * LOSS_STATS;
  const float inv = (float)st[1], thr = (float)st[2];
  const double g = gloss[plane];
  float k0, k1;   // dL/dI_j = k0 * (u_j-term) + k1
  if (AREA) {
    const double A = st[3], E = st[4];
    const double f = -g * A / ((E + 1e-8) * (E + 1e-8)) * st[1];
    k0 = (float)f;                  // times mask_j
    k1 = (float)(-f * E);
  } else {
    const double f = g * 2.0 / ((double)npix) * st[1];
    k0 = (float)f;                  // times (In_j - T_j)
    k1 = (float)(-f * st[4]);
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
       i += (long long)gridDim.x * blockDim.x) {
    const long long o = (long long)plane * gps + i;
    float dI;
    float2 u = make_float2(0.f, 0.f);
    float Iv;
    if (in.cplx) {
      u = ((const float2*)in.p)[(long long)plane * in.ps + i];
      Iv = u.x * u.x + u.y * u.y;
    } else {
      Iv = ((const float*)in.p)[(long long)plane * in.ps + i];
    }
    const float In = Iv * inv;
    if (AREA) dI = fmaf(k0, In > thr ? 1.f : 0.f, k1);
    else dI = fmaf(k0, In - tgt[(long long)plane * tps + i], k1);
    if (in.cplx) ((float2*)gin)[o] = make_float2(2.f * dI * u.x, 2.f * dI * u.y);
    else ((float*)gin)[o] = dI;
  }
}

// Work buffer: stats (planes x 8 doubles), then partials: psum, pa, pb
// (planes x nb doubles each) and pmax (planes x nb floats).
struct LossWork {
  double* stats;
  double* psum;
  double* pa;
  double* pb;
  float* pmax;
};
static LossWork loss_work(void* work, int planes, int nb) {
  LossWork w;
  w.stats = (double*)work;
  w.psum = w.stats + (long long)planes * LOSS_STATS;
  w.pa = w.psum + (long long)planes * nb;
  w.pb = w.pa + (long long)planes * nb;
  w.pmax = (float*)(w.pb + (long long)planes * nb);
  return w;
}

static int loss_forward(const char* what, bool area, void* stream, int planes, long long npix, int cplx,
                        const void* in, long long in_pstride, const float* tgt, long long tps, void* work,
                        float* loss) {
  if (planes < 1 || planes > 65535 || npix < 1 || !in || !work || !loss || (!area && !tgt)) {
    set_error("%s: bad arguments", what);
    return XL_EINVAL;
  }
  const int nb = loss_blocks(npix);
  const LossWork w = loss_work(work, planes, nb);
  const LossIn li{in, in_pstride, cplx ? 1 : 0};
  cudaStream_t st = (cudaStream_t)stream;
  loss_pass1<<<dim3(nb, planes), LOSS_THREADS, 0, st>>>(li, npix, w.psum, w.pmax);
  XL_CHECK_LAUNCH("loss_pass1");
  loss_finish1<<<(planes + 3) / 4, 128, 0, st>>>(w.psum, w.pmax, nb, planes, area ? 1e-8 : 0.0, w.stats);
  XL_CHECK_LAUNCH("loss_finish1");
  if (area) {
    loss_pass2<true><<<dim3(nb, planes), LOSS_THREADS, 0, st>>>(li, nullptr, 0, npix, w.stats, w.pa, w.pb);
    XL_CHECK_LAUNCH("loss_pass2");
    loss_finish2<true><<<(planes + 3) / 4, 128, 0, st>>>(w.pa, w.pb, nb, planes, 1.0 / npix, w.stats, loss);
  } else {
    loss_pass2<false><<<dim3(nb, planes), LOSS_THREADS, 0, st>>>(li, tgt, tps, npix, w.stats, w.pa, w.pb);
    XL_CHECK_LAUNCH("loss_pass2");
    loss_finish2<false><<<(planes + 3) / 4, 128, 0, st>>>(w.pa, w.pb, nb, planes, 1.0 / npix, w.stats, loss);
  }
  XL_CHECK_LAUNCH("loss_finish2");
  return XL_OK;
}

static int loss_backward(const char* what, bool area, void* stream, int planes, long long npix, int cplx,
                         const void* in, long long in_pstride, const float* tgt, long long tps, const void* work,
                         const float* gloss, void* gin) {
  if (planes < 1 || planes > 65535 || npix < 1 || !in || !work || !gloss || !gin || (!area && !tgt)) {
    set_error("%s: bad arguments", what);
    return XL_EINVAL;
  }
  const LossIn li{in, in_pstride, cplx ? 1 : 0};
  long long nblk = (npix + LOSS_THREADS - 1) / LOSS_THREADS;
  if (nblk > 152 * 8) nblk = 152 * 8;
  const dim3 grid((unsigned)nblk, planes);
  cudaStream_t st = (cudaStream_t)stream;
  if (area)
    loss_grad<true><<<grid, LOSS_THREADS, 0, st>>>(li, nullptr, 0, npix, (const double*)work, gloss, gin, npix);
  else
    loss_grad<false><<<grid, LOSS_THREADS, 0, st>>>(li, tgt, tps, npix, (const double*)work, gloss, gin, npix);
  XL_CHECK_LAUNCH("loss_grad");
  return XL_OK;
}

}  // namespace xl

using namespace xl;

extern "C" size_t xl_loss_work_bytes(int planes, long long npix) {
  if (planes < 1 || npix < 1) return 0;
  const size_t nb = (size_t)loss_blocks(npix);
  return (size_t)planes * (LOSS_STATS * sizeof(double) + 3 * nb * sizeof(double) + nb * sizeof(float));
}

extern "C" int xl_area_loss(void* stream, int planes, long long npix, int complex_in, const void* in,
                            long long in_pstride, void* work, float* loss) {
  return loss_forward("xl_area_loss", true, stream, planes, npix, complex_in, in, in_pstride, nullptr, 0, work,
                      loss);
}

extern "C" int xl_area_loss_grad(void* stream, int planes, long long npix, int complex_in, const void* in,
                                 long long in_pstride, const void* work, const float* gloss, void* gin) {
  return loss_backward("xl_area_loss_grad", true, stream, planes, npix, complex_in, in, in_pstride, nullptr, 0,
                       work, gloss, gin);
}

extern "C" int xl_norm_intensity_mse(void* stream, int planes, long long npix, int complex_in, const void* in,
                                     long long in_pstride, const float* target, long long target_pstride,
                                     void* work, float* loss) {
  return loss_forward("xl_norm_intensity_mse", false, stream, planes, npix, complex_in, in, in_pstride, target,
                      target_pstride, work, loss);
}

extern "C" int xl_norm_intensity_mse_grad(void* stream, int planes, long long npix, int complex_in,
                                          const void* in, long long in_pstride, const float* target,
                                          long long target_pstride, const void* work, const float* gloss,
                                          void* gin) {
  return loss_backward("xl_norm_intensity_mse_grad", false, stream, planes, npix, complex_in, in, in_pstride,
                       target, target_pstride, work, gloss, gin);
}
