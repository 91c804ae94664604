// Bare one-dimensional transforms: unnormalised complex64 FFTs of contiguous
// lines, forward or inverse, on the library's FFT engine.  They are the
// building block of the reference's Bluestein helpers compute_fft and
// Bluestein_method (wave_optics.py:385-460), which run jnp.fft.fft / ifft
// along an axis; the propagators do not use them (their transforms are fused
// into the line-transform kernels).
#include "line_fft.cuh"

namespace xl {

template <int LOGN> struct LineCfg {
  static constexpr int L = 1 << LOGN;
  static constexpr int T = L / 16;                          // threads per line
  static constexpr int G = (256 / T) > 1 ? (256 / T) : 1;   // lines per CTA
  static constexpr int XS = L + L / 16;
};

// One group of T threads per line; every thread of the CTA takes part in the
// barriers, lines past the end transform zeros and store nothing.
template <int LOGN, int DIR>
__global__ void __launch_bounds__(LineCfg<LOGN>::G * LineCfg<LOGN>::T)
    fft_lines_kernel(long long lines, const float2* __restrict__ in, float2* __restrict__ out) {
  using C = LineCfg<LOGN>;
  extern __shared__ __align__(16) float2 smem[];
  const int gi = threadIdx.x / C::T, j = threadIdx.x % C::T;
  const long long line = (long long)blockIdx.x * C::G + gi;
  const bool live = line < lines;
  float2 v[16];
  const float2* src = in + line * C::L;
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = live ? src[j + m * C::T] : make_float2(0.f, 0.f);
  block_fft_x<LOGN, 16, DIR, false, true>(v, j, smem + gi * C::XS, pass_tw<LOGN>());
  if (live) {
    float2* dst = out + line * C::L;
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[j + m * C::T] = v[m];
  }
}

// Lines of 1..16 points: the DFT sum directly, one thread per output point.
template <int DIR>
__global__ void dft_small_kernel(int logn, long long lines, const float2* __restrict__ in, float2* __restrict__ out) {
  const int L = 1 << logn;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= lines * L) return;
  const long long line = i / L;
  const int k = (int)(i % L);
  const float2* x = in + line * L;
  const float2* tw = tw_table(logn);   // e^{-2 pi i q / L}
  float2 acc = make_float2(0.f, 0.f);
  for (int n = 0; n < L; ++n) {
    const float2 w = tw[(n * k) & (L - 1)];
    acc = cadd(acc, DIR < 0 ? cmul(x[n], w) : cmulc(x[n], w));
  }
  out[i] = acc;
}

template <int LOGN, int DIR>
static int launch_lines(cudaStream_t st, long long lines, const float2* in, float2* out) {
  using C = LineCfg<LOGN>;
  const size_t sm = (size_t)C::G * C::XS * sizeof(float2);
  cudaError_t e = allow_smem(fft_lines_kernel<LOGN, DIR>, sm);
  if (e != cudaSuccess) return cuda_fail(e, "fft_lines smem");
  const long long grid = (lines + C::G - 1) / C::G;
  if (grid > 0x7fffffffLL) {
    set_error("xl_fft_lines: too many lines (%lld)", lines);
    return XL_EINVAL;
  }
  fft_lines_kernel<LOGN, DIR><<<(unsigned)grid, C::G * C::T, sm, st>>>(lines, in, out);
  XL_CHECK_LAUNCH("fft_lines");
  return XL_OK;
}

template <int DIR>
static int dispatch_lines(cudaStream_t st, int logn, long long lines, const float2* in, float2* out) {
  switch (logn) {
    case 5: return launch_lines<5, DIR>(st, lines, in, out);
    case 6: return launch_lines<6, DIR>(st, lines, in, out);
    case 7: return launch_lines<7, DIR>(st, lines, in, out);
    case 8: return launch_lines<8, DIR>(st, lines, in, out);
    case 9: return launch_lines<9, DIR>(st, lines, in, out);
    case 10: return launch_lines<10, DIR>(st, lines, in, out);
    case 11: return launch_lines<11, DIR>(st, lines, in, out);
    case 12: return launch_lines<12, DIR>(st, lines, in, out);
    case 13: return launch_lines<13, DIR>(st, lines, in, out);
    default: break;
  }
  const long long n = lines << logn;
  const long long grid = (n + 255) / 256;
  if (grid > 0x7fffffffLL) {
    set_error("xl_fft_lines: too many lines (%lld)", lines);
    return XL_EINVAL;
  }
  dft_small_kernel<DIR><<<(unsigned)grid, 256, 0, st>>>(logn, lines, in, out);
  XL_CHECK_LAUNCH("dft_small");
  return XL_OK;
}

}  // namespace xl

using namespace xl;

extern "C" int xl_fft_lines(void* stream, int log2_len, long long lines, int dir, const void* in, void* out) {
  if (log2_len < 0 || log2_len > 13 || lines < 0 || (dir != -1 && dir != 1)) {
    set_error("xl_fft_lines: need 0 <= log2_len <= 13, lines >= 0 and dir = -1 or +1 (got %d, %lld, %d)",
              log2_len, lines, dir);
    return XL_EINVAL;
  }
  if (lines == 0) return XL_OK;
  if (!in || !out) {
    set_error("xl_fft_lines: null pointer argument");
    return XL_EINVAL;
  }
  if (log2_len <= 4 && in == out) {
    set_error("xl_fft_lines: lines of fewer than 32 points are not transformed in place");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return dir < 0 ? dispatch_lines<-1>(st, log2_len, lines, (const float2*)in, (float2*)out)
                 : dispatch_lines<1>(st, log2_len, lines, (const float2*)in, (float2*)out);
}
