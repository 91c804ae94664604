// Table noise on the device: the misalignment and phase noise of shake_setup
// (optical_elements.py:2127-2217), for many optical tables in one launch.
//
// The reference draws with jax's PRNG; here every value comes from a
// counter-based generator, Philox4x32-10 (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011): a 128-bit counter
// and a 64-bit key give four 32-bit words, so any element of any table is
// drawn independently, with no generator state.  Each table has its own key;
// each kind of draw (the distances, the plane magnitudes, the two planes'
// signs, the waveplate signs and magnitudes) its own counter stream.
//
// The structure of the reference's draws is kept: the amplitude and phase
// noise planes share their magnitudes (the reference draws both uniforms from
// the same key, :2214-2215) and differ in their signs; with `discretize` a
// negative sign becomes 255 (the reference casts the sign to uint8, :2196).
#include <stdint.h>

#include "internal.h"
#include "xlgb.h"

namespace xl {

__host__ __device__ __forceinline__ void philox_round(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

// Philox4x32 with 10 rounds: counter c, key (k0, k1), in place.
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k0, k1);
    if (r < 9) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
  }
}

// Counter streams (word 2 of the counter).
enum : uint32_t {
  STREAM_DIST = 1,
  STREAM_MAG = 2,        // plane magnitudes (shared by the phase and amplitude planes)
  STREAM_SIGN_SLM = 3,
  STREAM_SIGN_AMP = 4,
  STREAM_WP_SIGN = 5,
  STREAM_WP_MAG = 6,
};

__device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

struct NoiseKernelArgs {
  XlNoiseArgs a;
  uint32_t key[XL_NOISE_MAX_TABLES][2];
};

// Plane noise: element e of plane q of table t; magnitude uniform in
// [min_phase, max_phase), signs +-1 (255 for -1 when discretised).
__global__ void noise_planes_kernel(const __grid_constant__ NoiseKernelArgs p) {
  const int t = blockIdx.y;
  const long long per_table = (long long)p.a.planes * p.a.resolution * p.a.resolution;
  const uint32_t k0 = p.key[t][0], k1 = p.key[t][1];
  const float lo = (float)p.a.min_phase, span = (float)(p.a.max_phase - p.a.min_phase);
  const float neg = p.a.discretize ? 255.f : -1.f;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per_table;
       e += (long long)gridDim.x * blockDim.x) {
    uint32_t cm[4] = {(uint32_t)e, (uint32_t)(e >> 32), STREAM_MAG, 0u};
    uint32_t cs[4] = {(uint32_t)e, (uint32_t)(e >> 32), STREAM_SIGN_SLM, 0u};
    uint32_t ca[4] = {(uint32_t)e, (uint32_t)(e >> 32), STREAM_SIGN_AMP, 0u};
    philox4x32_10(cm, k0, k1);
    philox4x32_10(cs, k0, k1);
    philox4x32_10(ca, k0, k1);
    const float mag = __fadd_rn(lo, __fmul_rn(span, u24(cm[0])));   // two roundings, no FMA
    const long long o = (long long)t * per_table + e;
    if (p.a.slms) p.a.slms[o] = ((cs[0] & 1u) ? 1.f : neg) * mag;
    if (p.a.amps) p.a.amps[o] = ((ca[0] & 1u) ? 1.f : neg) * mag;
  }
}

// Scalar noise: the distances' misalignment (uniform in [min_d, max_d)) and
// the waveplates' +-uniform(min_phase, max_phase) (signs always +-1).
__global__ void noise_scalars_kernel(const __grid_constant__ NoiseKernelArgs p) {
  const int t = blockIdx.x;
  const uint32_t k0 = p.key[t][0], k1 = p.key[t][1];
  for (int i = threadIdx.x; i < p.a.n_distances; i += blockDim.x) {
    uint32_t c[4] = {(uint32_t)i, 0u, STREAM_DIST, 0u};
    philox4x32_10(c, k0, k1);
    p.a.distances[(long long)t * p.a.n_distances + i] =
        __dadd_rn(p.a.min_d, __dmul_rn(p.a.max_d - p.a.min_d, u53(c[0], c[1])));
  }
  for (int i = threadIdx.x; i < p.a.n_wps; i += blockDim.x) {
    uint32_t cs[4] = {(uint32_t)i, 0u, STREAM_WP_SIGN, 0u};
    uint32_t cm[4] = {(uint32_t)i, 0u, STREAM_WP_MAG, 0u};
    philox4x32_10(cs, k0, k1);
    philox4x32_10(cm, k0, k1);
    const double mag = __dadd_rn(p.a.min_phase, __dmul_rn(p.a.max_phase - p.a.min_phase, u53(cm[0], cm[1])));
    p.a.wps[(long long)t * p.a.n_wps + i] = ((cs[0] & 1u) ? 1.0 : -1.0) * mag;
  }
}

}  // namespace xl

using namespace xl;

extern "C" int xl_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out) {
  if (!counter || !key || !out) {
    set_error("xl_philox4x32_10: null pointer");
    return XL_EINVAL;
  }
  uint32_t c[4] = {counter[0], counter[1], counter[2], counter[3]};
  philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = c[i];
  return XL_OK;
}

extern "C" int xl_table_noise(void* stream, const XlNoiseArgs* a, const uint32_t* keys) {
  if (!a || !keys || a->tables < 1 || a->tables > XL_NOISE_MAX_TABLES || a->planes < 0 || a->resolution < 0 ||
      a->n_distances < 0 || a->n_wps < 0 || (a->planes && a->resolution && !a->slms && !a->amps) ||
      (a->n_distances && !a->distances) || (a->n_wps && !a->wps)) {
    set_error("xl_table_noise: bad arguments");
    return XL_EINVAL;
  }
  NoiseKernelArgs p;
  p.a = *a;
  for (int t = 0; t < a->tables; ++t) {
    p.key[t][0] = keys[2 * t];
    p.key[t][1] = keys[2 * t + 1];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const long long per_table = (long long)a->planes * a->resolution * a->resolution;
  if (per_table > 0) {
    long long blocks = (per_table + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    noise_planes_kernel<<<dim3((unsigned)blocks, a->tables), 256, 0, st>>>(p);
    XL_CHECK_LAUNCH("noise_planes_kernel");
  }
  if (a->n_distances > 0 || a->n_wps > 0) {
    noise_scalars_kernel<<<a->tables, 64, 0, st>>>(p);
    XL_CHECK_LAUNCH("noise_scalars_kernel");
  }
  return XL_OK;
}
