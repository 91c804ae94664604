// AdamW for the optimisation tables: every float32 parameter tensor of a
// step updated in one launch, in one pass over memory (read p, g, m, v;
// write p, m, v), with the step count in device memory so the update can be
// recorded in a CUDA graph.
//
// The update is torch.optim.AdamW's (decoupled weight decay):
//   p *= 1 - lr wd;  m += (1 - b1)(g - m);  v = b2 v + (1 - b2) g^2;
//   p -= lr / (1 - b1^t) * m / (sqrt(v) / sqrt(1 - b2^t) + eps),
// t being the step count after its increment.
#include <stdint.h>

#include "internal.h"
#include "xlgb.h"

namespace xl {

struct AdamKernelArgs {
  XlAdamWArgs a;
};

struct AdamCoef {
  float b1, b2, step_size, rbc2, decay, eps;
};

__device__ __forceinline__ void adam_update(float g, float& p, float& m, float& v, const AdamCoef& a) {
  p *= a.decay;
  m = fmaf(1.f - a.b1, g - m, m);
  v = fmaf(a.b2, v, (1.f - a.b2) * g * g);
  const float denom = sqrtf(v) * a.rbc2 + a.eps;
  p -= a.step_size * (m / denom);
}

// Tensors whose four arrays are 16-byte aligned move four elements per load
// (float4); the rest, and the tail past a multiple of four, one at a time.
__global__ void __launch_bounds__(256) adamw_kernel(const __grid_constant__ AdamKernelArgs k) {
  const XlAdamWTensor& t = k.a.t[blockIdx.y];
  const float s = *k.a.step;
  AdamCoef a;
  a.b1 = k.a.beta1;
  a.b2 = k.a.beta2;
  a.step_size = k.a.lr / (1.f - powf(a.b1, s));
  a.rbc2 = 1.f / sqrtf(1.f - powf(a.b2, s));
  a.decay = 1.f - k.a.lr * k.a.weight_decay;
  a.eps = k.a.eps;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool vec = ((((uintptr_t)t.p) | ((uintptr_t)t.g) | ((uintptr_t)t.m) | ((uintptr_t)t.v)) & 15) == 0;
  long long done = 0;
  if (vec) {
    const long long n4 = t.n / 4;
    float4* p4 = (float4*)t.p;
    float4* m4 = (float4*)t.m;
    float4* v4 = (float4*)t.v;
    const float4* g4 = (const float4*)t.g;
    for (long long i = tid; i < n4; i += stride) {
      const float4 g = g4[i];
      float4 p = p4[i], m = m4[i], v = v4[i];
      adam_update(g.x, p.x, m.x, v.x, a);
      adam_update(g.y, p.y, m.y, v.y, a);
      adam_update(g.z, p.z, m.z, v.z, a);
      adam_update(g.w, p.w, m.w, v.w, a);
      p4[i] = p;
      m4[i] = m;
      v4[i] = v;
    }
    done = n4 * 4;
  }
  for (long long i = done + tid; i < t.n; i += stride) {
    float p = t.p[i], m = t.m[i], v = t.v[i];
    adam_update(t.g[i], p, m, v, a);
    t.p[i] = p;
    t.m[i] = m;
    t.v[i] = v;
  }
}

}  // namespace xl

using namespace xl;

extern "C" int xl_adamw_step(void* stream, const XlAdamWArgs* a) {
  if (!a || a->count < 1 || a->count > XL_ADAMW_MAX_TENSORS || !a->step) {
    set_error("xl_adamw_step: bad arguments");
    return XL_EINVAL;
  }
  long long nmax = 0;
  for (int i = 0; i < a->count; ++i) {
    const XlAdamWTensor& t = a->t[i];
    if (t.n < 0 || (t.n > 0 && (!t.p || !t.g || !t.m || !t.v))) {
      set_error("xl_adamw_step: tensor %d has a null pointer", i);
      return XL_EINVAL;
    }
    if (t.n > nmax) nmax = t.n;
  }
  if (nmax == 0) return XL_OK;
  long long blocks = (nmax / 4 + 255) / 256;
  const long long cap = (152LL * 8 + a->count - 1) / a->count;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  AdamKernelArgs k;
  k.a = *a;
  adamw_kernel<<<dim3((unsigned)blocks, a->count), 256, 0, (cudaStream_t)stream>>>(k);
  XL_CHECK_LAUNCH("adamw_kernel");
  return XL_OK;
}
