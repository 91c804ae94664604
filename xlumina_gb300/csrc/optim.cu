// AdamW for the optimisation tables: every float32 parameter tensor of a
// step updated in one launch, in one pass over memory (read p, g, m, v;
// write p, m, v), with the step count in device memory so the update can be
// recorded in a CUDA graph.
//
// The update is torch.optim.AdamW's (decoupled weight decay):
//   p *= 1 - lr wd;  m += (1 - b1)(g - m);  v = b2 v + (1 - b2) g^2;
//   p -= lr / (1 - b1^t) * m / (sqrt(v) / sqrt(1 - b2^t) + eps),
// t being the step count after its increment.
#include "internal.h"
#include "xlgb.h"

namespace xl {

struct AdamKernelArgs {
  XlAdamWArgs a;
};

__global__ void __launch_bounds__(256) adamw_kernel(const __grid_constant__ AdamKernelArgs k) {
  const XlAdamWTensor& t = k.a.t[blockIdx.y];
  const float s = *k.a.step;
  const float b1 = k.a.beta1, b2 = k.a.beta2;
  const float bc1 = 1.f - powf(b1, s), bc2 = 1.f - powf(b2, s);
  const float step_size = k.a.lr / bc1;
  const float rbc2 = 1.f / sqrtf(bc2);
  const float decay = 1.f - k.a.lr * k.a.weight_decay;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < t.n;
       i += (long long)gridDim.x * blockDim.x) {
    const float g = t.g[i];
    float m = t.m[i], v = t.v[i], p = t.p[i];
    p *= decay;
    m = fmaf(1.f - b1, g - m, m);
    v = fmaf(b2, v, (1.f - b2) * g * g);
    const float denom = sqrtf(v) * rbc2 + k.a.eps;
    p -= step_size * (m / denom);
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
  long long blocks = (nmax + 255) / 256;
  const long long cap = (152LL * 8 + a->count - 1) / a->count;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  AdamKernelArgs k;
  k.a = *a;
  adamw_kernel<<<dim3((unsigned)blocks, a->count), 256, 0, (cudaStream_t)stream>>>(k);
  XL_CHECK_LAUNCH("adamw_kernel");
  return XL_OK;
}
