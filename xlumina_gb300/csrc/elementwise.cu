// Stand-alone per-pixel kernels: a Jones program applied outside a
// propagator (masks whose result the caller reads directly).
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
    const int row = (int)(i / p.nx), col = (int)(i % p.nx);
    PixelCtx px{row, col, i, b};
    apply_prog(p.prog, e, px);
    const long long o = (long long)b * p.obs + i;
    p.out[0][o] = e[0];
    if (p.C > 1) p.out[1][o] = e[1];
    if (p.C > 2) p.out[2][o] = e[2];
  }
}

cudaError_t elem_upload_twiddles(const float2* host) {
  return cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
}

}  // namespace xl

using namespace xl;

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
