// Rayleigh-Sommerfeld propagation (scalar RS and vectorial VRS): the C ABI
// entry points.  The reference (wave_optics.py:281-289) zero-pads the N x N
// field to (2N-1)^2, multiplies fft2(U) by fft2(H) and crops [N-1:, N-1:];
// the kernels (rs_kernels.cuh) run the same linear convolution on a 2Q x 2Q
// grid, Q the next power of two >= N, in three passes.
#include <math.h>

#include <mutex>

#include "rs_host.h"

namespace xl {

#define XL_RS_DISPATCH(LOGQ_VAR, CALL)          \
  switch (LOGQ_VAR) {                           \
    case 4: return CALL(4);                     \
    case 5: return CALL(5);                     \
    case 6: return CALL(6);                     \
    case 7: return CALL(7);                     \
    case 8: return CALL(8);                     \
    case 9: return CALL(9);                     \
    case 10: return CALL(10);                   \
    case 11: return CALL(11);                   \
    case 12: return CALL(12);                   \
    default: break;                             \
  }

}  // namespace xl

using namespace xl;


extern "C" size_t xl_rs_spectrum_bytes(int ny, int nx) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE) return 0;
  const size_t P = (size_t)2 << rs_logq(ny, nx);
  return P * P * sizeof(float2);
}

extern "C" size_t xl_rs_spectrum_work_bytes(int ny, int nx) { return xl_rs_spectrum_bytes(ny, nx); }

extern "C" size_t xl_rs_work_bytes(int batch, int comps, int ny, int nx) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE || batch < 1 || comps < 1) return 0;
  const size_t P = (size_t)2 << rs_logq(ny, nx);
  return (size_t)batch * comps * ny * P * sizeof(float2);
}

static int transfer_spectrum(const char* what, void* stream, int ny, int nx, const double* offx,
                             const double* offy, double z, const double* zp, int count, long long sstride,
                             double wavelength, double scale, void* spectrum, void* work, int dz) {
  if (ny < 2 || nx < 2 || ny > XL_MAX_SIDE || nx > XL_MAX_SIDE) {
    set_error("%s: field side out of range (2..%d): %d x %d", what, XL_MAX_SIDE, ny, nx);
    return XL_EINVAL;
  }
  if (!offx || !offy || !spectrum || !work) {
    set_error("%s: null pointer argument", what);
    return XL_EINVAL;
  }
  if ((!zp && !(z != 0.0)) || !(wavelength > 0.0)) {
    set_error("%s: need z != 0 and wavelength > 0 (got z=%g, wavelength=%g)", what, z, wavelength);
    return XL_EINVAL;
  }
  if (count < 1 || (count > 1 && sstride < (long long)(xl_rs_spectrum_bytes(ny, nx) / sizeof(float2)))) {
    set_error("%s: bad spectrum count %d or stride %lld", what, count, sstride);
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int lq = rs_logq(ny, nx);
  for (int e = 0; e < count; ++e) {
    float2* spec = (float2*)spectrum + (long long)e * sstride;
    const double* zpe = zp ? zp + e : nullptr;
    int rc = XL_EUNSUPPORTED;
#define CALL(L) rc = rs_spectrum<L>(st, ny, nx, offx, offy, z, zpe, wavelength, scale, spec, (float2*)work, dz); break
    switch (lq) {
      case 4: CALL(4); case 5: CALL(5); case 6: CALL(6); case 7: CALL(7); case 8: CALL(8);
      case 9: CALL(9); case 10: CALL(10); case 11: CALL(11); case 12: CALL(12);
      default: set_error("%s: unsupported size", what);
    }
#undef CALL
    if (rc) return rc;
  }
  return XL_OK;
}

extern "C" int xl_rs_transfer_spectrum(void* stream, int ny, int nx, const double* offx,
                                       const double* offy, double z, double wavelength,
                                       double scale, void* spectrum, void* work) {
  return transfer_spectrum("xl_rs_transfer_spectrum", stream, ny, nx, offx, offy, z, nullptr, 1, 0, wavelength,
                           scale, spectrum, work, 0);
}

extern "C" int xl_rs_transfer_spectrum_dz(void* stream, int ny, int nx, const double* offx,
                                          const double* offy, double z, double wavelength,
                                          double scale, void* spectrum, void* work) {
  return transfer_spectrum("xl_rs_transfer_spectrum_dz", stream, ny, nx, offx, offy, z, nullptr, 1, 0,
                           wavelength, scale, spectrum, work, 1);
}

extern "C" int xl_rs_transfer_spectra_device_z(void* stream, int ny, int nx, const double* offx,
                                               const double* offy, const double* z, int count, double wavelength,
                                               double scale, int dz, void* spectra, long long spectrum_stride,
                                               void* work) {
  if (!z) {
    set_error("xl_rs_transfer_spectra_device_z: null distance array");
    return XL_EINVAL;
  }
  return transfer_spectrum("xl_rs_transfer_spectra_device_z", stream, ny, nx, offx, offy, 0.0, z, count,
                           spectrum_stride, wavelength, scale, spectra, work, dz ? 1 : 0);
}

static int rs_run(void* stream, const XlRsArgs* a, int stage) {
  if (!a) {
    set_error("xl_rs_propagate: null args");
    return XL_EINVAL;
  }
  if (a->ny < 2 || a->nx < 2 || a->ny > XL_MAX_SIDE || a->nx > XL_MAX_SIDE || a->batch < 1) {
    set_error("xl_rs_propagate: bad shape batch=%d ny=%d nx=%d", a->batch, a->ny, a->nx);
    return XL_EINVAL;
  }
  const bool scalar = a->comps_in == 1 && a->comps_out == 1;
  const bool vector = a->adjoint ? (a->comps_in == 3 && a->comps_out == 3)
                                 : (a->comps_in == 2 && a->comps_out == 3);
  if (!scalar && !vector) {
    set_error("xl_rs_propagate: comps_in/comps_out must be 1/1 (RS), 2/3 (VRS) or 3/3 (VRS adjoint), "
              "got %d/%d (adjoint=%d)", a->comps_in, a->comps_out, a->adjoint);
    return XL_EINVAL;
  }
  if (a->adjoint && (a->pre.nops || a->post.nops)) {
    set_error("xl_rs_propagate: the adjoint takes no fused programs");
    return XL_EINVAL;
  }
  const int nout = (a->adjoint && vector) ? 2 : a->comps_out;
  for (int c = 0; c < a->comps_in; ++c)
    if (!a->in[c]) { set_error("xl_rs_propagate: null input plane %d", c); return XL_EINVAL; }
  for (int c = 0; c < nout; ++c)
    if (!a->out[c]) { set_error("xl_rs_propagate: null output plane %d", c); return XL_EINVAL; }
  if ((!a->spectrum && !a->spectra) || !a->work) {
    set_error("xl_rs_propagate: null spectrum or workspace");
    return XL_EINVAL;
  }
  if (vector && (!a->x || !a->y || !a->z)) {
    set_error("xl_rs_propagate: VRS needs x, y and z arrays");
    return XL_EINVAL;
  }
  if (a->pre.nops < 0 || a->pre.nops > XL_MAX_OPS || a->post.nops < 0 || a->post.nops > XL_MAX_OPS) {
    set_error("xl_rs_propagate: op program too long");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  RsLaunch p;
  p.B = a->batch; p.cin = a->comps_in; p.cout = a->comps_out; p.ny = a->ny; p.nx = a->nx;
  for (int c = 0; c < 3; ++c) {
    p.in[c] = (const float2*)a->in[c];
    p.out[c] = (float2*)a->out[c];
  }
  p.ibs = a->in_bstride; p.obs = a->out_bstride;
  p.x = a->x; p.y = a->y; p.z = a->z;
  p.spec = (const float2*)a->spectrum; p.sstride = a->spectrum_stride; p.sidx = a->spectrum_index;
  p.specs = (const float2* const*)a->spectra;
  p.work = (float2*)a->work;
  p.pre = a->pre; p.post = a->post;
  p.adjoint = a->adjoint ? 1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  const int lq = rs_logq(a->ny, a->nx);
#define CALL(L) rs_propagate<L>(st, p, stage)
  XL_RS_DISPATCH(lq, CALL)
#undef CALL
  set_error("xl_rs_propagate: unsupported size");
  return XL_EUNSUPPORTED;
}

extern "C" int xl_rs_propagate(void* stream, const XlRsArgs* a) { return rs_run(stream, a, -1); }

extern "C" int xl_rs_stage(void* stream, const XlRsArgs* a, int stage) {
  if (stage < 0 || stage > 2) {
    set_error("xl_rs_stage: stage must be 0, 1 or 2 (got %d)", stage);
    return XL_EINVAL;
  }
  return rs_run(stream, a, stage);
}

// ---------------------------------------------------------------------------
// Allocation-free RS / VRS.
//
// Some callers of this library cannot call cudaMalloc.  Two examples: a host
// program that reserves all device memory for its own pool at start-up (a
// later cudaMalloc fails or fragments the pool), and a loop that drives
// optical hardware frame by frame, which cannot take the implicit device
// synchronisation and unbounded latency that cudaMalloc / cudaFree can cause.
// xl_rs_propagate_noalloc serves them.  It runs exactly the passes of
// xl_rs_propagate, but its workspace is the fixed device array below, so the
// caller passes only inputs (fields, transfer spectrum, coordinates) and
// outputs, and the call allocates no device memory.
//
// The array holds XL_RS_NOALLOC_MAX_WORK_BYTES on every GPU that loads the
// library, until the process exits.  All calls share it and it keeps the last
// call's contents; nothing in it needs clearing, because the first pass writes
// every element the later passes read.  Calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array.
static __device__ __align__(256) float2 g_rs_noalloc_scratch[XL_RS_NOALLOC_MAX_WORK_BYTES / sizeof(float2)];

static std::mutex g_noalloc_mu;
static float2* g_noalloc_ptr[256];

// Device address of the scratch array for the current device.  The array's
// name in host code is only a stand-in for the symbol, so the address is
// looked up once per device, with that device current.  The lookup also
// loads this file's device module, which is when the runtime allocates the
// array.
static cudaError_t noalloc_lookup(float2** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_rs_noalloc_scratch)) != cudaSuccess) return e;
    g_noalloc_ptr[dev] = (float2*)p;
  }
  if (out) *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

// Run at every device's set-up (xl_init, or the first call of any entry
// point), so that the array exists from then on: a host that hands the rest
// of device memory to its own pool afterwards still has it.
static cudaError_t noalloc_setup(const float2*) { return noalloc_lookup(nullptr); }
static const bool g_noalloc_registered = register_device_tables(&noalloc_setup, nullptr);

extern "C" int xl_rs_propagate_noalloc(void* stream, const XlRsArgs* a) {
  if (!a) {
    set_error("xl_rs_propagate_noalloc: null args");
    return XL_EINVAL;
  }
  const size_t need = xl_rs_work_bytes(a->batch, a->comps_out, a->ny, a->nx);
  if (need == 0) {
    set_error("xl_rs_propagate_noalloc: bad shape batch=%d comps_out=%d ny=%d nx=%d", a->batch,
              a->comps_out, a->ny, a->nx);
    return XL_EINVAL;
  }
  if (need > (size_t)XL_RS_NOALLOC_MAX_WORK_BYTES) {
    set_error("xl_rs_propagate_noalloc: this call needs %zu bytes of scratch, the fixed limit is %llu "
              "(e.g. one 1024x1024 VRS field or one 2048x2048 scalar field); use xl_rs_propagate with a "
              "caller workspace for larger work",
              need, (unsigned long long)XL_RS_NOALLOC_MAX_WORK_BYTES);
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  int dev = 0, sdev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "xl_rs_propagate_noalloc: cudaGetDevice");
  if ((e = cudaStreamGetDevice((cudaStream_t)stream, &sdev)) != cudaSuccess)
    return cuda_fail(e, "xl_rs_propagate_noalloc: cudaStreamGetDevice");
  if (sdev != dev) {
    set_error("xl_rs_propagate_noalloc: the stream belongs to device %d, the current device is %d", sdev, dev);
    return XL_EINVAL;
  }
  float2* scratch = nullptr;
  if ((e = noalloc_lookup(&scratch)) != cudaSuccess)
    return cuda_fail(e, "xl_rs_propagate_noalloc: cudaGetSymbolAddress");
  XlRsArgs b = *a;
  b.work = scratch;
  return rs_run(stream, &b, -1);
}
