// Chirp-z propagation (scalar CZT, vectorial VCZT, the high-NA focus): the C
// ABI entry points.  The reference (wave_optics.py:333-460) runs Bluestein's
// algorithm along y and then along x; the kernels (czt_kernels.cuh) run the x
// transform over rows with the fused prologue and the y transform over
// column tiles with the fused epilogue.
#include <cooperative_groups.h>
#include <math.h>

#include "czt_host.h"
#include "xlgb.h"

namespace xl {

#define XL_CZT_DISPATCH(LL, FN, ...)          \
  switch (LL) {                               \
    case 5: return FN<5>(__VA_ARGS__);        \
    case 6: return FN<6>(__VA_ARGS__);        \
    case 7: return FN<7>(__VA_ARGS__);        \
    case 8: return FN<8>(__VA_ARGS__);        \
    case 9: return FN<9>(__VA_ARGS__);        \
    case 10: return FN<10>(__VA_ARGS__);      \
    case 11: return FN<11>(__VA_ARGS__);      \
    case 12: return FN<12>(__VA_ARGS__);      \
    case 13: return FN<13>(__VA_ARGS__);      \
    default: break;                           \
  }

static int dispatch_rows(cudaStream_t st, const CztLaunch& p, int ll) {
  XL_CZT_DISPATCH(ll, czt_rows_launch, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", ll);
  return XL_EUNSUPPORTED;
}

static int dispatch_cols(cudaStream_t st, const CztLaunch& p, int ll) {
  XL_CZT_DISPATCH(ll, czt_cols_launch, st, p)
  set_error("czt: unsupported Bluestein length 2^%d", ll);
  return XL_EUNSUPPORTED;
}

// ---------------------------------------------------------------------------
// Chirp vectors per distance (wave_optics.py:299-331, 385-460) in float64.
// Phases are carried in turns and reduced to [-1/2, 1/2] before sincospi, so
// the rounding does not grow with the large arguments (the chirp
// h[q] = W^(q-m+1)^2/2 reaches ~1e7 turns at L = 8192).  Complex powers take
// the principal branch as numpy's do: W = e^{-2 pi i dW} with dW reduced to
// [-1/2, 1/2] first.
//
// GB300 runs float64 on few units per SM, so each (entry, axis) job is spread
// over a cluster of CZ_CL CTAs.  g = fft(1/h[:m+M], L) (1/h = conj h,
// |h| = 1) is a four-step transform: with n = n1 + CZ_CL n2 and
// k = k2 + (L / CZ_CL) k1, CTA n1 transforms its decimated sequence
// x[n1 + CZ_CL n2] (length L / CZ_CL, radix 2 in its shared memory) and
// multiplies by e^{-2 pi i n1 k2 / L}; after a cluster barrier every CTA forms
// L / CZ_CL outputs as CZ_CL-point DFTs over the CTAs' results, read through
// distributed shared memory.

constexpr int CZ_CL = 8;   // CTAs per job (the portable cluster size)

__device__ __forceinline__ double turn_frac(double t) { return t - rint(t); }

__device__ __forceinline__ double2 cis_turn(double t) {
  double s, c;
  sincospi(2.0 * turn_frac(t), &s, &c);
  return make_double2(c, s);
}

__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 c64(double2 v, bool conj, double scale) {
  return make_float2((float)(v.x * scale), (float)(conj ? -v.y * scale : v.y * scale));
}

__global__ void __cluster_dims__(CZ_CL, 1, 1) __launch_bounds__(256)
    czt_chirps_kernel(const __grid_constant__ XlCztChirpArgs a) {
  extern __shared__ double2 cz_smem[];
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int b = blockIdx.y, axis = blockIdx.z, tid = threadIdx.x, nt = blockDim.x;
  const int m = axis ? a.ny : a.nx, M = axis ? a.my : a.mx;
  const int logl = axis ? a.log2_ly : a.log2_lx, L = 1 << logl;
  const int logc = logl - 3, Lc = L / CZ_CL;              // CZ_CL = 2^3
  double2* u = cz_smem;          // Lc: this CTA's decimated sequence, then its transform
  double2* tw = cz_smem + Lc;    // Lc/2 twiddles e^{-2 pi i k / Lc}
  const double z = a.z[b];
  const double Dm = a.wavelength * z / a.dx;              // wave_optics.py:313
  const double o0 = axis ? a.yout0 : a.xout0, o1 = axis ? a.yout1 : a.xout1;
  const double f1 = o0 + Dm / 2, f2 = o1 + Dm / 2;       // :320-323
  const double D1 = f1 + (M * Dm + f2 - f1) / (2 * M);   // :435-437
  const double D2 = f2 + (M * Dm + f2 - f1) / (2 * M);
  const double dW = turn_frac((D2 - D1) / (M * Dm));     // W = e^{-2 pi i dW}
  const double dA = turn_frac(D1 / Dm);                  // A = e^{+2 pi i dA}
  const int hlen = (M > m ? M - 1 : m - 1) + m;          // h over q = -m+1 .. max(M-1, m-1)
  const int cnt = (m + M < hlen) ? m + M : hlen;         // h[:mp + 1]
  for (int k = tid; k < Lc / 2; k += nt) {
    double s, c;
    sincospi(-2.0 * k / Lc, &s, &c);
    tw[k] = make_double2(c, s);
  }
  for (int n2 = tid; n2 < Lc; n2 += nt) {
    const int q = rank + CZ_CL * n2;
    double2 v = make_double2(0.0, 0.0);
    if (q < cnt) {
      const double e = (double)(q - m + 1) * (double)(q - m + 1) * 0.5;
      v = cis_turn(dW * e);                              // conj(h[q]) = e^{+2 pi i dW e}
    }
    u[__brev((unsigned)n2) >> (32 - logc)] = v;
  }
  __syncthreads();
  for (int st = 0; st < logc; ++st) {
    const int half = 1 << st;
    for (int i = tid; i < Lc / 2; i += nt) {
      const int pos = i & (half - 1);
      const int ia = ((i >> st) << (st + 1)) + pos, ib = ia + half;
      const double2 t = dmul(tw[pos << (logc - 1 - st)], u[ib]);
      const double2 va = u[ia];
      u[ia] = make_double2(va.x + t.x, va.y + t.y);
      u[ib] = make_double2(va.x - t.x, va.y - t.y);
    }
    __syncthreads();
  }
  if (rank)
    for (int k2 = tid; k2 < Lc; k2 += nt) {
      double s, c;
      sincospi(-2.0 * (double)(rank * k2) / L, &s, &c);
      u[k2] = dmul(u[k2], make_double2(c, s));
    }
  __shared__ double2 w8[CZ_CL];   // e^{-2 pi i j / 8}
  if (tid < CZ_CL) {
    double s, c;
    sincospi(-2.0 * tid / CZ_CL, &s, &c);
    w8[tid] = make_double2(c, s);
  }
  cluster.sync();   // every CTA's transform is complete and visible to the cluster
  const bool adj = a.adjoint != 0;
  float2* g = (float2*)(axis ? a.g_y : a.g_x) + (long long)b * L;
  {
    for (int t = tid; t < Lc; t += nt) {   // outputs flat = rank Lc + t: k2 = flat / 8, k1 = flat % 8
      const int flat = rank * Lc + t, k2 = flat >> 3, k1 = flat & 7;
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll
      for (int r = 0; r < CZ_CL; ++r) {
        const double2* ru = cluster.map_shared_rank(u, r);
        const double2 y = dmul(ru[k2], w8[(r * k1) & 7]);
        acc.x += y.x;
        acc.y += y.y;
      }
      g[k2 + Lc * k1] = c64(acc, adj, 1.0);
    }
  }
  // pre[n] = A^-n h[m-1+n]; post[l] = h[m-1+l] e^{-2 pi i lf_l (1/2 - m/2) / Dm} / L
  // (wave_optics.py:404, 448-458); the adjoint stores conj(post) L and conj(pre) / L.
  float2* pre = (float2*)(axis ? a.pre_y : a.pre_x);
  float2* post = (float2*)(axis ? a.post_y : a.post_x);
  const double invL = 1.0 / L;
  float2* fpre = adj ? post + (long long)b * m : pre + (long long)b * m;
  for (int n = rank * nt + tid; n < m; n += CZ_CL * nt) {
    const double e = (double)n * (double)n * 0.5;
    const double2 v = cis_turn(turn_frac(-dA * n) + turn_frac(-dW * e));
    fpre[n] = adj ? c64(v, true, invL) : c64(v, false, 1.0);
  }
  float2* fpost = adj ? pre + (long long)b * M : post + (long long)b * M;
  for (int l = rank * nt + tid; l < M; l += CZ_CL * nt) {
    const double e = (double)l * (double)l * 0.5;
    const double lf = (double)l / M * (D2 - D1) + D1;
    const double2 v = cis_turn(turn_frac(-dW * e) + turn_frac(-lf * (0.5 - m / 2.0) / Dm));
    fpost[l] = adj ? c64(v, true, 1.0) : c64(v, false, invL);
  }
  if (axis == 0 && rank == 0 && tid == 0)
    ((float2*)a.cte)[b] = make_float2((float)(z * a.dx * a.dy * a.wavelength), 0.f);
  cluster.sync();   // no CTA leaves while another still reads its shared memory
}

}  // namespace xl

using namespace xl;

extern "C" int xl_czt_chirps(void* stream, const XlCztChirpArgs* a) {
  if (!a || a->batch < 1 || a->nx < 2 || a->ny < 2 || a->mx < 2 || a->my < 2) {
    set_error("xl_czt_chirps: bad shape");
    return XL_EINVAL;
  }
  if (a->log2_lx < 5 || a->log2_lx > 13 || a->log2_ly < 5 || a->log2_ly > 13 ||
      (1 << a->log2_lx) < a->nx + a->mx || (1 << a->log2_ly) < a->ny + a->my) {
    set_error("xl_czt_chirps: Bluestein lengths 2^%d, 2^%d must be in 32..8192 and exceed m + M - 1",
              a->log2_lx, a->log2_ly);
    return XL_EINVAL;
  }
  if (!a->z || !a->pre_x || !a->g_x || !a->post_x || !a->pre_y || !a->g_y || !a->post_y || !a->cte ||
      !(a->wavelength > 0) || a->dx == 0.0) {
    set_error("xl_czt_chirps: null pointer, wavelength <= 0 or dx = 0");
    return XL_EINVAL;
  }
  if (int rc = ensure_init()) return rc;
  if (a->batch > 65535) {
    set_error("xl_czt_chirps: at most 65535 entries per call");
    return XL_EINVAL;
  }
  const int ll = a->log2_lx > a->log2_ly ? a->log2_lx : a->log2_ly;
  const size_t sm = (size_t)3 * ((1 << ll) / CZ_CL) / 2 * sizeof(double2);
  cudaError_t e = allow_smem(czt_chirps_kernel, sm);
  if (e != cudaSuccess) return cuda_fail(e, "czt_chirps smem");
  czt_chirps_kernel<<<dim3(CZ_CL, a->batch, 2), 256, sm, (cudaStream_t)stream>>>(*a);
  XL_CHECK_LAUNCH("czt_chirps_kernel");
  return XL_OK;
}

extern "C" size_t xl_czt_work_bytes(int batch, int comps, int ny, int mx) {
  if (batch < 1 || comps < 1 || ny < 1 || mx < 1) return 0;
  const size_t mxp = ((size_t)mx + 31) / 32 * 32;  // column tiles may round mx up (tile widths divide 32)
  return (size_t)batch * comps * ny * mxp * sizeof(float2);
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
                         a->comps_out >= 1 && a->comps_out <= 3 &&
                         (a->comps_out >= a->comps_in || a->pre.nops > 0));   // a program may fold components
  if (!ok_modes) {
    set_error("xl_czt: mode %d with comps %d -> %d is not supported", a->mode, a->comps_in, a->comps_out);
    return XL_EINVAL;
  }
  const int llx = a->log2_lx, lly = a->log2_ly;
  if (llx < 5 || llx > 13 || lly < 5 || lly > 13 || (1 << llx) < a->nx + a->mx ||
      (1 << lly) < a->ny + a->my) {
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
  if (a->mode == XL_CZT_PLAIN && (a->z_batch || a->cte_batch)) {
    set_error("xl_czt: per-entry distances apply to the scalar and vectorial transforms only");
    return XL_EINVAL;
  }
  if ((a->f_in || a->f_out) && (a->mode == XL_CZT_PLAIN || a->z_batch)) {
    set_error("xl_czt: transfer planes apply to one distance in the scalar and vectorial modes");
    return XL_EINVAL;
  }
  if (!a->z_batch != !a->cte_batch) {
    set_error("xl_czt: z_batch and cte_batch go together");
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
  const int wt = czt_tile_w(lly);
  p.mxp = (a->mx + wt - 1) / wt * wt;
  p.lw = ilog2_ceil(wt);
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
  p.zb = a->z_batch;
  p.cteb = (const float2*)a->cte_batch;
  p.fin = (const float2*)a->f_in;
  p.fout = (const float2*)a->f_out;
  cudaStream_t st = (cudaStream_t)stream;
  if (stage < 0 || stage == 0)
    if (int rc = dispatch_rows(st, p, llx)) return rc;
  if (stage < 0 || stage == 1)
    if (int rc = dispatch_cols(st, p, lly)) return rc;
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
