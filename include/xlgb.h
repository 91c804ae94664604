/*
 * xlgb.h -- C ABI of libxlgb, the GB300 (sm_103a) light-propagation library
 * behind the xlumina_gb300 Python package.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * handle (cudaStream_t passed as void*), launches on that stream and returns
 * without synchronising.  Complex fields are complex64: interleaved
 * (re, im) float32 pairs, row-major planes of ny rows by nx columns.  The
 * library allocates no device memory: callers pass every output and
 * workspace buffer, sized with the *_bytes() helpers.
 *
 * Return value: XL_OK (0) or a negative XL_E* code; xl_last_error() gives a
 * one-line description of the most recent failure on the calling thread.
 *
 * The reference (XLuminA, pure Python on jax) has no native interface: each
 * entry point below replaces a jitted jax function of its Python API, cited
 * next to the declaration as file:line inside the XLuminA repository.
 */
#ifndef XLGB_H_
#define XLGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XL_OK 0
#define XL_EINVAL (-1)
#define XL_ENOMEM (-2)
#define XL_ETIMEOUT (-3)
#define XL_ECUDA (-4)
#define XL_EUNSUPPORTED (-5)

#define XL_MAX_OPS 8
#define XL_MAX_FFT 8192   /* longest FFT any kernel runs (RS transfer spectrum: 2Q) */
#define XL_MAX_SIDE 4096  /* longest field side (Q <= 4096) */

/* Per-pixel operations fused into the first / last pass of a propagator
 * (or run alone by xl_apply_ops).  Parameter i is a per-pixel float32 plane
 * when bit i of pmask is set (ptr[i], batch stride pbstride elements),
 * otherwise the scalar sval[i]. */
enum {
  XL_OP_NONE = 0,
  XL_OP_PHASE = 1,     /* scalar SLM, optical_elements.py:76-103: e0 *= exp(i p0) */
  XL_OP_SSLM = 2,      /* sSLM, optical_elements.py:186-222: e0 *= exp(i p0), e1 *= exp(i p1) */
  XL_OP_SSLM_AMP = 3,  /* sSLM_with_amplitude, :224-264: also *= p2, p3 */
  XL_OP_LCD = 4,       /* LCD retarder (eta=p0, theta=p1), :266-305, Ez kept */
  XL_OP_LP = 5,        /* linear_polarizer (alpha=p0), :307-332, Ez zeroed */
  XL_OP_SEPMASK = 6,   /* separable mask colfac[col]*rowfac[row] with FP64 pupil test
                          (thin lens, :678-703); sval[0] != 0 zeroes Ez (vector lens) */
  XL_OP_CMUL = 7,      /* multiply all components by a complex64 plane ptr[0] */
  XL_OP_HIGHNA = 8,    /* high-NA objective lens, optical_elements.py:515-594: ptr[0], ptr[1]
                          float64 x, y; dval[0] radius, dval[1] focal length, dval[2]
                          sin(theta_max), dval[3] 1/radius^2; Ez derived from Ex, Ey, output
                          (Ex, Ey, Ez).  ptr[2] (optional): the 6 coefficient planes from
                          xl_highna_coefficients, plane stride pbstride (ny*nx) */
  XL_OP_HIGHNA_EZ = 9  /* the same lens keeping only its Ez row: e0 = K20 Ex + K21 Ey, e1 = e2 = 0
                          (the focus a loss of |Ez|^2 alone needs, small_area_hybrid on the
                          Ez detector, hybrid_sharp_optical_table.py); same parameters */
};

typedef struct {
  int kind;
  int pmask;
  const void* ptr[4];
  float sval[4];
  long long pbstride;
  double dval[4];
} XlOp;

typedef struct {
  int nops;
  XlOp ops[XL_MAX_OPS];
} XlProg;

const char* xl_last_error(void);
int xl_version(void);

/* sizeof of the argument struct of that name ("XlCztArgs", ...), 0 if unknown:
 * lets a binding check its mirrors of the structs against this build. */
size_t xl_struct_size(const char* name);

/* Number of bounded waits (on TMA-copy barriers) that ran out of iterations
 * since the last reset, on the current device; such a launch records the
 * event and returns without hanging, its output is not valid.  Synchronous. */
int xl_device_timeouts(unsigned int* count, int reset);

/* Non-blocking check for kernel errors: *flag = 1 if a kernel of this
 * library had a bounded wait run out (its output is not valid) since the
 * last clear, on any device, else 0.  Kernels raise a word in mapped host
 * memory, so no device synchronisation is needed; work still queued is not
 * reflected, so read it after synchronising with the launches of interest.
 * clear != 0 resets the word.  The Python package checks it at the start of
 * every propagation call and after every synchronising step, and raises
 * (XL_ETIMEOUT). */
int xl_device_status(unsigned int* flag, int clear);

/* Limit of the kernels' bounded waits on their TMA copies, in ns, on the
 * current device (default 1e9, one second).  0 makes every such wait give up
 * at once: a test setting that takes the timeout path (the kernel lets its
 * copy in flight land, raises the status word and returns) without a fault
 * or a hang. */
int xl_set_wait_limit(unsigned long long ns);

/* Device address of page-locked host memory (cudaHostAlloc'd, or
 * registered with cudaHostRegister) that the current device can reach
 * directly: *dev = the pointer kernels use.  XL_EINVAL for any other pointer
 * (pageable or device memory).  Output planes of xl_rs_propagate may be such
 * host memory: the last pass then stores the propagated field straight over
 * the host link, with no separate device-to-host copy (the reference returns
 * device arrays that a caller copies with jax.device_get / np.asarray,
 * wave_optics.py:281-297). */
int xl_host_mapped(const void* host, void** dev);

/* Upload the twiddle tables to the current device.  Called once per device
 * before the first launch (every entry point calls it lazily as well). */
int xl_init(void);

/* ---- kernel variants ----------------------------------------------------
 * Some passes have several kernels for one transform length (thread shape,
 * columns per thread, barrier grouping).  All variants of a pass give the
 * same results to float32 rounding; which one is fastest is measured per
 * GPU by the package's autotuner, which selects it here.  The choice is
 * process-wide and read at every launch.  No counterpart in the reference:
 * its transforms are XLA's (wave_optics.py:281-289, 385-460). */
enum {
  XL_PASS_RS_COLS = 0,   /* RS / VRS column pass (forward FFT, spectrum, inverse FFT) */
  XL_PASS_CZT_ROWS = 1,  /* chirp-z x transform over rows */
  XL_PASS_CZT_COLS = 2,  /* chirp-z y transform over column tiles */
  XL_PASS_RS_ROWS = 3,   /* RS / VRS forward and inverse row passes */
  XL_NUM_PASSES = 4
};
/* Variants available for `pass` at transform length 2^log2_len (>= 1; 0 if
 * the pass or length is unknown).  Variant 0 is the default kernel shape
 * except at 4096 points: the RS column pass defaults to variant 8 (the
 * one-line kernel, persistent), the chirp-z x transform to variant 3
 * (registers sized for two CTAs per SM) and the chirp-z y transform to
 * variant 1 (persistent).  The others are the alternatives the autotuner
 * measures against the default.  RS column pass: 0 one line per thread,
 * 1-2 two lines per thread (packed FP32), 3-7 prefetching, barrier groups,
 * CTA shapes, 8 persistent one line, 9 (4096 points) radix 64, 10 (4096
 * points) as 8 with each unit's spectrum values kept in Tensor Memory.  Chirp-z x
 * transform: 0 the stage capped for two CTAs per SM, 1 for one, 2 no
 * stage, 3 as 0 with registers for two CTAs, 4 (4096 points, three
 * components) one component group, two CTAs per SM.  Chirp-z y transform:
 * 0 one CTA per column tile and entry, 1 persistent. */
int xl_kernel_variant_count(int pass, int log2_len);
/* Select variant `variant` (< the count) for later launches. */
int xl_set_kernel_variant(int pass, int log2_len, int variant);
/* The variant launches use now (negative XL_E* code for a bad argument). */
int xl_get_kernel_variant(int pass, int log2_len);

/* ---- Rayleigh-Sommerfeld (RS / VRS) ----------------------------------- */

/* The spectrum of dH/dz, the z-derivative of the same impulse response
 * (same arguments and layout as xl_rs_transfer_spectrum).  Propagating with
 * it gives d(output)/dz, the gradient with respect to a distance that jax.grad
 * takes through RS_propagation_jit (z is traced there, wave_optics.py:281-297). */
int xl_rs_transfer_spectrum_dz(void* stream, int ny, int nx, const double* offx, const double* offy,
                               double z, double wavelength, double scale, void* spectrum, void* work);

/* Transfer spectra (dz = 0) or their z-derivatives (dz = 1) for `count`
 * distances held in device memory (z[0 .. count-1], float64), written
 * spectrum_stride complex64 elements apart: what xl_rs_transfer_spectrum /
 * xl_rs_transfer_spectrum_dz give per distance, without reading the distances
 * back to the host, so that a distance being optimised stays on the device
 * and the call can be captured in a CUDA graph.  A distance of 0 gives NaN at
 * the zero offset, as the reference's formula (wave_optics.py:291-297). */
int xl_rs_transfer_spectra_device_z(void* stream, int ny, int nx, const double* offx, const double* offy,
                                    const double* z, int count, double wavelength, double scale, int dz,
                                    void* spectra, long long spectrum_stride, void* work);

/* Bytes of one transfer spectrum for an ny x nx field: (2Q)^2 complex64,
 * Q = next power of two >= max(ny, nx). */
size_t xl_rs_spectrum_bytes(int ny, int nx);
/* Bytes of workspace xl_rs_transfer_spectrum needs. */
size_t xl_rs_spectrum_work_bytes(int ny, int nx);

/* Transfer spectrum of the RS impulse response, wave_optics.py:291-297 and
 * the fft2(H) of :288.  offx / offy: device float64 arrays of length 2Q
 * holding the impulse-response offsets in wrapped order (entry d mod 2Q
 * holds the offset of index distance d, |d| <= n-1, built from the
 * reference's reflect-padded grid, :265-279); scale multiplies the spectrum
 * (dx*dy / (2Q)^2 for a propagator).  Output in the layout
 * xl_rs_propagate reads. */
int xl_rs_transfer_spectrum(void* stream, int ny, int nx, const double* offx, const double* offy,
                            double z, double wavelength, double scale, void* spectrum, void* work);

typedef struct {
  int batch;          /* fields in this call */
  int comps_in;       /* 1: scalar field; 2: (Ex, Ey) */
  int comps_out;      /* 1: scalar; 3: (Ex, Ey, Ez), Ez derived from Ex, Ey (VRS) */
  int ny, nx;
  const void* in[3];  /* complex64 input planes per component */
  long long in_bstride;
  void* out[3];       /* complex64 output planes per component */
  long long out_bstride;
  const double* x;    /* device coordinates, nx (VRS Ez derivation) */
  const double* y;    /* device coordinates, ny */
  const double* z;    /* device, one distance per batch entry (VRS Ez derivation) */
  const void* spectrum;        /* stacked transfer spectra (or NULL when `spectra` is set) */
  long long spectrum_stride;   /* complex64 elements between spectra */
  const int* spectrum_index;   /* device, spectrum used by each batch entry; NULL: entry 0 */
  void* work;                  /* >= xl_rs_work_bytes(batch, comps_out, ny, nx) */
  XlProg pre;                  /* fused before the first pass */
  XlProg post;                 /* fused after the last pass */
  int adjoint;                 /* 1: adjoint propagation (conjugate spectrum).  Scalar: 1 -> 1.
                                  VRS: comps_in = comps_out = 3 gradients (Ex, Ey, Ez) in; the Ez
                                  gradient is folded back into Ex, Ey with the weights X/r, Y/r of
                                  the forward Ez derivation; outputs out[0], out[1], and out[2]
                                  (optional) the propagated Ez gradient before the fold.  pre/post
                                  must be empty. */
  const void* const* spectra;  /* optional device array of `batch` spectrum pointers, one per batch
                                  entry (entries of different distances need no stacked copy);
                                  when set it replaces spectrum / spectrum_stride / spectrum_index */
} XlRsArgs;

size_t xl_rs_work_bytes(int batch, int comps, int ny, int nx);

/* RS / VRS propagation: RS_propagation_jit, wave_optics.py:281-289, and
 * VRS_propagation_jit, vectorized_optics.py:364-373, with the VRS Ez of
 * vectorized_optics.py:258-261.  Output = crop(ifft2(fft2(pad(E)) * S)),
 * S the transfer spectrum (its scale includes dx*dy / (2Q)^2). */
int xl_rs_propagate(void* stream, const XlRsArgs* args);

/* One pass of xl_rs_propagate, for callers that time or overlap the passes:
 * stage 0 = prologue + row spectra, 1 = column convolution (in place),
 * 2 = inverse rows + crop + epilogue.  Running 0, 1, 2 in order on one stream
 * equals xl_rs_propagate. */
int xl_rs_stage(void* stream, const XlRsArgs* args, int stage);

/* Allocation-free variant of xl_rs_propagate, for callers that cannot call
 * cudaMalloc (a host that reserves all device memory for its own pool, or a
 * hardware-driving loop that cannot take cudaMalloc's implicit
 * synchronisation).  No counterpart in the reference.  args->work is
 * ignored: the workspace is a fixed device array of
 * XL_RS_NOALLOC_MAX_WORK_BYTES inside the library, held on every GPU that
 * loads it until exit.  Calls needing more scratch than that
 * (xl_rs_work_bytes) fail with XL_EINVAL.  The array is created on a device
 * by the device's set-up: xl_init(), or the first call of any entry point
 * there.  A host that hands device memory to its own pool calls xl_init() on
 * each device before reserving it; that set-up (or the first call) must also
 * come before any stream capture.  The stream must belong to the current
 * device (XL_EINVAL otherwise).  All calls share the array and it keeps the
 * last call's contents: calls whose work overlaps on the GPU (other streams,
 * other host threads) race. */
#define XL_RS_NOALLOC_MAX_WORK_BYTES (64ull << 20)
int xl_rs_propagate_noalloc(void* stream, const XlRsArgs* args);

/* ---- Bare line transforms ----------------------------------------------
 * Unnormalised complex64 FFTs of `lines` contiguous lines of 2^log2_len
 * points (line l at in + l * 2^log2_len), forward (dir = -1: sum x[n]
 * e^{-2 pi i n k / L}) or inverse (dir = +1, no 1/L), in -> out.  In place
 * (in == out) for log2_len >= 5.  log2_len 0..13.  Replaces the
 * jnp.fft.fft / jnp.fft.ifft calls of the reference's Bluestein helpers
 * compute_fft and Bluestein_method (wave_optics.py:385-460, :401, :406,
 * :408); the propagators fuse their transforms instead. */
int xl_fft_lines(void* stream, int log2_len, long long lines, int dir, const void* in, void* out);

/* ---- Chirp-z (CZT / VCZT / high-NA focus) ----------------------------- */

enum {
  XL_CZT_SCALAR = 0,  /* CZT_jit, wave_optics.py:333-357: F * field -> B_y B_x -> F0 * cte */
  XL_CZT_VECTOR = 1,  /* VCZT, vectorized_optics.py:321-384: Ez = (Ex X/r + Ey Y/r) z/r, then as scalar */
  XL_CZT_PLAIN = 2    /* CZT_for_high_NA_jit, wave_optics.py:359-371: no transfer functions, * cte */
};

typedef struct {
  int batch, comps_in, comps_out, mode;
  int ny, nx;            /* input plane */
  int my, mx;            /* output plane */
  int log2_lx, log2_ly;  /* Bluestein lengths (>= nx + mx, >= ny + my) */
  const void* in[3];
  long long in_bstride;
  void* out[3];
  long long out_bstride;
  const double* x;       /* device float64 coordinates: nx, ny, mx, my */
  const double* y;
  const double* xout;
  const double* yout;
  double z, wavelength;
  double cte_re, cte_im; /* constant output factor */
  /* complex64 chirp data per axis (wave_optics.py:385-460, float64 on the host):
   * pre[n] = A^-n h[m-1+n] (m values); g = fft(1/h[:m+M], L) in natural
   * order; post[l] = h[m-1+l] e^{-i 2 pi l_f (1/2 - m/2)/Dm} / L */
  const void* pre_x;
  const void* g_x;
  const void* post_x;
  const void* pre_y;
  const void* g_y;
  const void* post_y;
  void* work;            /* >= xl_czt_work_bytes(batch, comps_out, ny, mx) */
  XlProg pre;            /* fused before the first pass (masks, XL_OP_HIGHNA) */
  int adjoint;           /* 1: conjugate transpose of the forward chirp-z.  The input plane
                            (ny, nx, x, y) is the forward's output grid and the output plane
                            (my, mx, xout, yout) its input grid; chirp vectors are the adjoint
                            ones (pre' = conj(post) L, g' = conj(g), post' = conj(pre) / L);
                            z, wavelength and cte as for the forward.  VCZT: 3 gradients in,
                            the Ez gradient folded into out[0], out[1]. */
  /* Per-entry distances (XL_CZT_SCALAR and XL_CZT_VECTOR; NULL: every entry uses z).
   * Entry b propagates over z_batch[b] (device float64) with its own chirp vectors,
   * packed entry after entry: pre_x + b nx, g_x + b 2^log2_lx, post_x + b mx, and the
   * same for y; cte_batch[b] (device complex64) replaces cte_re, cte_im (the adjoint
   * conjugates it, as it does cte). */
  const double* z_batch;
  const void* cte_batch;
  /* Optional (one distance only, scalar and vectorial modes): the transfer
   * function evaluated once on this call's input plane (f_in, ny x nx) and
   * output plane (f_out, my x mx), complex64 as xl_czt_transfer_plane writes
   * it; NULL: evaluated per pixel in the kernels.  Both are the forward's
   * H(z, X, Y) at the call's own coordinates (the adjoint conjugates). */
  const void* f_in;
  const void* f_out;
} XlCztArgs;

size_t xl_czt_work_bytes(int batch, int comps, int ny, int mx);

/* Chirp-z propagation: CZT (wave_optics.py:233-263), VCZT
 * (vectorized_optics.py:321-361) and VCZT_objective_lens's focus
 * (optical_elements.py:600-638 with XL_OP_HIGHNA in args->pre). */
int xl_czt(void* stream, const XlCztArgs* args);

/* One pass of xl_czt: 0 = prologue + x transform, 1 = y transform + epilogue. */
int xl_czt_stage(void* stream, const XlCztArgs* args, int stage);

/* Chirp vectors of a batch of distances, built on the device in float64 and
 * stored as complex64, packed entry after entry as XlCztArgs.z_batch reads
 * them.  Replaces the per-call host chirps of build_CZT_grid and
 * Bluestein_method (wave_optics.py:299-331, 385-460) for CZT_jit
 * (wave_optics.py:333-357) at many z: entry b has Dm = wavelength z[b] / dx,
 * f1 = out0 + Dm/2, f2 = out1 + Dm/2 per axis and the factor
 * cte[b] = z[b] dx dy wavelength.  The geometry is the forward's (input
 * ny x nx, output my x mx, Bluestein lengths 2^log2_l >= m + M, at least 32);
 * with adjoint = 1 the vectors are the adjoint set (pre' = conj(post) L,
 * g' = conj(g), post' = conj(pre) / L, of lengths mx, 2^log2_lx, nx on x). */
typedef struct {
  int batch;
  int ny, nx, my, mx;
  int log2_lx, log2_ly;
  int adjoint;
  const double* z;           /* device float64, batch entries */
  double wavelength, dx, dy;
  double xout0, xout1;       /* first and last output coordinates */
  double yout0, yout1;
  void* pre_x;               /* complex64 outputs, batch x (nx | 2^log2_lx | mx), adjoint (mx | . | nx) */
  void* g_x;
  void* post_x;
  void* pre_y;
  void* g_y;
  void* post_y;
  void* cte;                 /* complex64, batch entries */
} XlCztChirpArgs;

int xl_czt_chirps(void* stream, const XlCztChirpArgs* args);

/* The RS impulse response H(z, X, Y) of wave_optics.py:291-297 on the grid
 * (x, y) (device float64, nx and ny values), complex64, row-major ny x nx:
 * the F and F0 planes of CZT_jit (wave_optics.py:339-341), computed as the
 * chirp-z kernels compute them per pixel, for reuse by XlCztArgs.f_in /
 * f_out when a geometry is propagated repeatedly. */
int xl_czt_transfer_plane(void* stream, int ny, int nx, const double* x, const double* y, double z,
                          double wavelength, void* out);

/* ---- Elementwise ------------------------------------------------------ */

/* Apply a Jones program to batch x comps planes (out may alias in). */
int xl_apply_ops(void* stream, int batch, int comps, int ny, int nx, const void* const* in,
                 long long in_bstride, void* const* out, long long out_bstride, const XlProg* prog);

/* The per-pixel coefficients of the high-NA lens (optical_elements.py:528-594)
 * as 6 float32 planes of ny x nx: E' = K [Ex, Ey] with K = {K00, K01, K10,
 * K11, K20, K21}; they depend on the geometry only and are cached by callers. */
int xl_highna_coefficients(void* stream, int ny, int nx, const double* x, const double* y, double radius,
                           double f, void* out);

/* Backward of a Jones program: the gradients jax.grad takes through the masks
 * of optical_elements.py:76-332, :515-594 and :678-703.  `in` holds the
 * program's input planes and `gout` the gradient of its output (torch
 * convention for complex tensors, 2 dL/d conj(y)); `gin` receives the
 * gradient of the input (in[1], in[2] may be NULL for planes that are zero,
 * e.g. the Ez a propagator derives itself; gout[1], gout[2] may be NULL for
 * output planes whose gradient is zero).  pgrad[op*4 + i] (XL_MAX_OPS*4 entries, NULL skips)
 * receives dL/dp for parameter i of op: a float32 plane for a per-pixel
 * parameter (summed over the batch when the parameter is shared by it), or
 * one float64 accumulator that the call adds into for a scalar parameter. */
int xl_ops_backward(void* stream, int batch, int comps, int ny, int nx, const void* const* in,
                    long long in_bstride, const void* const* gout, long long gout_bstride,
                    void* const* gin, long long gin_bstride, const XlProg* prog, void* const* pgrad);

/* ---- Beam splitters ----------------------------------------------------- */

/* Two-port mixing of (Ex, Ey) planes by a complex 2x2 matrix M (row-major):
 * c = M00 a + M01 b, d = M10 a + M11 b.  This is BS_symmetric
 * (optical_elements.py:334-391: M = [[R, iT], [iT, R]] with the 1% loss of
 * :380-383), BS_symmetric_SI (:393-460: one input port, b absent) and the
 * lossless BS (:462-512: M = [[sqrt T, sqrt R e^{i phase}], [-sqrt R
 * e^{-i phase}, sqrt T]]).  The outputs' Ez is zero (not written). */
enum {
  XL_BS_MATRIX = 0,        /* M given in `m` */
  XL_BS_SYMMETRIC = 1,     /* BS_symmetric: M = [[R, iT], [iT, R]] from the angle `theta` */
  XL_BS_SINGLE_PORT0 = 2,  /* BS_symmetric_SI, port 0: c = R a, d = iT a */
  XL_BS_SINGLE_PORT1 = 3   /* BS_symmetric_SI, port 1: c = iT a, d = R a */
};

typedef struct {
  int batch, ny, nx;
  const void* in[2][2];       /* [port a, b][Ex, Ey] complex64 planes; port b may be NULL (zero) */
  long long in_bstride[2];    /* elements between batch entries, per port (0: one plane for the batch) */
  void* out[2][2];            /* [port c, d][Ex, Ey]; NULL planes are not written */
  long long out_bstride;
  const void* m;              /* XL_BS_MATRIX: device complex64 M, 4 entries per batch entry */
  long long m_bstride;        /* 0 (one M for the batch) or 4 */
  const double* theta;        /* the other kinds: device splitter angle(s), R = |sin| - 0.01 |cos|,
                                 T = 0.99 |cos| (optical_elements.py:376-383) */
  long long theta_bstride;    /* 0 (one angle for the batch) or 1 */
  int kind;                   /* XL_BS_* */
} XlBsArgs;

int xl_beam_splitter(void* stream, const XlBsArgs* args);

/* Bytes of workspace xl_beam_splitter_backward needs to return s. */
size_t xl_beam_splitter_work_bytes(int batch, int ny, int nx);

/* Backward of xl_beam_splitter (args as in the forward; args->out unused).
 * gout[4] = gradients of (c.Ex, c.Ey, d.Ex, d.Ey) (torch convention; NULL is
 * zero); gin[4] receives the gradients of (a.Ex, a.Ey, b.Ex, b.Ey) = M^H gout
 * (NULL skips); s (complex64, 4 per batch entry, may be NULL) receives
 * S_ij = sum conj(gout_i) in_j over pixels and both components, whose
 * conjugate is the gradient of M_ij (fixed-order sums); for the angle kinds,
 * dtheta (device float64 per batch entry, may be NULL; needs s) receives
 * dL/dtheta = sum_ij Re(dM_ij/dtheta S_ij). */
int xl_beam_splitter_backward(void* stream, const XlBsArgs* args, const void* const* gout,
                              long long gout_bstride, void* const* gin, long long gin_bstride, void* s,
                              void* work, void* dtheta);

/* ---- Reductions for gradients -------------------------------------------- */

/* out[p] = sum_i Re(conj(a_i) b_i) over planes p of npix complex64 pixels, in
 * a fixed order (work: xl_mse_intensity_work_bytes(planes, npix)). */
int xl_re_inner(void* stream, int planes, long long npix, const void* a, long long a_pstride, const void* b,
                long long b_pstride, void* work, void* out);

/* Per-plane MSE of kind 0 intensity (= xl_mse_intensity), 1 amplitude
 * sum (|a| - |b|)^2 / npix (MSE_Amplitude, loss_functions.py:109-121) or
 * 2 phase sum (arg a - arg b)^2 / npix (MSE_Phase, :123-135; vMSE_* at
 * :61-107 are the per-component forms); work and out as xl_mse_intensity.
 * The gradient takes gloss per plane and writes ga and / or gb (torch's
 * convention for complex tensors; zero where |a| or |b| is zero). */
int xl_plane_mse(void* stream, int kind, int planes, long long npix, const void* a, long long a_pstride,
                 const void* b, long long b_pstride, void* work, void* out);
int xl_plane_mse_grad(void* stream, int kind, int planes, long long npix, const void* a, long long a_pstride,
                      const void* b, long long b_pstride, const void* gloss, void* ga, void* gb);

/* ---- Fused loss epilogues (planes of npix pixels; complex_in = 1: the
 * planes are complex64 fields and the intensity |u|^2 is formed in the
 * kernel; 0: float32 intensities; in_pstride in elements).  Two reduction
 * passes with float64 block partials summed in a fixed order, so repeated
 * calls give identical results.  work: xl_loss_work_bytes(planes, npix),
 * which the forward fills with the statistics its gradient reads (keep it
 * between the two calls).  loss: planes float32 values (device).  Gradients
 * take the upstream gradient per plane (gloss, device float32) and write gin
 * (contiguous planes): for a complex input torch's convention 2 dL/d conj(u)
 * = 2 dL/dI u. */
size_t xl_loss_work_bytes(int planes, long long npix);

/* small_area_hybrid (loss_functions.py:24-40) per plane: In = I / (sum I +
 * 1e-8), mask = In > 0.7 max In, loss = sum mask / (sum mask In + 1e-8)
 * (vectorized_loss_hybrid, :42-50, is the planes > 1 form). */
int xl_area_loss(void* stream, int planes, long long npix, int complex_in, const void* in, long long in_pstride,
                 void* work, float* loss);
int xl_area_loss_grad(void* stream, int planes, long long npix, int complex_in, const void* in,
                      long long in_pstride, const void* work, const float* gloss, void* gin);

/* The 4f table's normalised intensity MSE (experiments/four_f_optical_table.py:
 * 129-141) per plane: In = I / sum I, loss = sum (In - T)^2 / npix, against
 * float32 target planes (target_pstride elements apart; 0: one target). */
int xl_norm_intensity_mse(void* stream, int planes, long long npix, int complex_in, const void* in,
                          long long in_pstride, const float* target, long long target_pstride, void* work,
                          float* loss);
int xl_norm_intensity_mse_grad(void* stream, int planes, long long npix, int complex_in, const void* in,
                               long long in_pstride, const float* target, long long target_pstride,
                               const void* work, const float* gloss, void* gin);

/* The distance gradient through the VRS Ez derivation (vectorized_optics.py:258-261):
 * out[b] = sum_i Re(conj(gez_i) dEz_i/dz), dEz/dz = -(Ex X + Ey Y) z / r^3, for
 * the Jones-program output (ex, ey) and the propagated Ez gradient gez of each
 * batch entry; x, y, z (one per entry) are device float64.  work as above. */
int xl_vrs_dz_ez(void* stream, int batch, int ny, int nx, const void* ex, const void* ey, long long e_bstride,
                 const void* gez, long long g_bstride, const double* x, const double* y, const double* z,
                 void* work, void* out);

/* The distance gradient of one RS / VRS call per batch entry, in one pass:
 * out[b] = sum_c sum_i Re(conj(g_c) d_c) + [VRS] sum_i Re(conj(gez_i) dEz_i/dz)
 * for the output gradients g (comps planes), the propagation d of the same
 * input through the dH/dz spectrum (xl_rs_transfer_spectrum_dz), and for VRS
 * (ex non-NULL) the Jones-program output (ex, ey), the adjoint's unfolded Ez
 * gradient gez and the grid / distances as in xl_vrs_dz_ez.  g, d and gez
 * share bstride; work: xl_mse_intensity_work_bytes(batch, ny * nx). */
int xl_rs_z_gradient(void* stream, int batch, int ny, int nx, int comps, const void* const* g, const void* const* d,
                     long long bstride, const void* ex, const void* ey, long long e_bstride, const void* gez,
                     const double* x, const double* y, const double* z, void* work, void* out);

/* ---- Table noise --------------------------------------------------------- */

/* The noise of shake_setup (optical_elements.py:2127-2217) for many optical
 * tables in one launch, from a counter-based generator (Philox4x32-10) keyed
 * per table: distance misalignment uniform in [min_d, max_d); phase and
 * amplitude noise planes +-uniform(min_phase, max_phase) that share their
 * magnitudes (as the reference's draws do) and differ in their signs, a
 * negative sign being 255 when `discretize` (the reference's uint8 cast);
 * waveplate noise +-uniform(min_phase, max_phase). */
#define XL_NOISE_MAX_TABLES 256
typedef struct {
  int tables;                   /* optical tables, one key each (<= XL_NOISE_MAX_TABLES) */
  int resolution;               /* side of the noise planes */
  int planes;                   /* planes per table (2 x the number of sSLMs) */
  int n_distances, n_wps;       /* distances and waveplate angles per table */
  double min_d, max_d;          /* misalignment range (um) */
  double min_phase, max_phase;  /* phase / amplitude noise range */
  int discretize;
  double* distances;            /* device, tables x n_distances */
  float* slms;                  /* device, tables x planes x resolution^2 (NULL: not drawn) */
  float* amps;                  /* device, same shape (NULL: not drawn) */
  double* wps;                  /* device, tables x n_wps */
} XlNoiseArgs;

/* keys: host array of 2 words per table. */
int xl_table_noise(void* stream, const XlNoiseArgs* args, const uint32_t* keys);

/* The generator on the host: out = Philox4x32-10(counter[4], key[2]). */
int xl_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out);

/* ---- Optimiser ----------------------------------------------------------- */

/* One AdamW step (torch.optim.AdamW's update, decoupled weight decay) over up
 * to XL_ADAMW_MAX_TENSORS float32 tensors in one launch; `step` is the device
 * step count after its increment (so the call can be recorded in a CUDA
 * graph).  The optimisation tables' update (optax.adamw in the reference's
 * experiments, e.g. experiments/hybrid_optimizer.py:33). */
#define XL_ADAMW_MAX_TENSORS 32
typedef struct {
  float* p;
  const float* g;
  float* m;
  float* v;
  long long n;
} XlAdamWTensor;
typedef struct {
  int count;
  XlAdamWTensor t[XL_ADAMW_MAX_TENSORS];
  float lr, beta1, beta2, eps, weight_decay;
  const float* step;
} XlAdamWArgs;

int xl_adamw_step(void* stream, const XlAdamWArgs* args);

/* ---- Losses ------------------------------------------------------------ */

/* Intensity MSE, MSE_Intensity of loss_functions.py:137-149, per plane:
 * out[p] = sum_i (|a_i|^2 - |b_i|^2)^2 / npix for planes p of npix complex64
 * pixels (plane strides in elements; b_pstride 0 broadcasts one target).
 * The sum runs in a fixed order (float64 partials in `work`, of
 * xl_mse_intensity_work_bytes), so repeated calls give identical results. */
size_t xl_mse_intensity_work_bytes(int planes, long long npix);
int xl_mse_intensity(void* stream, int planes, long long npix, const void* a, long long a_pstride,
                     const void* b, long long b_pstride, void* work, void* out);

/* Its gradients for upstream gradients gloss[p] (torch's convention for
 * complex tensors): ga = 4 gloss (|a|^2 - |b|^2) a / npix, gb = -4 gloss
 * (|a|^2 - |b|^2) b / npix, written as contiguous planes (either may be NULL). */
int xl_mse_intensity_grad(void* stream, int planes, long long npix, const void* a, long long a_pstride,
                          const void* b, long long b_pstride, const void* gloss, void* ga, void* gb);

#ifdef __cplusplus
}
#endif

#endif /* XLGB_H_ */
