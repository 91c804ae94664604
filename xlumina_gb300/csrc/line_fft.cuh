// Pieces shared by the line-transform kernels of the propagators (RS / VRS and
// chirp-z): the FFT engine's pass twiddle tables in device memory,
// column-tiled addressing, TMA staging of input rows, persistent-grid sizing,
// and the registration of each translation unit's device tables.
//
// Every translation unit that includes this header gets its own copy of the
// static device objects below (whole-program compilation: one device module
// per unit) and registers, from a static initialiser, the function that
// fills them and the reader of its timeout counter.
#pragma once

#include <stdint.h>

#include <vector>

#include "common.cuh"
#include "fft_pair.cuh"
#include "internal.h"

namespace xl {

// ---- pass twiddle tables (FftTw layout, 16 elements per thread) for every
// transform length 2^5 .. 2^13, one after the other, filled at set-up from
// float64 values ----
__host__ __device__ constexpr int ptw_size(int logp) {
  // sum over passes 1.. of (radix - 1) * stride, radix 16 then the remainder
  int nfull = logp / 4, rem = logp % 4, npass = nfull + (rem ? 1 : 0), o = 0, ns = 1;
  for (int q = 0; q < npass; ++q) {
    const int r = q < nfull ? 16 : (1 << rem);
    if (q >= 1) o += (r - 1) * ns;
    ns *= r;
  }
  return o > 0 ? o : 1;
}
__host__ __device__ constexpr int ptw_off(int logp) {
  int o = 0;
  for (int l = 5; l < logp; ++l) o += ptw_size(l);
  return o;
}
constexpr int PTW_TOTAL = ptw_off(14);

static __device__ float2 g_ptw[PTW_TOTAL];
// the same tables in the two-line engine's form, (wr, wr, wi, wi) per entry
static __device__ float4 g_ptw4[PTW_TOTAL];

template <int LOGP> __device__ __forceinline__ const float2* pass_tw() {
  static_assert(ptw_size(LOGP) == FftTw<LOGP, 16>::SIZE, "pass table size");
  return g_ptw + ptw_off(LOGP);
}
template <int LOGP> __device__ __forceinline__ const float4* pass_tw4() { return g_ptw4 + ptw_off(LOGP); }

// Address of (row r, column col) in a column-tiled plane with `rows` rows:
// element (r, col) at ((col / W) rows + r) W + col % W.
template <int W>
__device__ __forceinline__ long long tiled(int r, int col, int rows) {
  return ((long long)(col / W) * rows + r) * W + (col % W);
}

// ---- rows staged into shared memory by TMA bulk copies: up to
// XL_ROW_STREAMS planes (input components and per-pixel parameter planes of
// the fused program), each copied G rows at a time ----
#define XL_ROW_STREAMS 8
#define XL_ROW_PREFETCH 4
struct RowStream {
  const char* src;      // row 0 of batch entry 0
  long long bstride;    // bytes between batch entries (0: shared by the batch)
  int row_bytes;        // bytes of one row (the plane's row stride), a multiple of 16
  int soff;             // byte offset of the stream's G rows in the stage
};
struct RowStage {
  int n;                       // staged streams
  int row_bytes;               // sum of the streams' row bytes
  RowStream s[XL_ROW_STREAMS];
  int fld[3];                  // stage offset of input component c, -1: read from global memory
  int prm[XL_MAX_OPS][4];      // stage offset of parameter plane i of op k, -1: global memory
  // planes the prologue reads from global memory (not staged, or the lens
  // coefficient planes); the chirp-z x transform prefetches them into L2 one
  // row group ahead (in the RS forward row pass, whose planes are all staged
  // in the benchmarked cases, the prefetch code cost 1.5 % and is left out)
  int npf;
  RowStream pf[XL_ROW_PREFETCH];   // soff unused
};

// Per-pixel parameters of the fused program, from the stage when the plane is
// staged, else from global memory.
struct StagedParams {
  const unsigned char* stage;
  const RowStage* st;
  int gi, nx, n;
  __device__ __forceinline__ float operator()(const XlOp& op, int k, int i, const PixelCtx& px) const {
    if (!(op.pmask & (1 << i))) return op.sval[i];
    const int off = st->prm[k][i];
    if (off >= 0) return ((const float*)(stage + off))[gi * nx + n];
    return __ldg((const float*)op.ptr[i] + (long long)px.batch * op.pbstride + px.pix);
  }
};

// Issue the bulk copies of row group (batch b, rows r0 .. r0 + rows - 1) on an
// armed barrier (one thread).
__device__ __forceinline__ void stage_rows(const RowStage& st, unsigned char* stage, unsigned long long* mbar,
                                           int b, int r0, int rows) {
  mbar_arrive_expect_tx(mbar, (unsigned)(rows * st.row_bytes));
  for (int s = 0; s < st.n; ++s) {
    const RowStream& q = st.s[s];
    bulk_copy_g2s(stage + q.soff, q.src + (long long)b * q.bstride + (long long)r0 * q.row_bytes,
                  (unsigned)(rows * q.row_bytes), mbar);
  }
}

// Prefetch into L2 the rows of group (batch b, rows r0 .. r0 + rows - 1) of
// the planes the prologue reads from global memory (one thread).
__device__ __forceinline__ void prefetch_rows(const RowStage& st, int b, int r0, int rows) {
  for (int s = 0; s < st.npf; ++s) {
    const RowStream& q = st.pf[s];
    l2_prefetch(q.src + (long long)b * q.bstride + (long long)r0 * q.row_bytes, (unsigned)(rows * q.row_bytes));
  }
}

// Which planes to stage: every input component and every per-pixel parameter
// plane of the fused program whose rows are 16-byte aligned, while the stage
// fits next to `fixed_smem` bytes of other shared memory within `cap` (the
// CTA's shared memory, barrier included; a smaller cap leaves room for more
// CTAs per SM, the planes that do not fit are read from global memory).
static inline void plan_row_stage(int cin, const float2* const* in, long long ibs, int nx, const XlProg& prog,
                                  int G, size_t fixed_smem, RowStage& st, size_t cap = 226 * 1024) {
  st.n = 0;
  st.row_bytes = 0;
  for (int c = 0; c < 3; ++c) st.fld[c] = -1;
  for (int k = 0; k < XL_MAX_OPS; ++k)
    for (int i = 0; i < 4; ++i) st.prm[k][i] = -1;
  int off = 0;
  auto add = [&](const void* src, long long bstride_bytes, int row_bytes) -> int {
    if (st.n >= XL_ROW_STREAMS || !src) return -1;
    if (((uintptr_t)src % 16) || (bstride_bytes % 16) || (row_bytes % 16)) return -1;
    if (fixed_smem + (size_t)off + (size_t)G * row_bytes + 16 > cap) return -1;
    RowStream& q = st.s[st.n++];
    q.src = (const char*)src;
    q.bstride = bstride_bytes;
    q.row_bytes = row_bytes;
    q.soff = off;
    const int o = off;
    off += G * row_bytes;
    st.row_bytes += row_bytes;
    return o;
  };
  // planes left in global memory: prefetched into L2 where the bulk prefetch
  // allows it (16-byte aligned rows)
  st.npf = 0;
  auto prefetch = [&](const void* src, long long bstride_bytes, int row_bytes) {
    if (st.npf >= XL_ROW_PREFETCH || !src) return;
    if (((uintptr_t)src % 16) || (bstride_bytes % 16) || (row_bytes % 16)) return;
    RowStream& q = st.pf[st.npf++];
    q.src = (const char*)src;
    q.bstride = bstride_bytes;
    q.row_bytes = row_bytes;
    q.soff = 0;
  };
  for (int c = 0; c < cin && c < 3; ++c) {
    st.fld[c] = add(in[c], ibs * 8, nx * 8);
    if (st.fld[c] < 0) prefetch(in[c], ibs * 8, nx * 8);
  }
  for (int k = 0; k < prog.nops; ++k) {
    const XlOp& op = prog.ops[k];
    for (int i = 0; i < 4; ++i)
      if (op.pmask & (1 << i)) {
        st.prm[k][i] = add(op.ptr[i], op.pbstride * 4, nx * 4);
        if (st.prm[k][i] < 0) prefetch(op.ptr[i], op.pbstride * 4, nx * 4);
      }
    // the lens's precomputed coefficient planes (6 x ny x nx float32, shared
    // by the batch): the Ez row's two, or all six
    if ((op.kind == XL_OP_HIGHNA || op.kind == XL_OP_HIGHNA_EZ) && op.ptr[2]) {
      const char* cp = (const char*)op.ptr[2];
      for (int q = op.kind == XL_OP_HIGHNA_EZ ? 4 : 0; q < 6; ++q) prefetch(cp + q * op.pbstride * 4, 0, nx * 4);
    }
  }
}

// SM count of the current device (cached per device).
static inline int device_sms() {
  static int sms[256];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return 132;
  if (!sms[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 132;
    sms[dev] = v;
  }
  return sms[dev];
}

// Grid of a persistent kernel: every resident CTA slot, at most `work` CTAs.
template <typename K>
static int persistent_grid(K kernel, int threads, size_t smem, int work) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const long long g = (long long)per_sm * device_sms();
  return (int)(g < work ? g : work);
}

// ---- this translation unit's device tables ----
template <int LOGP>
static void fill_pass_tables(std::vector<float2>& out, const float2* host) {
  const float2* twN = host + (1 << LOGP);
  for (int i = 0; i < FftTw<LOGP, 16>::SIZE; ++i) out[ptw_off(LOGP) + i] = pass_twiddle_entry<LOGP, 16>(i, twN);
  if constexpr (LOGP < 13) fill_pass_tables<LOGP + 1>(out, host);
}

static cudaError_t line_tu_tables(const float2* host) {
  cudaError_t e = cudaMemcpyToSymbol(g_tw, host, sizeof(g_tw));
  if (e != cudaSuccess) return e;
  std::vector<float2> ptw(PTW_TOTAL, make_float2(1.f, 0.f));
  fill_pass_tables<5>(ptw, host);
  if ((e = cudaMemcpyToSymbol(g_ptw, ptw.data(), sizeof(g_ptw))) != cudaSuccess) return e;
  std::vector<float4> ptw4(PTW_TOTAL);
  for (int i = 0; i < PTW_TOTAL; ++i) ptw4[i] = pair_tw(ptw[i]);
  return cudaMemcpyToSymbol(g_ptw4, ptw4.data(), sizeof(g_ptw4));
}

static cudaError_t line_tu_timeouts(unsigned int* count, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(count, g_line_timeouts, sizeof(unsigned int));
  if (e != cudaSuccess || !reset) return e;
  const unsigned int zero = 0;
  return cudaMemcpyToSymbol(g_line_timeouts, &zero, sizeof(unsigned int));
}

static cudaError_t line_tu_status(unsigned int* word, unsigned long long limit_ns) {
  cudaError_t e = cudaMemcpyToSymbol(g_status_word, &word, sizeof(word));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(g_wait_limit_ns, &limit_ns, sizeof(limit_ns));
}

static const bool line_tu_registered = register_device_tables(&line_tu_tables, &line_tu_timeouts, &line_tu_status);

}  // namespace xl
