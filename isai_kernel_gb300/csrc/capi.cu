// Remaining C ABI: status strings, the device residual check, the block
// transpose (BCSC view) used by the adjoint solves, the transposed SpMV and
// the masked outer-product gradient.
#include <algorithm>
#include <climits>

#include "blas1.cuh"
#include "common.cuh"

namespace bilu {

size_t transpose_ws(int mb, long long nnzb);
int transpose_pattern(int mb, int nbcol, const int* cptr, const int* cind, long long nnzb,
                      int* rptr, int* rind, int* src, Carver& ws, cudaStream_t st);
size_t syncfree_ws(int nb);
int diag_positions(int nb, const int* row, const int* col, int* diag, int* h_bad, Carver& ws,
                   cudaStream_t st);
size_t level_sched_ws(int nb, long long nnzb);
int sptrsv_level_impl(int nb, long long nnzb, int bs, const int* row, const int* col,
                      const int* diag, const double* val, int lower, int unit, const double* b,
                      double* x, Carver& ws, cudaStream_t st);
int spmv_any(int mb, int bs, int prec, const int* row, const int* col, const void* val,
             const void* x, int x32, void* y, int y32, cudaStream_t st, int layout);

namespace {

// out[t] = (in[src[d]])^T for block d (bs x bs transpose inside the block)
__global__ void k_gather_blocks_T(long long nnzb, int bs, const int* __restrict__ src,
                                  const double* __restrict__ in, double* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int bs2 = bs * bs;
  if (t >= nnzb * bs2) return;
  long long d = t / bs2;
  int e = (int)(t - d * bs2), r = e / bs, c = e - r * bs;
  out[t] = in[(long long)src[d] * bs2 + c * bs + r];
}

// G[p] (+)= scale * u_I v_J^T for block p = (I, J); thread per element
__global__ void k_masked_outer(int mb, int bs, long long nnzb, const int* __restrict__ row,
                               const int* __restrict__ col, const double* __restrict__ u,
                               const double* __restrict__ v, double scale, int accumulate,
                               double* __restrict__ G) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int bs2 = bs * bs;
  if (t >= nnzb * bs2) return;
  long long p = t / bs2;
  int e = (int)(t - p * bs2), r = e / bs, c = e - r * bs;
  int lo = 0, hi = mb - 1;
  while (lo < hi) {
    int m = (lo + hi + 1) >> 1;
    if (row[m] <= p) lo = m; else hi = m - 1;
  }
  double g = scale * u[(long long)lo * bs + r] * v[(long long)col[p] * bs + c];
  G[t] = accumulate ? G[t] + g : g;
}

__global__ void k_diff_sq(long long n, const double* __restrict__ a, const double* __restrict__ b,
                          double* __restrict__ partial) {
  double s0 = 0, s1 = 0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double d = a[e] - b[e];
    s0 = fma(d, d, s0);
    s1 = fma(b[e], b[e], s1);
  }
  __shared__ double r0[kRedThreads / 32], r1[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { r0[warp] = s0; r1[warp] = s1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0, a1 = 0;
    for (int w = 0; w < kRedThreads / 32; ++w) { a0 += r0[w]; a1 += r1[w]; }
    partial[(long long)blockIdx.x * kPartStride] = a0;
    partial[(long long)blockIdx.x * kPartStride + 1] = a1;
  }
}

__global__ void k_reduce2(const double* __restrict__ partial, double* out) {
  int i = threadIdx.x;
  if (i >= 2) return;
  double s = 0;
  for (int c = 0; c < kRedCTAs; ++c) s += partial[(long long)c * kPartStride + i];
  out[i] = s;
}

}  // namespace

size_t bsr_transpose_ws(int mb, long long nnzb) {
  return transpose_ws(mb, nnzb) + carve_size(sizeof(int) * (size_t)(nnzb + 1));
}

// T = M^T as BCSR with transposed blocks (the BCSC view of M).
int bsr_transpose_impl(int mb, int bs, const int* row, const int* col, const double* val,
                       long long nnzb, int* trow, int* tcol, double* tval, Carver& ws,
                       cudaStream_t st) {
  int* src = ws.take<int>((size_t)nnzb + 1);
  if (!src) return BILU_ERR_WORKSPACE;
  BILU_TRY(transpose_pattern(mb, mb, row, col, nnzb, trow, tcol, src, ws, st));
  if (nnzb > 0 && val && tval) {
    long long total = nnzb * bs * bs;
    k_gather_blocks_T<<<ceil_div(total, 256), 256, 0, st>>>(nnzb, bs, src, val, tval);
    BILU_LAUNCH_CHECK();
  }
  return BILU_OK;
}

}  // namespace bilu

using namespace bilu;

extern "C" const char* bilu_status_string(int s) {
  switch (s) {
    case BILU_OK: return "ok";
    case BILU_ERR_ARG: return "invalid argument";
    case BILU_ERR_PATTERN: return "invalid sparsity pattern";
    case BILU_ERR_ZERO_PIVOT: return "zero pivot";
    case BILU_ERR_TIMEOUT: return "sync-free wait timed out";
    case BILU_ERR_CUDA: return "CUDA error";
    case BILU_ERR_NOT_CONVERGED: return "not converged";
    case BILU_ERR_WORKSPACE: return "workspace too small";
    case BILU_ERR_UNSUPPORTED: return "unsupported block size, precision or file kind";
    case BILU_ERR_IO: return "file missing, unreadable, malformed or corrupt";
    default: return "unknown status";
  }
}

extern "C" int bilu_version(void) { return 10000; }

extern "C" int bilu_last_cuda_error(void) { return g_last_cuda_error; }

extern "C" unsigned long long bilu_kernel_launches(void) {
  return __atomic_load_n(&g_launches, __ATOMIC_RELAXED);
}

extern "C" size_t bilu_bsr_transpose_ws_bytes(int mb, int nnzb) { return bsr_transpose_ws(mb, nnzb); }

extern "C" int bilu_bsr_transpose(int mb, int bs, const int* d_row, const int* d_col,
                                  const double* d_val, int* d_trow, int* d_tcol, double* d_tval,
                                  void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (mb < 0 || bs < 1 || bs > 8 || !d_row || !d_trow) return BILU_ERR_ARG;
  int nnzb = 0;
  if (mb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_row + mb, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
    BILU_TRY_CUDA(cudaStreamSynchronize(S(stream)));
  }
  Carver ws(d_ws, ws_bytes);
  return bsr_transpose_impl(mb, bs, d_row, d_col, d_val, nnzb, d_trow, d_tcol, d_tval, ws,
                            S(stream));
}

// workspace: transposed copy of the factor + transpose scratch + sync state
static size_t sptrsv_t_ws(int nb, long long nnzb, int bs) {
  return carve_size(sizeof(int) * (size_t)(nb + 1)) + carve_size(sizeof(int) * (size_t)nnzb) +
         carve_size(sizeof(double) * (size_t)nnzb * bs * bs) +
         std::max(bsr_transpose_ws(nb, nnzb),
                  level_sched_ws(nb, nnzb) + carve_size(sizeof(int) * ((size_t)nb + 1)) +
                      carve_size(sizeof(int) * 2));
}

extern "C" size_t bilu_sptrsv_transpose_ws_bytes(int nb, int nnzb, int bs) {
  return sptrsv_t_ws(nb, nnzb, bs);
}

extern "C" int bilu_sptrsv_transpose(int nb, int bs, const int* d_row, const int* d_col,
                                     const double* d_val, int lower, const double* d_b,
                                     double* d_x, void* d_ws, size_t ws_bytes,
                                     bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)) ||
      (nb > 0 && (const void*)d_b == (const void*)d_x))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  int nnzb = 0;
  if (nb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_row + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  Carver ws(d_ws, ws_bytes);
  int* trow = ws.take<int>((size_t)nb + 1);
  int* tcol = ws.take<int>((size_t)nnzb);
  double* tval = ws.take<double>((size_t)nnzb * bs * bs);
  if (!trow || (nnzb && (!tcol || !tval))) return BILU_ERR_WORKSPACE;
  {
    Carver w2 = ws;
    BILU_TRY(bsr_transpose_impl(nb, bs, d_row, d_col, d_val, nnzb, trow, tcol, tval, w2, st));
  }
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, trow, tcol, diag, nullptr, ws, st));
  // L^T: upper, unit (strict upper of the transposed diagonal block);
  // U^T: lower, non-unit (lower part incl. diagonal)
  return sptrsv_level_impl(nb, nnzb, bs, trow, tcol, diag, tval, lower ? 0 : 1, lower ? 1 : 0, d_b,
                           d_x, ws, st);
}

extern "C" size_t bilu_spmv_transpose_ws_bytes(int mb, int nnzb) {
  return bsr_transpose_ws(mb, nnzb) + carve_size(sizeof(int) * (size_t)(mb + 1)) +
         carve_size(sizeof(int) * (size_t)nnzb) + carve_size(sizeof(double) * (size_t)nnzb * 64);
}

extern "C" int bilu_bcsr_spmv_transpose(int mb, int bs, const int* d_row, const int* d_col,
                                        const double* d_val, const double* d_x, double* d_y,
                                        void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (mb < 0 || (mb > 0 && (!d_row || !d_col || !d_val || !d_x || !d_y))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  int nnzb = 0;
  if (mb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_row + mb, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  Carver ws(d_ws, ws_bytes);
  int* trow = ws.take<int>((size_t)mb + 1);
  int* tcol = ws.take<int>((size_t)nnzb);
  double* tval = ws.take<double>((size_t)nnzb * bs * bs);
  if (!trow || (nnzb && (!tcol || !tval))) return BILU_ERR_WORKSPACE;
  BILU_TRY(bsr_transpose_impl(mb, bs, d_row, d_col, d_val, nnzb, trow, tcol, tval, ws, st));
  return spmv_any(mb, bs, BILU_FP64, trow, tcol, tval, d_x, 0, d_y, 0, st, -1);
}

extern "C" int bilu_masked_outer(int mb, int bs, const int* d_row, const int* d_col,
                                 const double* d_u, const double* d_v, double scale,
                                 int accumulate, double* d_G, bilu_stream_t stream) {
  if (mb < 0 || bs < 1 || bs > 8) return BILU_ERR_ARG;
  cudaStream_t st = S(stream);
  int nnzb = 0;
  if (mb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_row + mb, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  if (nnzb == 0) return BILU_OK;
  long long total = (long long)nnzb * bs * bs;
  k_masked_outer<<<ceil_div(total, 256), 256, 0, st>>>(mb, bs, nnzb, d_row, d_col, d_u, d_v,
                                                       scale, accumulate, d_G);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

extern "C" size_t bilu_rel_errors_ws_bytes(int nb, int bs) {
  return carve_size(sizeof(double) * (size_t)nb * bs) +
         carve_size(sizeof(double) * kRedCTAs * kPartStride) + carve_size(sizeof(double) * 8);
}

extern "C" int bilu_rel_errors(int nb, int bs, const int* d_row, const int* d_col,
                               const double* d_val, const double* d_b, const double* d_x_true,
                               const double* d_x, double* h_out, void* d_ws, size_t ws_bytes,
                               bilu_stream_t stream) {
  if (nb < 0 || !h_out || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  long long n = (long long)nb * bs;
  Carver ws(d_ws, ws_bytes);
  double* ax = ws.take<double>((size_t)n);
  double* part = ws.take<double>((size_t)kRedCTAs * kPartStride);
  double* out = ws.take<double>(8);
  if (!ax || !part || !out) return BILU_ERR_WORKSPACE;
  double h[4] = {0, 0, 0, 0};
  BILU_TRY(spmv_any(nb, bs, BILU_FP64, d_row, d_col, d_val, d_x, 0, ax, 0, st, -1));
  // ||b - Ax||^2 and ||b||^2
  k_diff_sq<<<kRedCTAs, kRedThreads, 0, st>>>(n, ax, d_b, part);
  BILU_LAUNCH_CHECK();
  k_reduce2<<<1, 32, 0, st>>>(part, out);
  BILU_LAUNCH_CHECK();
  if (d_x_true) {
    k_diff_sq<<<kRedCTAs, kRedThreads, 0, st>>>(n, d_x, d_x_true, part);
    BILU_LAUNCH_CHECK();
    k_reduce2<<<1, 32, 0, st>>>(part, out + 2);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  h_out[1] = h[1] > 0 ? sqrt(h[0]) / sqrt(h[1]) : INFINITY;
  h_out[0] = d_x_true ? (h[3] > 0 ? sqrt(h[2]) / sqrt(h[3]) : 0.0) : 0.0;
  return BILU_OK;
}
