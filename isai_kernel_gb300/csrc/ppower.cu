// Symbolic block-pattern product C = pattern(X * A) (no counterpart in the
// reference): the building block of ISAI(k), whose M_L / M_U patterns are
// the lower / upper triangle of pattern(A^k) instead of pattern(A).
//
// One warp per row i: the column lists of the rows of A named by row i of X
// are gathered into shared memory, sorted by a bitonic network and reduced
// to their distinct values.  Rows whose gathered length exceeds kCap report
// BILU_ERR_UNSUPPORTED (the row index in the error word) instead of being
// truncated.  Two passes: counts (then a scan gives the row pointer), fill.
#include <climits>

#include "common.cuh"
#include "scan.cuh"

namespace bilu {

namespace {

constexpr int kCap = 1024;    // gathered entries per row (power of two)
constexpr int kPPWarps = 4;   // warps (rows) per CTA: 16 KB of shared memory

template <bool FILL>
__global__ void __launch_bounds__(32 * kPPWarps) k_symprod(int n, const int* __restrict__ Xrow,
                                                           const int* __restrict__ Xcol,
                                                           const int* __restrict__ Arow,
                                                           const int* __restrict__ Acol,
                                                           int* __restrict__ Crow_or_cnt,
                                                           int* __restrict__ Ccol, int* err) {
  __shared__ int buf[kPPWarps][kCap];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long i = (long long)blockIdx.x * kPPWarps + w;
  if (i >= n) return;
  int* b = buf[w];
  int m = 0;
  for (int p = __ldg(Xrow + i), pe = __ldg(Xrow + i + 1); p < pe; ++p) {
    const int c = __ldg(Xcol + p);
    const int as = __ldg(Arow + c), len = __ldg(Arow + c + 1) - as;
    if (m + len > kCap) {
      if (lane == 0) atomicMin(err, (int)i);
      return;
    }
    for (int q = lane; q < len; q += 32) b[m + q] = __ldg(Acol + as + q);
    m += len;
  }
  int m2 = 1;
  while (m2 < m) m2 <<= 1;
  for (int t = m + lane; t < m2; t += 32) b[t] = INT_MAX;
  __syncwarp();
  // bitonic sort of b[0..m2)
  for (int k = 2; k <= m2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < m2; t += 32) {
        const int u = t ^ j;
        if (u > t) {
          const int x = b[t], y = b[u];
          const bool up = (t & k) == 0;
          if ((x > y) == up) {
            b[t] = y;
            b[u] = x;
          }
        }
      }
      __syncwarp();
    }
  }
  // distinct values, in order
  int base = FILL ? Crow_or_cnt[i] : 0, total = 0;
  for (int t0 = 0; t0 < m; t0 += 32) {
    const int t = t0 + lane;
    const bool first = t < m && (t == 0 || b[t] != b[t - 1]);
    const unsigned bal = __ballot_sync(0xffffffffu, first);
    if (FILL && first) Ccol[base + total + __popc(bal & ((1u << lane) - 1u))] = b[t];
    total += __popc(bal);
  }
  if (!FILL && lane == 0) Crow_or_cnt[i] = total;
}

}  // namespace

size_t pattern_product_ws(int n) {
  return carve_size(sizeof(int) * 2) + scan_ws_bytes((long long)n + 1);
}

int pattern_product_rowptr(int n, const int* Xrow, const int* Xcol, const int* Arow,
                           const int* Acol, int* Crow, int* h_nnz, int* h_bad, Carver& ws,
                           cudaStream_t st) {
  int* err = ws.take<int>(2);
  if (!err) return BILU_ERR_WORKSPACE;
  int init = INT_MAX, he = INT_MAX;
  BILU_TRY_CUDA(cudaMemcpyAsync(err, &init, sizeof(int), cudaMemcpyHostToDevice, st));
  if (n > 0) {
    k_symprod<false><<<ceil_div(n, kPPWarps), 32 * kPPWarps, 0, st>>>(n, Xrow, Xcol, Arow, Acol,
                                                                      Crow, nullptr, err);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(&he, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_bad) *h_bad = he == INT_MAX ? -1 : he;
  if (he != INT_MAX) return BILU_ERR_UNSUPPORTED;
  return scan_exclusive(Crow, Crow, n, h_nnz, ws, st);
}

int pattern_product_fill(int n, const int* Xrow, const int* Xcol, const int* Arow,
                         const int* Acol, const int* Crow, int* Ccol, Carver& ws,
                         cudaStream_t st) {
  int* err = ws.take<int>(2);
  if (!err) return BILU_ERR_WORKSPACE;
  int init = INT_MAX, he = INT_MAX;
  BILU_TRY_CUDA(cudaMemcpyAsync(err, &init, sizeof(int), cudaMemcpyHostToDevice, st));
  if (n > 0) {
    k_symprod<true><<<ceil_div(n, kPPWarps), 32 * kPPWarps, 0, st>>>(
        n, Xrow, Xcol, Arow, Acol, const_cast<int*>(Crow), Ccol, err);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(&he, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  return he == INT_MAX ? BILU_OK : BILU_ERR_UNSUPPORTED;
}

}  // namespace bilu

using namespace bilu;

extern "C" size_t bilu_pattern_product_ws_bytes(int nb) { return pattern_product_ws(nb); }

extern "C" int bilu_pattern_product_rowptr(int nb, const int* d_Xrow, const int* d_Xcol,
                                           const int* d_Arow, const int* d_Acol, int* d_Crow,
                                           int* h_nnz, int* h_bad_row, void* d_ws,
                                           size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || !d_Crow || !h_nnz || (nb > 0 && (!d_Xrow || !d_Xcol || !d_Arow || !d_Acol)))
    return BILU_ERR_ARG;
  Carver ws(d_ws, ws_bytes);
  return pattern_product_rowptr(nb, d_Xrow, d_Xcol, d_Arow, d_Acol, d_Crow, h_nnz, h_bad_row, ws,
                                S(stream));
}

extern "C" int bilu_pattern_product_fill(int nb, const int* d_Xrow, const int* d_Xcol,
                                         const int* d_Arow, const int* d_Acol,
                                         const int* d_Crow, int* d_Ccol, void* d_ws,
                                         size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || !d_Crow || (nb > 0 && (!d_Xrow || !d_Xcol || !d_Arow || !d_Acol || !d_Ccol)))
    return BILU_ERR_ARG;
  Carver ws(d_ws, ws_bytes);
  return pattern_product_fill(nb, d_Xrow, d_Xcol, d_Arow, d_Acol, d_Crow, d_Ccol, ws, S(stream));
}
