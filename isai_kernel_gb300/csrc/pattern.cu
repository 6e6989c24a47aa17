// Format conversions and sparsity patterns on the GPU (integer work,
// bit-exact with the reference's host builders).
//
//   csr_to_bsr5                            csr2bsr.h:14
//   bsr2csr_cusparse                       bsr2csr.h:19
//   build_bcsc_pattern_from_bsr_scalarILU  isai_bsr.h:246
//   build_triangular_bcsr_pattern_from_A   bcsc2bcsr.h:11
//   build_map_bcsc2bcsr_host               bcsc2bcsr.h:32
//   reorder_bcsc_val_to_bcsr_bs5           bcsc2bcsr.h:63
//   bcsc_to_bcsr                           bcsc2bcsrAndSpMV.h:76
//
// Transposes use atomic cursors for the scatter and then a warp-per-segment
// rank sort (rank = number of smaller keys in the segment), so the output
// order is ascending and independent of the atomic order.
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace bilu {

namespace {

constexpr int kT = 256;

// err[0]: first offending block row (atomicMin), err[1]: kind (atomicMax)
// kind 1 = column out of range, 2 = columns not strictly ascending,
// 3 = missing diagonal block, 4 = row pointer decreasing
__device__ __forceinline__ void report(int* err, int row, int kind) {
  atomicMin(err, row);
  atomicMax(err + 1, kind);
}

__global__ void k_fill_int(int* p, long long n, int v) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// Per block row: validate and count qualifying off-diagonal entries into
// the column counters (ISAI pattern) -- cnt[] preset to 1 for the diagonal.
__global__ void k_isai_count(int nb, const int* __restrict__ row, const int* __restrict__ col,
                             int lower, int* cnt, int* err) {
  int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= nb) return;
  int s = row[br], e = row[br + 1];
  if (e < s) { report(err, br, 4); return; }
  int prev = -1;
  for (int p = s; p < e; ++p) {
    int bc = col[p];
    if (bc < 0 || bc >= nb) { report(err, br, 1); return; }
    if (bc <= prev) { report(err, br, 2); return; }
    prev = bc;
    if (bc == br) continue;
    if (lower ? (bc > br) : (bc < br)) continue;
    atomicAdd(cnt + bc, 1);
  }
}

__global__ void k_isai_scatter(int nb, const int* __restrict__ row, const int* __restrict__ col,
                               int lower, const int* __restrict__ Mptr, int* cursor, int* tmp) {
  int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= nb) return;
  for (int p = row[br]; p < row[br + 1]; ++p) {
    int bc = col[p];
    if (bc == br || bc < 0 || bc >= nb) continue;
    if (lower ? (bc > br) : (bc < br)) continue;
    tmp[Mptr[bc] + atomicAdd(cursor + bc, 1)] = br;
  }
  tmp[Mptr[br] + atomicAdd(cursor + br, 1)] = br;
}

// Warp per segment: out[ptr[s] + rank(key)] = key (and payload), keys
// distinct inside a segment.
__global__ void k_segment_rank_sort(int nseg, const int* __restrict__ ptr,
                                    const int* __restrict__ key, const int* __restrict__ pay,
                                    int* __restrict__ key_out, int* __restrict__ pay_out) {
  int lane = threadIdx.x & 31;
  int sgi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (sgi >= nseg) return;
  int s = ptr[sgi], e = ptr[sgi + 1];
  for (int i = s + lane; i < e; i += 32) {
    int k = key[i], rank = 0;
    for (int j = s; j < e; ++j) rank += key[j] < k;
    key_out[s + rank] = k;
    if (pay_out) pay_out[s + rank] = pay[i];
  }
}

__global__ void k_tri_count(int nb, const int* __restrict__ row, const int* __restrict__ col,
                            int lower, int* cnt) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  int c = 0;
  for (int p = row[r]; p < row[r + 1]; ++p) c += lower ? (col[p] <= r) : (col[p] >= r);
  cnt[r] = c;
}

__global__ void k_tri_fill(int nb, const int* __restrict__ row, const int* __restrict__ col,
                           int lower, const int* __restrict__ Trow, int* __restrict__ Tcol) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  int o = Trow[r];
  for (int p = row[r]; p < row[r + 1]; ++p)
    if (lower ? (col[p] <= r) : (col[p] >= r)) Tcol[o++] = col[p];
}

// Thread per BCSC column: binary search of each entry in its BCSR row.
__global__ void k_map(int nb, const int* __restrict__ cptr, const int* __restrict__ cind,
                      const int* __restrict__ rrow, const int* __restrict__ rcol,
                      int* __restrict__ map, unsigned long long* bad) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nb) return;
  for (int k = cptr[c]; k < cptr[c + 1]; ++k) {
    int r = cind[k];
    int lo = rrow[r], hi = rrow[r + 1] - 1, found = -1;
    while (lo <= hi) {
      int m = (lo + hi) >> 1, v = rcol[m];
      if (v == c) { found = m; break; }
      if (v < c) lo = m + 1; else hi = m - 1;
    }
    if (found < 0) {
      // first mismatch in the reference's visiting order (column-major)
      atomicMin(bad, ((unsigned long long)(unsigned)c << 32) | (unsigned)r);
      map[k] = -1;
    } else {
      map[k] = found;
    }
  }
}

// dst[map[k]] = src[k], blocks of bs2 doubles copied as double2 pairs when
// the block size allows it; dst32 (optional) receives the same values
// rounded to FP32 in the same pass (the FP32-stored factors of the mixed
// apply), instead of a second read of dst.
__global__ void k_reorder(long long nnzb, int bs2, const int* __restrict__ map,
                          const double* __restrict__ src, double* __restrict__ dst,
                          float* __restrict__ dst32) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = nnzb * bs2;
  if (t >= total) return;
  long long k = t / bs2;
  int e = (int)(t - k * bs2);
  const long long d = (long long)map[k] * bs2 + e;
  const double v = src[t];
  dst[d] = v;
  if (dst32) dst32[d] = __double2float_rn(v);
}

__global__ void k_reorder_v2(long long nnzb, int half, const int* __restrict__ map,
                             const double2* __restrict__ src, double2* __restrict__ dst,
                             float2* __restrict__ dst32) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = nnzb * half;
  if (t >= total) return;
  long long k = t / half;
  int e = (int)(t - k * half);
  const long long d = (long long)map[k] * half + e;
  const double2 v = src[t];
  dst[d] = v;
  if (dst32) dst32[d] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
}

// bcsc -> bcsr: count blocks per row
__global__ void k_count_rows(long long nnzb, const int* __restrict__ ind, int mb, int* cnt,
                             int* err) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnzb) return;
  int r = ind[k];
  if (r < 0 || r >= mb) { report(err, r, 1); return; }
  atomicAdd(cnt + r, 1);
}

__global__ void k_csc_scatter(int nbcol, const int* __restrict__ cptr,
                              const int* __restrict__ cind, const int* __restrict__ rptr,
                              int* cursor, int* key, int* src) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nbcol) return;
  for (int k = cptr[c]; k < cptr[c + 1]; ++k) {
    int r = cind[k];
    int d = rptr[r] + atomicAdd(cursor + r, 1);
    key[d] = c;
    src[d] = k;
  }
}

__global__ void k_gather_blocks(long long nnzb, int bs2, const int* __restrict__ src,
                                const double* __restrict__ in, double* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnzb * bs2) return;
  long long d = t / bs2;
  int e = (int)(t - d * bs2);
  out[t] = in[(long long)src[d] * bs2 + e];
}

// csr -> bsr, warp per block row.  Count the distinct block columns of the
// bs scalar rows: an entry counts if no earlier entry of the segment has
// the same block column.
__global__ void k_c2b_count(int nb, int bs, const int* __restrict__ crow,
                            const int* __restrict__ ccol, int ncols, int* __restrict__ cnt,
                            int* err) {
  int lane = threadIdx.x & 31;
  int br = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (br >= nb) return;
  int s = crow[br * bs], e = crow[br * bs + bs];
  int c = 0;
  for (int i = s + lane; i < e; i += 32) {
    int gc = ccol[i];
    if (gc < 0 || gc >= ncols) { report(err, br, 1); continue; }
    int bc = gc / bs;
    bool first = true;
    for (int j = s; j < i && first; ++j) first = (ccol[j] / bs) != bc;
    c += first;
  }
  c = warp_sum(c);
  if (lane == 0) cnt[br] = c;
}

__global__ void k_c2b_fill(int nb, int bs, const int* __restrict__ crow,
                           const int* __restrict__ ccol, const double* __restrict__ cval,
                           const int* __restrict__ brow, int* __restrict__ bcol,
                           double* __restrict__ bval) {
  int lane = threadIdx.x & 31;
  int br = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (br >= nb) return;
  int s = crow[br * bs], e = crow[br * bs + bs];
  int base = brow[br], u = brow[br + 1] - base;
  // 1) distinct block columns in ascending order (column range checked by
  //    the count phase, which reports BILU_ERR_PATTERN)
  for (int i = s + lane; i < e; i += 32) {
    int bc = ccol[i] / bs;
    bool first = true;
    for (int j = s; j < i && first; ++j) first = (ccol[j] / bs) != bc;
    if (!first) continue;
    int rank = 0;
    for (int j = s; j < e; ++j) {
      int bj = ccol[j] / bs;
      if (bj < bc) {
        bool fj = true;
        for (int q = s; q < j && fj; ++q) fj = (ccol[q] / bs) != bj;
        rank += fj;
      }
    }
    if (rank < u) bcol[base + rank] = bc;
  }
  // 2) zero the blocks
  int bs2 = bs * bs;
  for (long long t = lane; t < (long long)u * bs2; t += 32) bval[(long long)base * bs2 + t] = 0.0;
  __syncwarp();
  // 3) lane per scalar row accumulates its entries in order (the reference's
  //    std::map accumulation order for a given position)
  if (lane < bs) {
    int rr = br * bs + lane;
    for (int p = crow[rr]; p < crow[rr + 1]; ++p) {
      int gc = ccol[p], bc = gc / bs, lc = gc - bc * bs;
      int lo = 0, hi = u - 1, k = -1;
      while (lo <= hi) {
        int m = (lo + hi) >> 1, v = bcol[base + m];
        if (v == bc) { k = m; break; }
        if (v < bc) lo = m + 1; else hi = m - 1;
      }
      if (k >= 0) bval[((long long)(base + k) * bs + lane) * bs + lc] += cval[p];
    }
  }
}

// bsr -> csr (row direction): thread per (block, row r) writes bs entries.
__global__ void k_b2c_rowptr(int mb, int bs, const int* __restrict__ brow, int* __restrict__ crow) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > (long long)mb * bs) return;
  if (t == (long long)mb * bs) { crow[t] = brow[mb] * bs * bs; return; }
  int br = (int)(t / bs), r = (int)(t - (long long)br * bs);
  int len = brow[br + 1] - brow[br];
  crow[t] = brow[br] * bs * bs + r * len * bs;
}

__global__ void k_b2c_fill(int mb, int bs, long long nnzb, const int* __restrict__ brow,
                           const int* __restrict__ bcol, const double* __restrict__ bval,
                           const int* __restrict__ crow, int* __restrict__ ccol,
                           double* __restrict__ cval) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnzb * bs) return;
  long long p = t / bs;
  int r = (int)(t - p * bs);
  // block row of block p: last br with brow[br] <= p
  int lo = 0, hi = mb - 1;
  while (lo < hi) {
    int m = (lo + hi + 1) >> 1;
    if (brow[m] <= p) lo = m; else hi = m - 1;
  }
  int br = lo;
  int k = (int)(p - brow[br]);
  long long o = (long long)crow[(long long)br * bs + r] + (long long)k * bs;
  int bc = bcol[p];
  for (int c = 0; c < bs; ++c) {
    ccol[o + c] = bc * bs + c;
    cval[o + c] = bval[(p * bs + r) * bs + c];
  }
}

int read_err(int* d_err, int* h_err, cudaStream_t st) {
  BILU_TRY_CUDA(cudaMemcpyAsync(h_err, d_err, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  return BILU_OK;
}

int init_err(int* d_err, cudaStream_t st) {
  int init[2] = {0x7fffffff, 0};
  BILU_TRY_CUDA(cudaMemcpyAsync(d_err, init, sizeof(init), cudaMemcpyHostToDevice, st));
  return BILU_OK;
}

}  // namespace

// --------------------------------------------------------------- ISAI pattern
size_t isai_pattern_ws(int nb, long long nnzb) {
  return carve_size(sizeof(int) * 2) + carve_size(sizeof(int) * (size_t)(nb + 1)) +
         carve_size(sizeof(int) * (size_t)(nnzb + nb)) + scan_ws_bytes(nb + 1);
}

int isai_pattern_colptr_impl(int nb, const int* row, const int* col, int lower, int* Mptr,
                             int* h_nnz, Carver& ws, cudaStream_t st) {
  int* err = ws.take<int>(2);
  if (!err) return BILU_ERR_WORKSPACE;
  BILU_TRY(init_err(err, st));
  if (nb > 0) {
    k_fill_int<<<ceil_div(nb, kT), kT, 0, st>>>(Mptr, nb, 1);
    BILU_LAUNCH_CHECK();
    k_isai_count<<<ceil_div(nb, kT), kT, 0, st>>>(nb, row, col, lower, Mptr, err);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY(scan_exclusive(Mptr, Mptr, nb, h_nnz, ws, st));
  int h_err[2];
  BILU_TRY(read_err(err, h_err, st));
  if (h_err[1] != 0) return BILU_ERR_PATTERN;
  return BILU_OK;
}

int isai_pattern_fill_impl(int nb, const int* row, const int* col, int lower, const int* Mptr,
                           int* Mind, int mnnz, Carver& ws, cudaStream_t st) {
  int* cursor = ws.take<int>((size_t)nb + 1);
  int* tmp = ws.take<int>((size_t)mnnz + 1);
  if (!cursor || !tmp) return BILU_ERR_WORKSPACE;
  if (nb == 0) return BILU_OK;
  BILU_TRY_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * nb, st));
  k_isai_scatter<<<ceil_div(nb, kT), kT, 0, st>>>(nb, row, col, lower, Mptr, cursor, tmp);
  BILU_LAUNCH_CHECK();
  k_segment_rank_sort<<<ceil_div(nb, 8), 256, 0, st>>>(nb, Mptr, tmp, nullptr, Mind, nullptr);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// --------------------------------------------------------------- tri pattern
int tri_pattern_rowptr_impl(int nb, const int* row, const int* col, int lower, int* Trow,
                            int* h_nnz, Carver& ws, cudaStream_t st) {
  if (nb > 0) {
    k_tri_count<<<ceil_div(nb, kT), kT, 0, st>>>(nb, row, col, lower, Trow);
    BILU_LAUNCH_CHECK();
  }
  return scan_exclusive(Trow, Trow, nb, h_nnz, ws, st);
}

int tri_pattern_fill_impl(int nb, const int* row, const int* col, int lower, const int* Trow,
                          int* Tcol, cudaStream_t st) {
  if (nb == 0) return BILU_OK;
  k_tri_fill<<<ceil_div(nb, kT), kT, 0, st>>>(nb, row, col, lower, Trow, Tcol);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// --------------------------------------------------------------- map / reorder
int map_impl(int nb, const int* cptr, const int* cind, const int* rrow, const int* rcol, int* map,
             int* h_bad, Carver& ws, cudaStream_t st) {
  unsigned long long* bad = ws.take<unsigned long long>(1);
  if (!bad) return BILU_ERR_WORKSPACE;
  unsigned long long init = ~0ull, hb = 0;
  BILU_TRY_CUDA(cudaMemcpyAsync(bad, &init, sizeof(init), cudaMemcpyHostToDevice, st));
  if (nb > 0) {
    k_map<<<ceil_div(nb, kT), kT, 0, st>>>(nb, cptr, cind, rrow, rcol, map, bad);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (hb != ~0ull) {
    if (h_bad) {
      h_bad[0] = (int)(hb & 0xffffffffu);
      h_bad[1] = (int)(hb >> 32);
    }
    return BILU_ERR_PATTERN;
  }
  return BILU_OK;
}

int reorder_impl(long long nnzb, int bs, const int* map, const double* src, double* dst,
                 cudaStream_t st, float* dst32 = nullptr) {
  if (nnzb == 0) return BILU_OK;
  int bs2 = bs * bs;
  if (bs2 % 2 == 0) {
    long long total = nnzb * (bs2 / 2);
    k_reorder_v2<<<ceil_div(total, kT), kT, 0, st>>>(nnzb, bs2 / 2, map, (const double2*)src,
                                                     (double2*)dst, (float2*)dst32);
  } else {
    long long total = nnzb * bs2;
    k_reorder<<<ceil_div(total, kT), kT, 0, st>>>(nnzb, bs2, map, src, dst, dst32);
  }
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// --------------------------------------------------------------- transpose
size_t transpose_ws(int mb, long long nnzb) {
  return carve_size(sizeof(int) * 2) + carve_size(sizeof(int) * (size_t)(mb + 1)) +
         3 * carve_size(sizeof(int) * (size_t)(nnzb + 1)) + scan_ws_bytes(mb + 1);
}

// BCSC (cptr over nbcol columns) -> BCSR pattern with ascending columns and
// src[d] = BCSC index of BCSR entry d.
int transpose_pattern(int mb, int nbcol, const int* cptr, const int* cind, long long nnzb,
                      int* rptr, int* rind, int* src, Carver& ws, cudaStream_t st) {
  int* err = ws.take<int>(2);
  int* cursor = ws.take<int>((size_t)mb + 1);
  int* key = ws.take<int>((size_t)nnzb + 1);
  int* pay = ws.take<int>((size_t)nnzb + 1);
  if (!err || !cursor || !key || !pay) return BILU_ERR_WORKSPACE;
  BILU_TRY(init_err(err, st));
  BILU_TRY_CUDA(cudaMemsetAsync(rptr, 0, sizeof(int) * (mb + 1), st));
  if (nnzb > 0) {
    k_count_rows<<<ceil_div(nnzb, kT), kT, 0, st>>>(nnzb, cind, mb, rptr, err);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY(scan_exclusive(rptr, rptr, mb, nullptr, ws, st));
  int h_err[2];
  BILU_TRY(read_err(err, h_err, st));
  if (h_err[1] != 0) return BILU_ERR_PATTERN;
  if (mb == 0 || nnzb == 0) return BILU_OK;
  BILU_TRY_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * mb, st));
  k_csc_scatter<<<ceil_div(nbcol, kT), kT, 0, st>>>(nbcol, cptr, cind, rptr, cursor, key, pay);
  BILU_LAUNCH_CHECK();
  k_segment_rank_sort<<<ceil_div(mb, 8), 256, 0, st>>>(mb, rptr, key, pay, rind, src);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int gather_blocks(long long nnzb, int bs, const int* src, const double* in, double* out,
                  cudaStream_t st) {
  if (nnzb == 0) return BILU_OK;
  long long total = nnzb * bs * bs;
  k_gather_blocks<<<ceil_div(total, kT), kT, 0, st>>>(nnzb, bs * bs, src, in, out);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

}  // namespace bilu

using namespace bilu;

// --------------------------------------------------------------- C ABI
extern "C" size_t bilu_isai_pattern_ws_bytes(int nb, int nnzb) {
  return isai_pattern_ws(nb, nnzb);
}

extern "C" int bilu_isai_pattern_colptr(int nb, const int* d_Arow, const int* d_Acol, int lower,
                                        int* d_Mptr, int* h_nnz, void* d_ws, size_t ws_bytes,
                                        bilu_stream_t stream) {
  if (nb < 0 || !d_Mptr || (nb > 0 && (!d_Arow || !d_Acol))) return BILU_ERR_ARG;
  Carver ws(d_ws, ws_bytes);
  return isai_pattern_colptr_impl(nb, d_Arow, d_Acol, lower != 0, d_Mptr, h_nnz, ws, S(stream));
}

extern "C" int bilu_isai_pattern_fill(int nb, const int* d_Arow, const int* d_Acol, int lower,
                                      const int* d_Mptr, int* d_Mind, void* d_ws,
                                      size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_Arow || !d_Acol || !d_Mptr || !d_Mind))) return BILU_ERR_ARG;
  int mnnz = 0;  // bounded by nnzb(A) + nb, the size the workspace query used
  if (nb > 0)
    BILU_TRY_CUDA(cudaMemcpyAsync(&mnnz, d_Mptr + nb, sizeof(int), cudaMemcpyDeviceToHost,
                                  S(stream)));
  BILU_TRY_CUDA(cudaStreamSynchronize(S(stream)));
  Carver ws(d_ws, ws_bytes);
  if (!ws.take<int>(2)) return BILU_ERR_WORKSPACE;  // same layout as the count phase
  return isai_pattern_fill_impl(nb, d_Arow, d_Acol, lower != 0, d_Mptr, d_Mind, mnnz, ws,
                                S(stream));
}

extern "C" size_t bilu_tri_pattern_ws_bytes(int nb) { return scan_ws_bytes(nb + 1); }

extern "C" int bilu_tri_pattern_rowptr(int nb, const int* d_Arow, const int* d_Acol, int lower,
                                       int* d_Trow, int* h_nnz, void* d_ws, size_t ws_bytes,
                                       bilu_stream_t stream) {
  if (nb < 0 || !d_Trow || (nb > 0 && (!d_Arow || !d_Acol))) return BILU_ERR_ARG;
  Carver ws(d_ws, ws_bytes);
  return tri_pattern_rowptr_impl(nb, d_Arow, d_Acol, lower != 0, d_Trow, h_nnz, ws, S(stream));
}

extern "C" int bilu_tri_pattern_fill(int nb, const int* d_Arow, const int* d_Acol, int lower,
                                     const int* d_Trow, int* d_Tcol, bilu_stream_t stream) {
  if (nb < 0) return BILU_ERR_ARG;
  return tri_pattern_fill_impl(nb, d_Arow, d_Acol, lower != 0, d_Trow, d_Tcol, S(stream));
}

extern "C" size_t bilu_map_ws_bytes(void) { return carve_size(sizeof(unsigned long long)); }

extern "C" int bilu_map_bcsc2bcsr(int nb, const int* d_cscPtr, const int* d_cscInd,
                                  const int* d_csrRow, const int* d_csrCol, int* d_map,
                                  int* h_bad, void* d_ws, size_t ws_bytes,
                                  bilu_stream_t stream) {
  if (nb < 0) return BILU_ERR_ARG;
  Carver ws(d_ws, ws_bytes);
  return map_impl(nb, d_cscPtr, d_cscInd, d_csrRow, d_csrCol, d_map, h_bad, ws, S(stream));
}

extern "C" int bilu_reorder_bcsc_to_bcsr(int nnzb, int bs, const int* d_map, const double* d_src,
                                         double* d_dst, bilu_stream_t stream) {
  if (nnzb < 0 || bs < 1 || bs > 8) return BILU_ERR_ARG;
  return reorder_impl(nnzb, bs, d_map, d_src, d_dst, S(stream));
}

extern "C" size_t bilu_bcsc_to_bcsr_ws_bytes(int mb, int nnzb) {
  return transpose_ws(mb, nnzb) + carve_size(sizeof(int) * (size_t)(nnzb + 1));
}

extern "C" int bilu_bcsc_to_bcsr(int mb, int nbcol, int bs, const int* d_cscPtr,
                                 const int* d_cscInd, const double* d_cscVal, int* d_rowPtr,
                                 int* d_colInd, double* d_val, void* d_ws, size_t ws_bytes,
                                 bilu_stream_t stream) {
  if (mb < 0 || nbcol < 0 || bs < 1 || bs > 8) return BILU_ERR_ARG;
  int nnzb = 0;
  if (nbcol > 0)
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_cscPtr + nbcol, sizeof(int), cudaMemcpyDeviceToHost,
                                  S(stream)));
  BILU_TRY_CUDA(cudaStreamSynchronize(S(stream)));
  Carver ws(d_ws, ws_bytes);
  int* src = ws.take<int>((size_t)nnzb + 1);
  if (!src) return BILU_ERR_WORKSPACE;
  BILU_TRY(transpose_pattern(mb, nbcol, d_cscPtr, d_cscInd, nnzb, d_rowPtr, d_colInd, src, ws,
                             S(stream)));
  if (d_cscVal && d_val) BILU_TRY(gather_blocks(nnzb, bs, src, d_cscVal, d_val, S(stream)));
  return BILU_OK;
}

extern "C" size_t bilu_csr_to_bsr_ws_bytes(int n, int bs) {
  int nb = bs > 0 ? n / bs : 0;
  return carve_size(sizeof(int) * 2) + scan_ws_bytes(nb + 1);
}

extern "C" int bilu_csr_to_bsr_rowptr(int n, int bs, const int* d_csrRowPtr,
                                      const int* d_csrColInd, int* d_bsrRowPtr, int* h_nnzb,
                                      void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (n < 0 || bs < 1 || bs > 8 || n % bs) return BILU_ERR_ARG;
  int nb = n / bs;
  Carver ws(d_ws, ws_bytes);
  int* err = ws.take<int>(2);
  if (!err) return BILU_ERR_WORKSPACE;
  cudaStream_t st = S(stream);
  BILU_TRY(init_err(err, st));
  if (nb > 0) {
    k_c2b_count<<<ceil_div(nb, 8), 256, 0, st>>>(nb, bs, d_csrRowPtr, d_csrColInd, n,
                                                 d_bsrRowPtr, err);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY(scan_exclusive(d_bsrRowPtr, d_bsrRowPtr, nb, h_nnzb, ws, st));
  int h_err[2];
  BILU_TRY(read_err(err, h_err, st));
  return h_err[1] ? BILU_ERR_PATTERN : BILU_OK;
}

extern "C" int bilu_csr_to_bsr_fill(int n, int bs, const int* d_csrRowPtr, const int* d_csrColInd,
                                    const double* d_csrVal, const int* d_bsrRowPtr,
                                    int* d_bsrColInd, double* d_bsrVal, bilu_stream_t stream) {
  if (n < 0 || bs < 1 || bs > 8 || n % bs) return BILU_ERR_ARG;
  int nb = n / bs;
  if (nb == 0) return BILU_OK;
  k_c2b_fill<<<ceil_div(nb, 8), 256, 0, S(stream)>>>(nb, bs, d_csrRowPtr, d_csrColInd, d_csrVal,
                                                     d_bsrRowPtr, d_bsrColInd, d_bsrVal);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

extern "C" int bilu_bsr_to_csr(int mb, int bs, const int* d_bsrRowPtr, const int* d_bsrColInd,
                               const double* d_bsrVal, int* d_csrRowPtr, int* d_csrColInd,
                               double* d_csrVal, bilu_stream_t stream) {
  if (mb < 0 || bs < 1 || bs > 8) return BILU_ERR_ARG;
  cudaStream_t st = S(stream);
  int nnzb = 0;
  if (mb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&nnzb, d_bsrRowPtr + mb, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  long long nrow = (long long)mb * bs + 1;
  k_b2c_rowptr<<<ceil_div(nrow, kT), kT, 0, st>>>(mb, bs, d_bsrRowPtr, d_csrRowPtr);
  BILU_LAUNCH_CHECK();
  if (nnzb == 0) return BILU_OK;
  long long total = (long long)nnzb * bs;
  k_b2c_fill<<<ceil_div(total, kT), kT, 0, st>>>(mb, bs, nnzb, d_bsrRowPtr, d_bsrColInd,
                                                 d_bsrVal, d_csrRowPtr, d_csrColInd, d_csrVal);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}
