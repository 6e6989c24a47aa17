// BSR SpMV / SpMM and the ISAI preconditioner apply (sm_103a).
//
// Replaces bcsr_spmv (bcsc2bcsrAndSpMV.h:49, thread per block row, scalar
// loops) and the DMMA variants of bsr_tensor_SpMV.h:21-400.  On GB300 the FP64
// pipe (measured 1.2 TFLOP/s DFMA, 1.05 TFLOP/s DMMA m8n8k4) is the binding
// limit of an FP64 BSR SpMV (1 DFMA per 8 B of values), so the layout spends
// FP64 instructions only on the block products: one lane per scalar row
// accumulates across every block of its block row and needs no reduction.
// The bs lanes of a block row read the bs rows of each block, so every block
// (bs*bs*8 bytes) is fetched in whole 32-byte sectors by one group, and the x
// segment is a broadcast within the group.
#include <algorithm>

#include <mutex>

#include "common.cuh"

namespace bilu {

namespace {

template <class T>
struct Vec;
template <>
struct Vec<double> {
  static constexpr int W = 2;
  using V = double2;
};
template <>
struct Vec<float> {
  static constexpr int W = 4;
  using V = float4;
};

__device__ __forceinline__ double to_acc(double v, double) { return v; }
__device__ __forceinline__ double to_acc(float v, double) { return (double)v; }
__device__ __forceinline__ float to_acc(double v, float) { return (float)v; }
__device__ __forceinline__ float to_acc(float v, float) { return v; }

// Load the BS-long x segment of block column bc into registers (AccT).
template <int BS, class XT, class AccT>
__device__ __forceinline__ void load_x(const XT* __restrict__ x, long long bc, AccT* xr) {
  const XT* p = x + bc * BS;
  constexpr int W = Vec<XT>::W;
  if constexpr (BS % W == 0) {
    // the segment starts at bc*BS elements: 16-byte aligned when BS is a
    // multiple of the vector width
    using V = typename Vec<XT>::V;
#pragma unroll
    for (int c = 0; c < BS / W; ++c) {
      V v = __ldg(reinterpret_cast<const V*>(p) + c);
      if constexpr (W == 2) {
        xr[2 * c] = to_acc(v.x, AccT());
        xr[2 * c + 1] = to_acc(v.y, AccT());
      } else {
        xr[4 * c] = to_acc(v.x, AccT());
        xr[4 * c + 1] = to_acc(v.y, AccT());
        xr[4 * c + 2] = to_acc(v.z, AccT());
        xr[4 * c + 3] = to_acc(v.w, AccT());
      }
    }
  } else {
#pragma unroll
    for (int c = 0; c < BS; ++c) xr[c] = to_acc(__ldg(p + c), AccT());
  }
}

// Row r of block p (BS values) into registers, streaming loads.
template <int BS, class VT, class AccT>
__device__ __forceinline__ void load_row(const VT* __restrict__ val, long long p, int r, AccT* a) {
  const VT* q = val + (p * BS + r) * BS;
  constexpr int W = Vec<VT>::W;
  if constexpr (BS % W == 0) {
    using V = typename Vec<VT>::V;
#pragma unroll
    for (int c = 0; c < BS / W; ++c) {
      V v = ld_stream(reinterpret_cast<const V*>(q) + c);
      if constexpr (W == 2) {
        a[2 * c] = to_acc(v.x, AccT());
        a[2 * c + 1] = to_acc(v.y, AccT());
      } else {
        a[4 * c] = to_acc(v.x, AccT());
        a[4 * c + 1] = to_acc(v.y, AccT());
        a[4 * c + 2] = to_acc(v.z, AccT());
        a[4 * c + 3] = to_acc(v.w, AccT());
      }
    }
  } else {
#pragma unroll
    for (int c = 0; c < BS; ++c) a[c] = to_acc(ld_stream(q + c), AccT());
  }
}

// Rows with more blocks than this are worth the CTA's help: power-law hub
// rows hold up to ~2000 blocks, and a lane group alone runs one dependent
// FMA chain over all of them while the rest of the GPU idles.
constexpr int kLongSpmvRow = 64;

// The CTA's long rows (slots in group order, -1 for none): its NG groups
// take the blocks g, g + NG, ... of each (two accumulators, even and odd
// turns), the NG partials are added in group order.  Out of line so that
// the short rows' loop keeps its registers.  Called by every thread.
template <int BS, class VT, class XT, class YT, class AccT, int NSLOT, int NG>
__device__ __noinline__ void spmv_long_rows(const int* long_rows, const int* __restrict__ row,
                                            const int* __restrict__ col,
                                            const VT* __restrict__ val,
                                            const XT* __restrict__ x, YT* __restrict__ y,
                                            float* __restrict__ y32, AccT* red, bool in_group,
                                            int cg, int r) {
  for (int i = 0; i < NSLOT; ++i) {
    const int br = long_rows[i];
    if (br < 0) continue;  // uniform across the CTA (shared memory)
    const int rs = __ldg(row + br), re = __ldg(row + br + 1);
    AccT a0 = 0, a1 = 0;
    if (in_group) {
      int p = rs + cg;
      for (; p + NG < re; p += 2 * NG) {
        AccT v0[BS], v1[BS], x0[BS], x1[BS];
        load_row<BS, VT, AccT>(val, p, r, v0);
        load_row<BS, VT, AccT>(val, p + NG, r, v1);
        load_x<BS, XT, AccT>(x, __ldg(col + p), x0);
        load_x<BS, XT, AccT>(x, __ldg(col + p + NG), x1);
#pragma unroll
        for (int k = 0; k < BS; ++k) {
          a0 = fma(v0[k], x0[k], a0);
          a1 = fma(v1[k], x1[k], a1);
        }
      }
      if (p < re) {
        AccT v0[BS], x0[BS];
        load_row<BS, VT, AccT>(val, p, r, v0);
        load_x<BS, XT, AccT>(x, __ldg(col + p), x0);
#pragma unroll
        for (int k = 0; k < BS; ++k) a0 = fma(v0[k], x0[k], a0);
      }
      red[cg * BS + r] = a0 + a1;
    }
    __syncthreads();
    if (threadIdx.x < BS) {
      AccT t = 0;
      for (int q = 0; q < NG; ++q) t += red[q * BS + threadIdx.x];
      y[(long long)br * BS + threadIdx.x] = (YT)t;
      if (y32) y32[(long long)br * BS + threadIdx.x] = (float)t;
    }
    __syncthreads();
  }
}

// y = M x: lane group of BS lanes per block row, lane r owns scalar row r.
// A group handles RPG consecutive block rows and issues the loads of the
// next U blocks of all of them before any arithmetic, so a warp keeps
// RPG*U independent block loads per lane in flight; each row's sum runs in
// block order whatever U and RPG are (the same bits).  Chosen by
// launch_spmv from measurements on the 128^3 7-point pattern (7 blocks a
// row) and its triangle (4 a row): FP64 values U = 1, RPG = 2 (two
// independent DFMA chains per lane; one chain is latency-bound: 0.48 ->
// 0.40 ms on the 7-point FP64 operator, the same on the triangle); FP32
// values U = 4 with RPG = 1 for wider rows (0.199 -> 0.176 ms on the FP32
// operator), RPG = 1 at 8 CTAs per SM for bs 4 rows of ~4 blocks, else
// RPG = 2.  LONG (matrices with rows of more than kLongSpmvRow blocks):
// such a row is skipped by its group and summed after the short rows by
// the whole CTA (dynamic shared memory: the CTA's long-row slots and the
// group partials); the other instance has no CTA barrier at all.
template <int BS, class VT, class XT, class YT, class AccT, int RPG, int U, int MINB, bool LONG>
__global__ void __launch_bounds__(256, MINB) k_bsr_spmv(int mb, const int* __restrict__ row,
                                                     const int* __restrict__ col,
                                                     const VT* __restrict__ val,
                                                     const XT* __restrict__ x,
                                                     YT* __restrict__ y,
                                                     float* __restrict__ y32) {
  constexpr int G = 32 / BS;  // lane groups per warp
  int lane = threadIdx.x & 31;
  int g = lane / BS, r = lane - g * BS;
  long long base = (((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * G + g) * RPG;
  const bool active = g < G && base < mb;
  if (!LONG && !active) return;
  int s[RPG], e[RPG];
  bool skip[RPG], mine_long = false;
  extern __shared__ int long_slots[];  // LONG: [8*G*RPG] slots, then the partials
  const int cg = (threadIdx.x >> 5) * G + g;
#pragma unroll
  for (int q = 0; q < RPG; ++q) {
    bool ok = active && base + q < mb;
    s[q] = ok ? __ldg(row + base + q) : 0;
    e[q] = ok ? __ldg(row + base + q + 1) : 0;
    skip[q] = false;
    if constexpr (LONG) {
      skip[q] = e[q] - s[q] > kLongSpmvRow;
      if (g < G && r == 0) long_slots[cg * RPG + q] = skip[q] ? (int)(base + q) : -1;
      if (skip[q]) e[q] = s[q];
      mine_long |= skip[q];
    }
  }
  AccT acc[RPG];
#pragma unroll
  for (int q = 0; q < RPG; ++q) acc[q] = 0;
  // batches of U blocks per row; every load of a batch (column indices,
  // block rows, x segments) is issued before its FMAs
  for (int off = 0; active; off += U) {
    bool any = false;
#pragma unroll
    for (int q = 0; q < RPG; ++q) any |= s[q] + off < e[q];
    if (!any) break;
    int c[RPG][U];
#pragma unroll
    for (int q = 0; q < RPG; ++q)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        int p = s[q] + off + u;
        c[q][u] = p < e[q] ? __ldg(col + p) : -1;
      }
    AccT a[RPG][U][BS], xv[RPG][U][BS];
#pragma unroll
    for (int q = 0; q < RPG; ++q)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (c[q][u] >= 0) {
          load_row<BS, VT, AccT>(val, s[q] + off + u, r, a[q][u]);
        } else {
#pragma unroll
          for (int k = 0; k < BS; ++k) a[q][u][k] = 0;
        }
      }
    // x segments (mostly L2 hits) are consumed as they arrive, which keeps
    // the register footprint low enough for 4 CTAs per SM with FP32 values
#pragma unroll
    for (int q = 0; q < RPG; ++q)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (c[q][u] >= 0) {
          load_x<BS, XT, AccT>(x, c[q][u], xv[q][u]);
#pragma unroll
          for (int k = 0; k < BS; ++k) acc[q] = fma(a[q][u][k], xv[q][u][k], acc[q]);
        }
      }
  }
#pragma unroll
  for (int q = 0; q < RPG; ++q)
    if (active && base + q < mb && !skip[q]) {
      y[(base + q) * BS + r] = (YT)acc[q];
      if (y32) y32[(base + q) * BS + r] = (float)acc[q];  // optional FP32 copy
    }
  if constexpr (LONG) {
    constexpr int NSLOT = 8 * G * RPG;
    // one CTA barrier, which also says whether the CTA holds a long row
    if (__syncthreads_or(mine_long))
      spmv_long_rows<BS, VT, XT, YT, AccT, NSLOT, 8 * G>(
          long_slots, row, col, val, x, y, y32,
          reinterpret_cast<AccT*>(long_slots + ((NSLOT + 1) & ~1)), g < G, cg, r);
  }
}

// Layout word of a matrix for the SpMV: bit 0 = rows of more than
// kLongSpmvRow blocks present (the LONG instance); bit 1 = more than
// kWideSpmvRow blocks a row on average (FP32 values: one row per lane
// group).  (Taking several blocks of a row side by side, or rows in length
// order, was measured slower on the power-law patterns: the product is
// latency-bound there, not bound by the lanes an uneven warp leaves idle.)
constexpr int kLayoutLong = 1;
constexpr int kLayoutWide = 2;
constexpr int kWideSpmvRow = 5;

template <int BS, class VT, class XT, class YT, int RPG, int U, int MINB, bool LONG>
int launch_spmv_cfg(int mb, const int* row, const int* col, const VT* val, const XT* x, YT* y,
                    cudaStream_t st, float* y32) {
  using AccT = VT;
  constexpr int G = 32 / BS;
  long long groups = (mb + RPG - 1) / RPG;
  long long warps = (groups + G - 1) / G;
  unsigned grid = ceil_div(warps, 8);
  if constexpr (LONG) {
    constexpr int NSLOT = 8 * G * RPG;
    const size_t smem = sizeof(int) * ((NSLOT + 1) & ~1) + sizeof(AccT) * 8 * G * BS;
    k_bsr_spmv<BS, VT, XT, YT, AccT, RPG, U, MINB, true><<<grid, 256, smem, st>>>(
        mb, row, col, val, x, y, y32);
  } else {
    k_bsr_spmv<BS, VT, XT, YT, AccT, RPG, U, MINB, false><<<grid, 256, 0, st>>>(
        mb, row, col, val, x, y, y32);
  }
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// Patterns with long rows (power-law: rows of ~12 blocks on average, hubs
// of up to 2000) are latency-bound per lane group and keep two blocks a
// batch (FP64) or two rows a group (FP32); the configurations measured
// faster on the stencil patterns (above) apply to patterns without long
// rows, FP64 at block sizes 4 and 5.
template <int BS, class VT, class XT, class YT>
int launch_spmv(int mb, const int* row, const int* col, const VT* val, const XT* x, YT* y,
                cudaStream_t st, int layout, float* y32 = nullptr) {
  if (mb == 0) return BILU_OK;
  const bool lng = (layout & kLayoutLong) != 0;
  if constexpr (sizeof(VT) == 8) {
    if (lng)
      return launch_spmv_cfg<BS, VT, XT, YT, 1, 2, 2, true>(mb, row, col, val, x, y, st, y32);
    if constexpr (BS <= 5)
      return launch_spmv_cfg<BS, VT, XT, YT, 2, 1, 4, false>(mb, row, col, val, x, y, st, y32);
    else
      return launch_spmv_cfg<BS, VT, XT, YT, 1, 2, 2, false>(mb, row, col, val, x, y, st, y32);
  } else if constexpr (BS == 8 && sizeof(XT) == 8) {
    // two rows of 8x8 blocks with FP64 x segments spill at 64 registers
    if (lng)
      return launch_spmv_cfg<BS, VT, XT, YT, 1, 4, 4, true>(mb, row, col, val, x, y, st, y32);
    return launch_spmv_cfg<BS, VT, XT, YT, 1, 4, 4, false>(mb, row, col, val, x, y, st, y32);
  } else {
    if (lng)
      return launch_spmv_cfg<BS, VT, XT, YT, 2, 4, 4, true>(mb, row, col, val, x, y, st, y32);
    if (layout & kLayoutWide)
      return launch_spmv_cfg<BS, VT, XT, YT, 1, 4, 4, false>(mb, row, col, val, x, y, st, y32);
    // bs 4 rows of ~4 blocks (the ISAI triangles of a 7-point pattern): one
    // row per group at 32 registers, 8 CTAs per SM (0.2214 -> 0.2185 ms
    // for the 128^3 inner apply)
    if constexpr (BS == 4)
      return launch_spmv_cfg<BS, VT, XT, YT, 1, 4, 8, false>(mb, row, col, val, x, y, st, y32);
    return launch_spmv_cfg<BS, VT, XT, YT, 2, 4, 4, false>(mb, row, col, val, x, y, st, y32);
  }
}

// Multi-RHS: Y[n,k] = M X[n,k], row-major with ld = k.  One warp per block
// row; lane c (and c+32) owns right-hand side c; blocks are broadcast reads.
template <int BS, class VT, int KW>
__global__ void __launch_bounds__(256) k_bsr_spmm(int mb, int k, const int* __restrict__ row,
                                                  const int* __restrict__ col,
                                                  const VT* __restrict__ val,
                                                  const double* __restrict__ X,
                                                  double* __restrict__ Y) {
  using AccT = VT;
  int lane = threadIdx.x & 31;
  long long br = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (br >= mb) return;
  AccT acc[KW][BS];
#pragma unroll
  for (int w = 0; w < KW; ++w)
#pragma unroll
    for (int r = 0; r < BS; ++r) acc[w][r] = 0;
  int s = row[br], e = row[br + 1];
  for (int p = s; p < e; ++p) {
    long long bc = col[p];
    const VT* blk = val + (long long)p * BS * BS;
#pragma unroll
    for (int kk = 0; kk < BS; ++kk) {
      AccT xv[KW];
#pragma unroll
      for (int w = 0; w < KW; ++w) {
        int c = lane + 32 * w;
        xv[w] = c < k ? (AccT)X[(bc * BS + kk) * k + c] : (AccT)0;
      }
#pragma unroll
      for (int r = 0; r < BS; ++r) {
        AccT a = (AccT)blk[r * BS + kk];
#pragma unroll
        for (int w = 0; w < KW; ++w) acc[w][r] = fma(a, xv[w], acc[w][r]);
      }
    }
  }
#pragma unroll
  for (int w = 0; w < KW; ++w) {
    int c = lane + 32 * w;
    if (c < k)
#pragma unroll
      for (int r = 0; r < BS; ++r) Y[(br * BS + r) * k + c] = (double)acc[w][r];
  }
}

template <int BS, class VT>
int launch_spmm(int mb, int k, const int* row, const int* col, const VT* val, const double* X,
                double* Y, cudaStream_t st) {
  if (mb == 0) return BILU_OK;
  unsigned grid = ceil_div(mb, 8);
  if (k <= 32)
    k_bsr_spmm<BS, VT, 1><<<grid, 256, 0, st>>>(mb, k, row, col, val, X, Y);
  else
    k_bsr_spmm<BS, VT, 2><<<grid, 256, 0, st>>>(mb, k, row, col, val, X, Y);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

__global__ void k_f64_to_f32(size_t n, const double* __restrict__ s, float* __restrict__ d) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) d[i] = __double2float_rn(s[i]);
}

template <int BS>
int spmv_f64(int mb, const int* row, const int* col, const double* val, const double* x,
             double* y, cudaStream_t st, int lr) {
  return launch_spmv<BS, double, double, double>(mb, row, col, val, x, y, st, lr);
}

template <int BS>
int spmv_f32(int mb, const int* row, const int* col, const float* val, const void* x, int x32,
             void* y, int y32, cudaStream_t st, int lr) {
  if (x32 && y32)
    return launch_spmv<BS, float, float, float>(mb, row, col, val, (const float*)x, (float*)y, st,
                                                lr);
  if (x32)
    return launch_spmv<BS, float, float, double>(mb, row, col, val, (const float*)x, (double*)y,
                                                 st, lr);
  if (y32)
    return launch_spmv<BS, float, double, float>(mb, row, col, val, (const double*)x, (float*)y,
                                                 st, lr);
  return launch_spmv<BS, float, double, double>(mb, row, col, val, (const double*)x, (double*)y,
                                                st, lr);
}

// FP32 values and x, FP64 y plus its FP32 copy y32
template <int BS>
int spmv_f32_dual(int mb, const int* row, const int* col, const float* val, const float* x,
                  double* y, float* y32, cudaStream_t st, int lr) {
  return launch_spmv<BS, float, float, double>(mb, row, col, val, x, y, st, lr, y32);
}

__global__ void k_row_len_max(int mb, const int* __restrict__ row, int* out) {
  int m = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < mb;
       i += (long long)gridDim.x * blockDim.x)
    m = max(m, __ldg(row + i + 1) - __ldg(row + i));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}

template <int BS>
int spmm_f64(int mb, int k, const int* row, const int* col, const double* val, const double* X,
             double* Y, cudaStream_t st) {
  return launch_spmm<BS, double>(mb, k, row, col, val, X, Y, st);
}
template <int BS>
int spmm_f32(int mb, int k, const int* row, const int* col, const float* val, const double* X,
             double* Y, cudaStream_t st) {
  return launch_spmm<BS, float>(mb, k, row, col, val, X, Y, st);
}

}  // namespace

// SpMV layout word of a block pattern (see kLayoutLong): one reduction
// over the row pointers into d_words (one device int), then a synchronising
// read of it and of the block count row[mb].  The engine calls it once per
// matrix at setup.
int spmv_layout_of(int mb, int bs, const int* row, void* d_words, cudaStream_t st,
                   int* h_layout) {
  (void)bs;
  *h_layout = 0;
  if (mb <= 0) return BILU_OK;
  int h[2] = {0, 0};  // longest row, blocks
  int* d = static_cast<int*>(d_words);
  BILU_TRY_CUDA(cudaMemsetAsync(d, 0, sizeof(int), st));
  k_row_len_max<<<(unsigned)std::min<long long>(ceil_div(mb, 256), 152 * 8), 256, 0, st>>>(
      mb, row, d);
  BILU_LAUNCH_CHECK();
  BILU_TRY_CUDA(cudaMemcpyAsync(&h[0], d, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaMemcpyAsync(&h[1], row + mb, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  *h_layout = (h[0] > kLongSpmvRow ? kLayoutLong : 0) |
              ((long long)h[1] > (long long)kWideSpmvRow * mb ? kLayoutWide : 0);
  return BILU_OK;
}

namespace {

__device__ int g_layout_word;  // scratch of the cached check (under its lock)

// The standalone entry points do not know the pattern: the answer is cached
// per (row pointer array, block rows, block size), most recent first.  A
// stale entry (a buffer reused for another pattern) can only cost speed:
// both kernels are exact for any row length.
struct LayoutEntry {
  const int* row;
  int mb, bs, layout;
};
std::mutex g_layout_mu;
LayoutEntry g_layout_cache[16] = {};
int g_layout_next = 0;

// under g_layout_mu: the entry of (row, mb, bs), or null
LayoutEntry* layout_find(int mb, int bs, const int* row) {
  for (LayoutEntry& e : g_layout_cache)
    if (e.row == row && e.mb == mb && e.bs == bs && row) return &e;
  return nullptr;
}

int layout_cached(int mb, int bs, const int* row, cudaStream_t st, int* out) {
  std::lock_guard<std::mutex> lock(g_layout_mu);
  if (const LayoutEntry* e = layout_find(mb, bs, row)) {
    *out = e->layout;
    return BILU_OK;
  }
  void* words = nullptr;
  BILU_TRY_CUDA(cudaGetSymbolAddress(&words, g_layout_word));
  int layout = 0;
  BILU_TRY(spmv_layout_of(mb, bs, row, words, st, &layout));
  g_layout_cache[g_layout_next] = LayoutEntry{row, mb, bs, layout};
  g_layout_next = (g_layout_next + 1) % 16;
  *out = layout;
  return BILU_OK;
}

}  // namespace

// internal entry point used by the solver; layout: the pattern's layout
// word when the caller knows it (spmv_layout_of), -1 to look it up
int spmv_any(int mb, int bs, int prec, const int* row, const int* col, const void* val,
             const void* x, int x32, void* y, int y32, cudaStream_t st, int layout) {
  int lr = layout;
  if (layout < 0) BILU_TRY(layout_cached(mb, bs, row, st, &lr));
  if (prec == BILU_FP64) {
    if (x32 || y32) return BILU_ERR_ARG;
    return BILU_DISPATCH_BS(bs, spmv_f64, mb, row, col, (const double*)val, (const double*)x,
                            (double*)y, st, lr);
  }
  return BILU_DISPATCH_BS(bs, spmv_f32, mb, row, col, (const float*)val, x, x32, y, y32, st, lr);
}

int convert_f64_f32(size_t count, const double* src, float* dst, cudaStream_t st) {
  if (count == 0) return BILU_OK;
  unsigned grid = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  k_f64_to_f32<<<grid, 256, 0, st>>>(count, src, dst);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// FP32 path: b is rounded to FP32 once (n conversions; converting inside the
// SpMV would cost one FP64-pipe conversion per block element, the slowest
// operation on GB300), staged in the output buffer (n doubles hold n floats),
// then y32 = M_L b32 and x = M_U y32 with FP32 accumulation.
int isai_apply_impl(int nb, int bs, int prec, const int* Lrow, const int* Lcol, const void* Lval,
                    const int* Urow, const int* Ucol, const void* Uval, const double* b,
                    void* tmp, double* x, cudaStream_t st, int longL, int longU) {
  if (prec == BILU_FP32) {
    float* b32 = reinterpret_cast<float*>(x);
    BILU_TRY(convert_f64_f32((size_t)nb * bs, b, b32, st));
    BILU_TRY(spmv_any(nb, bs, prec, Lrow, Lcol, Lval, b32, 1, tmp, 1, st, longL));
    return spmv_any(nb, bs, prec, Urow, Ucol, Uval, tmp, 1, x, 0, st, longU);
  }
  BILU_TRY(spmv_any(nb, bs, prec, Lrow, Lcol, Lval, b, 0, tmp, 0, st, longL));
  return spmv_any(nb, bs, prec, Urow, Ucol, Uval, tmp, 0, x, 0, st, longU);
}

// Solver form: the FP32 copy of the input is already there (written by the
// kernel that produced the FP64 basis vector).
int isai_apply_f32_staged(int nb, int bs, const int* Lrow, const int* Lcol, const float* Lval,
                          const int* Urow, const int* Ucol, const float* Uval, const float* b32,
                          float* tmp, double* x, cudaStream_t st, float* x32, int longL,
                          int longU) {
  BILU_TRY(spmv_any(nb, bs, BILU_FP32, Lrow, Lcol, Lval, b32, 1, tmp, 1, st, longL));
  if (x32) {  // x also in FP32 (input of an FP32 operator product)
    int lr = longU;
    if (longU < 0) BILU_TRY(layout_cached(nb, bs, Urow, st, &lr));
    return BILU_DISPATCH_BS(bs, spmv_f32_dual, nb, Urow, Ucol, Uval, tmp, x, x32, st, lr);
  }
  return spmv_any(nb, bs, BILU_FP32, Urow, Ucol, Uval, tmp, 1, x, 0, st, longU);
}

}  // namespace bilu

using namespace bilu;

extern "C" int bilu_bcsr_spmv(int mb, int bs, const int* d_row, const int* d_col,
                              const double* d_val, const double* d_x, double* d_y,
                              bilu_stream_t stream) {
  if (mb < 0 || (mb > 0 && (!d_row || !d_col || !d_val || !d_x || !d_y))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return spmv_any(mb, bs, BILU_FP64, d_row, d_col, d_val, d_x, 0, d_y, 0, S(stream), -1);
}

extern "C" int bilu_spmv_layout(int mb, int bs, const int* d_row, bilu_stream_t stream,
                                int* h_layout) {
  if (mb < 0 || !h_layout || (mb > 0 && !d_row)) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return layout_cached(mb, bs, d_row, S(stream), h_layout);
}

extern "C" int bilu_debug_spmv_layout_set(int mb, int bs, const int* d_row, int layout) {
  if (mb < 0 || (mb > 0 && !d_row) || layout < 0 || layout > (kLayoutLong | kLayoutWide))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_layout_mu);
  if (LayoutEntry* e = layout_find(mb, bs, d_row)) {
    e->layout = layout;
  } else {
    g_layout_cache[g_layout_next] = LayoutEntry{d_row, mb, bs, layout};
    g_layout_next = (g_layout_next + 1) % 16;
  }
  return BILU_OK;
}

extern "C" int bilu_bcsr_spmv_f32(int mb, int bs, const int* d_row, const int* d_col,
                                  const float* d_val, const void* d_x, int x_fp32, void* d_y,
                                  int y_fp32, bilu_stream_t stream) {
  if (mb < 0 || (mb > 0 && (!d_row || !d_col || !d_val || !d_x || !d_y))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return spmv_any(mb, bs, BILU_FP32, d_row, d_col, d_val, d_x, x_fp32 != 0, d_y, y_fp32 != 0,
                  S(stream), -1);
}

extern "C" int bilu_bcsr_spmm(int mb, int bs, int k, const int* d_row, const int* d_col,
                              const double* d_val, const double* d_X, double* d_Y,
                              bilu_stream_t stream) {
  if (mb < 0 || k < 1 || k > 64) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return BILU_DISPATCH_BS(bs, spmm_f64, mb, k, d_row, d_col, d_val, d_X, d_Y, S(stream));
}

extern "C" int bilu_bcsr_spmm_f32(int mb, int bs, int k, const int* d_row, const int* d_col,
                                  const float* d_val, const double* d_X, double* d_Y,
                                  bilu_stream_t stream) {
  if (mb < 0 || k < 1 || k > 64) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return BILU_DISPATCH_BS(bs, spmm_f32, mb, k, d_row, d_col, d_val, d_X, d_Y, S(stream));
}

extern "C" int bilu_convert_f64_to_f32(size_t count, const double* d_src, float* d_dst,
                                       bilu_stream_t stream) {
  if (count == 0) return BILU_OK;
  if (!d_src || !d_dst) return BILU_ERR_ARG;
  unsigned grid = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  k_f64_to_f32<<<grid, 256, 0, S(stream)>>>(count, d_src, d_dst);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

extern "C" int bilu_isai_apply(int nb, int bs, int prec, const int* d_Lrow, const int* d_Lcol,
                               const void* d_Lval, const int* d_Urow, const int* d_Ucol,
                               const void* d_Uval, const double* d_b, void* d_tmp, double* d_x,
                               bilu_stream_t stream) {
  if (nb < 0 || (prec != BILU_FP64 && prec != BILU_FP32)) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return isai_apply_impl(nb, bs, prec, d_Lrow, d_Lcol, d_Lval, d_Urow, d_Ucol, d_Uval, d_b,
                         d_tmp, d_x, S(stream), -1, -1);
}
