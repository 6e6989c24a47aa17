// Sync-free kernels with per-block-row ready flags (sm_103a):
//
//   bsrilu02_inplace (bsrilu.h:20, cuSPARSE bsrilu02)   -> k_bilu0
//   spTrSolveL / spTrSolveU (cape_sptrsv.h:8,55)         -> k_sptrsv
//
// A warp owns one block row at a time.  Rows are handed out by an atomic
// ticket counter, so every row a warp waits on was taken by a warp that is
// already running (the reference maps rows to threads statically and relies
// on scheduling order).  A finished row publishes its flag with st.release
// after a __threadfence by every writer lane; waiters poll with ld.acquire
// and read the producer's data through L2 (ld.cg).  Every wait is bounded:
// after kSpinLimit polls the waiter sets the error word to BILU_ERR_TIMEOUT,
// and all other waiters see the error word and leave, so no launch hangs.
#include <climits>

#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace bilu {

namespace {

constexpr unsigned FULL = 0xffffffffu;

struct SyncState {
  int* flags;         // nb ready flags
  int* ticket;        // row counter
  int* err;           // 0 or a bilu_status
  int* zp;            // first zero pivot row (INT_MAX if none)
  long long spin;     // polls before a wait gives up
  int withhold;       // test hook: this row never publishes (-1: none)
  const int* order;   // ticket -> block row (dependency-level order), or null
};

// Warp-wide wait until flags[K] != 0.  Returns false if the launch aborted.
__device__ __forceinline__ bool warp_wait(const int* flag, int* err, long long spin) {
  long long n = 0;
  while (true) {
    int v = ld_acquire(flag);
    if (__all_sync(FULL, v != 0)) return true;
    if (__any_sync(FULL, ld_relaxed(err) != 0)) return false;
    if (++n > spin) {
      if ((threadIdx.x & 31) == 0) atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    __nanosleep(32);
  }
}

// Single-lane wait (lanes of a warp may wait on different rows).
__device__ __forceinline__ bool lane_wait(const int* flag, int* err, long long spin) {
  long long n = 0;
  while (ld_acquire(flag) == 0) {
    if (ld_relaxed(err) != 0) return false;
    if (++n > spin) {
      atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    __nanosleep(32);
  }
  return true;
}

__device__ __forceinline__ int find_in_row(const int* __restrict__ col, int s, int e, int key) {
  int lo = s, hi = e - 1;
  while (lo <= hi) {
    int m = (lo + hi) >> 1;
    int v = __ldg(col + m);
    if (v == key) return m;
    if (v < key) lo = m + 1; else hi = m - 1;
  }
  return -1;
}

__global__ void k_diag_pos(int nb, const int* __restrict__ row, const int* __restrict__ col,
                           int* __restrict__ diag, int* bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  int s = row[i], e = row[i + 1];
  int prev = -1;
  for (int p = s; p < e; ++p) {
    int c = col[p];
    if (c <= prev || c < 0 || c >= nb) { atomicMin(bad, i); diag[i] = -1; return; }
    prev = c;
  }
  int d = find_in_row(col, s, e, i);
  diag[i] = d;
  if (d < 0) atomicMin(bad, i);
}

// ------------------------------------------------------------------ BILU(0)
// Scalar ILU(0) on the block pattern in IKJ order, blockwise:
//   for K < I in row I:  L_IK = A_IK U_KK^-1 (row-wise forward elimination),
//                        A_IJ -= L_IK U_KJ for J > K present in rows I and K;
//   then LU of the diagonal block (no pivoting) and U_IJ = L_II^-1 A_IJ.
// Each element sees the same sequence of a -= l*u updates as the scalar IKJ
// loop, with ascending k.
template <int BS>
__global__ void __launch_bounds__(128) k_bilu0(int nb, const int* __restrict__ row,
                                               const int* __restrict__ col,
                                               const int* __restrict__ diag, double* val,
                                               SyncState ss) {
  constexpr int BS2 = BS * BS;
  constexpr int EPL = BS2 > 32 ? 2 : 1;
  constexpr int TL = BS2 / EPL + (BS2 % EPL ? 1 : 0);
  constexpr int TPW = 32 / TL;         // blocks updated per pass in phase 2
  constexpr int SPAN = 32 / TPW;
  constexpr int GU = 32 / BS;          // U blocks per pass (lane = column)
  int lane = threadIdx.x & 31;
  int team = lane / SPAN, tl = lane - team * SPAN;
  bool team_on = team < TPW && tl < TL;
  while (true) {
    int I = 0;
    if (lane == 0) I = atomicAdd(ss.ticket, 1);
    I = __shfl_sync(FULL, I, 0);
    if (I >= nb) return;
    if (ss.order) I = __ldg(ss.order + I);
    if (__any_sync(FULL, ld_relaxed(ss.err) != 0)) return;
    int rs = __ldg(row + I), re = __ldg(row + I + 1), dI = __ldg(diag + I);
    for (int pk = rs; pk < dI; ++pk) {
      int K = __ldg(col + pk);
      if (!warp_wait(ss.flags + K, ss.err, ss.spin)) return;
      int dK = __ldg(diag + K), ke = __ldg(row + K + 1);
      double* L = val + (long long)pk * BS2;
      const double* Ukk = val + (long long)dK * BS2;
      // phase 1: lane r owns row r of A_IK
      if (lane < BS) {
        double a[BS];
#pragma unroll
        for (int c = 0; c < BS; ++c) a[c] = L[lane * BS + c];
#pragma unroll
        for (int k = 0; k < BS; ++k) {
          a[k] = a[k] / __ldcg(Ukk + k * BS + k);
#pragma unroll
          for (int c = k + 1; c < BS; ++c) a[c] -= a[k] * __ldcg(Ukk + k * BS + c);
        }
#pragma unroll
        for (int c = 0; c < BS; ++c) L[lane * BS + c] = a[c];
      }
      __syncwarp();
      // phase 2: A_IJ -= L_IK U_KJ, team per candidate block J of row I
      for (int pj0 = pk + 1; pj0 < re; pj0 += TPW) {
        int pj = pj0 + team;
        int pos = -1;
        if (team < TPW && pj < re) pos = find_in_row(col, dK + 1, ke, __ldg(col + pj));
        if (team_on && pos >= 0) {
          double* Aij = val + (long long)pj * BS2;
          const double* Ukj = val + (long long)pos * BS2;
#pragma unroll
          for (int q = 0; q < EPL; ++q) {
            int e = tl * EPL + q;
            if (e < BS2) {
              int r = e / BS, c = e - r * BS;
              double v = Aij[e];
#pragma unroll
              for (int k = 0; k < BS; ++k) v -= L[r * BS + k] * __ldcg(Ukj + k * BS + c);
              Aij[e] = v;
            }
          }
        }
      }
      __syncwarp();
    }
    // diagonal block: lane c owns column c
    double* D = val + (long long)dI * BS2;
    double dc[BS];
    if (lane < BS) {
#pragma unroll
      for (int r = 0; r < BS; ++r) dc[r] = D[r * BS + lane];
    } else {
#pragma unroll
      for (int r = 0; r < BS; ++r) dc[r] = 1.0;
    }
#pragma unroll
    for (int r = 1; r < BS; ++r) {
#pragma unroll
      for (int k = 0; k < r; ++k) {
        double lk = dc[r] / dc[k];  // meaningful on lane k
        double l = __shfl_sync(FULL, lk, k);
        if (lane == k) dc[r] = l;
        else if (lane > k && lane < BS) dc[r] -= l * dc[k];
      }
    }
    if (lane < BS) {
      if (dc[lane] == 0.0) atomicMin(ss.zp, I);
#pragma unroll
      for (int r = 0; r < BS; ++r) D[r * BS + lane] = dc[r];
    }
    __syncwarp();
    // U blocks right of the diagonal: U_IJ = L_II^-1 A_IJ, lane per column
    for (int pj0 = dI + 1; pj0 < re; pj0 += GU) {
      int slot = lane / BS, c = lane - slot * BS;
      int pj = pj0 + slot;
      if (slot < GU && pj < re) {
        double* U = val + (long long)pj * BS2;
        double u[BS];
#pragma unroll
        for (int r = 0; r < BS; ++r) u[r] = U[r * BS + c];
#pragma unroll
        for (int r = 1; r < BS; ++r)
#pragma unroll
          for (int k = 0; k < r; ++k) u[r] -= D[r * BS + k] * u[k];
#pragma unroll
        for (int r = 1; r < BS; ++r) U[r * BS + c] = u[r];
      }
    }
    __threadfence();
    __syncwarp();
    if (lane == 0 && I != ss.withhold) st_release(ss.flags + I, 1);
  }
}

// ------------------------------------------------------------------ SpTRSV
// Block-row solve on a packed factor.  LOWER: x_I = b_I - sum_{K<I} B_IK x_K
// then the diagonal block's lower part; otherwise the upper part and J > I
// in reverse ticket order.  UNIT: the diagonal block contributes its strict
// triangle and no division (unit diagonal).  Lane (slot, r) accumulates row
// r of blocks slot, slot+G, ...; slots are summed by shuffles.
template <int BS, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(128) k_sptrsv(int nb, const int* __restrict__ row,
                                                const int* __restrict__ col,
                                                const int* __restrict__ diag,
                                                const double* __restrict__ val,
                                                const double* __restrict__ b, double* x,
                                                SyncState ss) {
  constexpr int BS2 = BS * BS;
  constexpr int G = 32 / BS;
  int lane = threadIdx.x & 31;
  int slot = lane / BS, r = lane - slot * BS;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ss.ticket, 1);
    t = __shfl_sync(FULL, t, 0);
    if (t >= nb) return;
    int I = ss.order ? __ldg(ss.order + t) : (LOWER ? t : nb - 1 - t);
    int rs = __ldg(row + I), re = __ldg(row + I + 1), dI = __ldg(diag + I);
    int ps = LOWER ? rs : dI + 1, pe = LOWER ? dI : re;
    double s = 0.0;
    bool ok = true;
    for (int p0 = ps; p0 < pe; p0 += G) {
      int p = p0 + slot;
      if (slot < G && p < pe && ok) {
        int K = __ldg(col + p);
        ok = lane_wait(ss.flags + K, ss.err, ss.spin);
        if (ok) {
          const double* blk = val + (long long)p * BS2 + r * BS;
          const double* xk = x + (long long)K * BS;
#pragma unroll
          for (int c = 0; c < BS; ++c) s = fma(__ldg(blk + c), __ldcg(xk + c), s);
        }
      }
    }
    if (__any_sync(FULL, !ok)) return;
    double tot = 0.0;
#pragma unroll
    for (int g = 0; g < G; ++g) tot += __shfl_sync(FULL, s, g * BS + r);
    // diagonal block on lane 0
    double xr[BS];
#pragma unroll
    for (int q = 0; q < BS; ++q) xr[q] = __shfl_sync(FULL, tot, q);
    if (lane == 0) {
      const double* D = val + (long long)dI * BS2;
      const double* bi = b + (long long)I * BS;
      if (LOWER) {
#pragma unroll
        for (int q = 0; q < BS; ++q) {
          double v = bi[q] - xr[q];
#pragma unroll
          for (int c = 0; c < q; ++c) v -= __ldg(D + q * BS + c) * xr[c];
          xr[q] = UNIT ? v : v / __ldg(D + q * BS + q);
        }
      } else {
#pragma unroll
        for (int q = BS - 1; q >= 0; --q) {
          double v = bi[q] - xr[q];
#pragma unroll
          for (int c = q + 1; c < BS; ++c) v -= __ldg(D + q * BS + c) * xr[c];
          xr[q] = UNIT ? v : v / __ldg(D + q * BS + q);
        }
      }
#pragma unroll
      for (int q = 0; q < BS; ++q) x[(long long)I * BS + q] = xr[q];
      __threadfence();
      if (I != ss.withhold) st_release(ss.flags + I, 1);
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ levels
// Dependency level of every block row (1 + the deepest row it waits on),
// thread per row, sync-free like the solves: rows are taken in ticket order,
// a row waits (bounded) for the levels of its dependencies and publishes its
// own.  The lower DAG follows the strictly lower blocks, the upper DAG the
// strictly upper ones in reverse order.
template <bool LOWER>
__global__ void __launch_bounds__(256) k_levels(int nb, const int* __restrict__ row,
                                                const int* __restrict__ col,
                                                const int* __restrict__ diag, int* level,
                                                int* ticket, int* err, long long spin) {
  while (true) {
    int t = atomicAdd(ticket, 1);
    if (t >= nb) return;
    int I = LOWER ? t : nb - 1 - t;
    int ps = LOWER ? __ldg(row + I) : __ldg(diag + I) + 1;
    int pe = LOWER ? __ldg(diag + I) : __ldg(row + I + 1);
    int lv = 0;
    for (int p = ps; p < pe; ++p) {
      const int* f = level + __ldg(col + p);
      long long n = 0;
      int v;
      while ((v = ld_acquire(f)) == 0) {
        if (ld_relaxed(err) != 0) return;
        if (++n > spin) {
          atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
          return;
        }
        __nanosleep(32);
      }
      lv = max(lv, v);
    }
    st_release(level + I, lv + 1);
  }
}

__global__ void k_level_count(int nb, const int* __restrict__ level, int* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) atomicAdd(cnt + level[i] - 1, 1);
}

__global__ void k_level_scatter(int nb, const int* __restrict__ level, int* cursor, int* order) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) order[atomicAdd(cursor + level[i] - 1, 1)] = i;
}

int occupancy_grid(const void* fn, int threads) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0) != cudaSuccess || per < 1)
    per = 1;
  return sms * per;
}

int sync_init(SyncState& ss, int nb, Carver& ws, cudaStream_t st, long long spin = kSpinLimit,
              int withhold = -1) {
  ss.spin = spin;
  ss.withhold = withhold;
  ss.order = nullptr;
  ss.flags = ws.take<int>((size_t)nb + 1);
  int* misc = ws.take<int>(4);
  if (!ss.flags || !misc) return BILU_ERR_WORKSPACE;
  ss.ticket = misc;
  ss.err = misc + 1;
  ss.zp = misc + 2;
  BILU_TRY_CUDA(cudaMemsetAsync(ss.flags, 0, sizeof(int) * ((size_t)nb + 1), st));
  int init[4] = {0, 0, INT_MAX, 0};
  BILU_TRY_CUDA(cudaMemcpyAsync(misc, init, sizeof(init), cudaMemcpyHostToDevice, st));
  return BILU_OK;
}

int sync_finish(const SyncState& ss, int* h_zp, cudaStream_t st) {
  int h[2] = {0, 0};
  BILU_TRY_CUDA(cudaMemcpyAsync(h, ss.err, sizeof(h), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_zp) *h_zp = h[1] == INT_MAX ? -1 : h[1];
  if (h[0] != 0) return h[0];
  if (h[1] != INT_MAX) return BILU_ERR_ZERO_PIVOT;
  return BILU_OK;
}

// Ticket order by dependency level (ascending).  Rows of one level are
// independent, so consecutive tickets can run concurrently; every row's
// dependencies sit at lower levels, i.e. at earlier tickets.
int build_order(int nb, const int* row, const int* col, const int* diag, int lower, int* order,
                Carver& ws, cudaStream_t st) {
  int* level = ws.take<int>((size_t)nb + 1);
  int* cnt = ws.take<int>((size_t)nb + 1);
  int* misc = ws.take<int>(4);
  if (!level || !cnt || !misc) return BILU_ERR_WORKSPACE;
  BILU_TRY_CUDA(cudaMemsetAsync(level, 0, sizeof(int) * ((size_t)nb + 1), st));
  BILU_TRY_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * ((size_t)nb + 1), st));
  BILU_TRY_CUDA(cudaMemsetAsync(misc, 0, sizeof(int) * 4, st));
  if (nb == 0) return BILU_OK;
  const void* fn = lower ? (const void*)k_levels<true> : (const void*)k_levels<false>;
  int grid = std::min<long long>(occupancy_grid(fn, 256), (nb + 255) / 256);
  if (lower)
    k_levels<true><<<grid, 256, 0, st>>>(nb, row, col, diag, level, misc, misc + 1, kSpinLimit);
  else
    k_levels<false><<<grid, 256, 0, st>>>(nb, row, col, diag, level, misc, misc + 1, kSpinLimit);
  BILU_LAUNCH_CHECK();
  int herr = 0;
  BILU_TRY_CUDA(cudaMemcpyAsync(&herr, misc + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (herr != 0) return herr;
  k_level_count<<<ceil_div(nb, 256), 256, 0, st>>>(nb, level, cnt);
  BILU_LAUNCH_CHECK();
  BILU_TRY(scan_exclusive(cnt, cnt, nb, nullptr, ws, st));
  k_level_scatter<<<ceil_div(nb, 256), 256, 0, st>>>(nb, level, cnt, order);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

template <int BS>
int launch_bilu0(int nb, const int* row, const int* col, const int* diag, double* val,
                 SyncState ss, cudaStream_t st) {
  int grid = occupancy_grid((const void*)k_bilu0<BS>, 128);
  grid = std::min<long long>(grid, (nb + 3) / 4 + 1);
  k_bilu0<BS><<<grid, 128, 0, st>>>(nb, row, col, diag, val, ss);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

template <int BS>
int launch_sptrsv(int nb, const int* row, const int* col, const int* diag, const double* val,
                  int lower, int unit, const double* b, double* x, SyncState ss,
                  cudaStream_t st) {
  const void* fn = lower ? (unit ? (const void*)k_sptrsv<BS, true, true>
                                 : (const void*)k_sptrsv<BS, true, false>)
                         : (unit ? (const void*)k_sptrsv<BS, false, true>
                                 : (const void*)k_sptrsv<BS, false, false>);
  int grid = occupancy_grid(fn, 128);
  grid = std::min<long long>(grid, (nb + 3) / 4 + 1);
  if (lower && unit) k_sptrsv<BS, true, true><<<grid, 128, 0, st>>>(nb, row, col, diag, val, b, x, ss);
  else if (lower) k_sptrsv<BS, true, false><<<grid, 128, 0, st>>>(nb, row, col, diag, val, b, x, ss);
  else if (unit) k_sptrsv<BS, false, true><<<grid, 128, 0, st>>>(nb, row, col, diag, val, b, x, ss);
  else k_sptrsv<BS, false, false><<<grid, 128, 0, st>>>(nb, row, col, diag, val, b, x, ss);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

}  // namespace

size_t syncfree_ws(int nb) {
  // flags + order + (levels, counts, misc, scan) + sync misc + error words
  return carve_size(sizeof(int) * ((size_t)nb + 1)) * 4 + carve_size(sizeof(int) * 4) * 2 +
         carve_size(sizeof(int) * 2) + scan_ws_bytes(nb + 1);
}

// diagonal positions (validates the pattern); returns BILU_ERR_PATTERN with
// the first bad row in *h_bad
int diag_positions(int nb, const int* row, const int* col, int* diag, int* h_bad, Carver& ws,
                   cudaStream_t st) {
  int* bad = ws.take<int>(2);
  if (!bad) return BILU_ERR_WORKSPACE;
  int init = INT_MAX, hb = INT_MAX;
  BILU_TRY_CUDA(cudaMemcpyAsync(bad, &init, sizeof(int), cudaMemcpyHostToDevice, st));
  if (nb > 0) {
    k_diag_pos<<<ceil_div(nb, 256), 256, 0, st>>>(nb, row, col, diag, bad);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_bad) *h_bad = hb == INT_MAX ? -1 : hb;
  return hb == INT_MAX ? BILU_OK : BILU_ERR_PATTERN;
}

int bilu0_impl(int nb, int bs, const int* row, const int* col, const int* diag, double* val,
               int* h_zp, Carver& ws, cudaStream_t st) {
  int* order = ws.take<int>((size_t)nb + 1);
  if (!order) return BILU_ERR_WORKSPACE;
  {
    Carver w2 = ws;
    BILU_TRY(build_order(nb, row, col, diag, 1, order, w2, st));
  }
  SyncState ss;
  BILU_TRY(sync_init(ss, nb, ws, st));
  ss.order = order;
  if (nb > 0) BILU_TRY(BILU_DISPATCH_BS(bs, launch_bilu0, nb, row, col, diag, val, ss, st));
  return sync_finish(ss, h_zp, st);
}

int sptrsv_impl(int nb, int bs, const int* row, const int* col, const int* diag,
                const double* val, int lower, int unit, const double* b, double* x, Carver& ws,
                cudaStream_t st, long long spin = kSpinLimit, int withhold = -1) {
  int* order = ws.take<int>((size_t)nb + 1);
  if (!order) return BILU_ERR_WORKSPACE;
  {
    Carver w2 = ws;
    BILU_TRY(build_order(nb, row, col, diag, lower, order, w2, st));
  }
  SyncState ss;
  BILU_TRY(sync_init(ss, nb, ws, st, spin, withhold));
  ss.order = order;
  if (nb > 0)
    BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv, nb, row, col, diag, val, lower, unit, b, x, ss,
                              st));
  return sync_finish(ss, nullptr, st);
}

// Solve with a precomputed analysis (diagonal positions + level order).
// With sync=false the call returns without waiting for the GPU; the error
// word is then not read back (use for repeated solves inside a solver).
int sptrsv_ordered(int nb, int bs, const int* row, const int* col, const int* diag,
                   const int* order, const double* val, int lower, int unit, const double* b,
                   double* x, Carver& ws, cudaStream_t st, bool sync) {
  SyncState ss;
  BILU_TRY(sync_init(ss, nb, ws, st));
  ss.order = order;
  if (nb > 0)
    BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv, nb, row, col, diag, val, lower, unit, b, x, ss,
                              st));
  return sync ? sync_finish(ss, nullptr, st) : BILU_OK;
}

}  // namespace bilu

using namespace bilu;

extern "C" size_t bilu_sptrsv_analysis_bytes(int nb) {
  return 2 * carve_size(sizeof(int) * ((size_t)nb + 1));
}

extern "C" size_t bilu_sptrsv_solve_ws_bytes(int nb) { return syncfree_ws(nb); }

extern "C" int bilu_sptrsv_analysis(int nb, int bs, const int* d_row, const int* d_col, int lower,
                                    void* d_info, void* d_ws, size_t ws_bytes,
                                    bilu_stream_t stream) {
  if (nb < 0 || !d_info || (nb > 0 && (!d_row || !d_col))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver info(d_info, bilu_sptrsv_analysis_bytes(nb));
  int* diag = info.take<int>((size_t)nb + 1);
  int* order = info.take<int>((size_t)nb + 1);
  Carver ws(d_ws, ws_bytes);
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return build_order(nb, d_row, d_col, diag, lower != 0, order, ws, S(stream));
}

extern "C" int bilu_sptrsv_solve(int nb, int bs, const int* d_row, const int* d_col,
                                 const double* d_val, int lower, int unit, const void* d_info,
                                 const double* d_b, double* d_x, void* d_ws, size_t ws_bytes,
                                 bilu_stream_t stream) {
  if (nb < 0 || !d_info || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver info(const_cast<void*>(d_info), bilu_sptrsv_analysis_bytes(nb));
  const int* diag = info.take<int>((size_t)nb + 1);
  const int* order = info.take<int>((size_t)nb + 1);
  Carver ws(d_ws, ws_bytes);
  return sptrsv_ordered(nb, bs, d_row, d_col, diag, order, d_val, lower != 0, unit != 0, d_b, d_x,
                        ws, S(stream), true);
}

extern "C" size_t bilu_bsrilu0_ws_bytes(int nb) {
  return syncfree_ws(nb) + carve_size(sizeof(int) * ((size_t)nb + 1));
}

extern "C" int bilu_bsrilu0(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                            double* d_val, int* h_info, void* d_ws, size_t ws_bytes,
                            bilu_stream_t stream) {
  if (h_info) *h_info = -1;
  if (nb < 0 || nnzb < 0 || (nb > 0 && (!d_row || !d_col || !d_val))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  int bad = -1;
  int rc = diag_positions(nb, d_row, d_col, diag, &bad, ws, S(stream));
  if (rc != BILU_OK) {
    if (h_info) *h_info = bad;
    return rc;
  }
  return bilu0_impl(nb, bs, d_row, d_col, diag, d_val, h_info, ws, S(stream));
}

extern "C" size_t bilu_sptrsv_ws_bytes(int nb) {
  return syncfree_ws(nb) + carve_size(sizeof(int) * ((size_t)nb + 1));
}

extern "C" int bilu_sptrsv(int nb, int bs, const int* d_row, const int* d_col, const double* d_val,
                           int lower, const double* d_b, double* d_x, void* d_ws,
                           size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return sptrsv_impl(nb, bs, d_row, d_col, diag, d_val, lower != 0, lower != 0, d_b, d_x, ws,
                     S(stream));
}

extern "C" int bilu_sptrsv_ex(int nb, int bs, const int* d_row, const int* d_col,
                              const double* d_val, int lower, int unit, const double* d_b,
                              double* d_x, void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return sptrsv_impl(nb, bs, d_row, d_col, diag, d_val, lower != 0, unit != 0, d_b, d_x, ws,
                     S(stream));
}

// Test hook: the sync-free solve with block row `withhold_row` never
// publishing its ready flag and a short spin budget, so the rows that depend
// on it give up and the call returns BILU_ERR_TIMEOUT.  Every wait is bounded;
// the launch ends by itself and the context stays usable.
extern "C" int bilu_debug_sptrsv_withhold(int nb, int bs, const int* d_row, const int* d_col,
                                          const double* d_val, int lower, const double* d_b,
                                          double* d_x, int withhold_row, long long spin_limit,
                                          void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 1 || !d_row || !d_col || !d_val || !d_b || !d_x || spin_limit < 1 ||
      spin_limit > kSpinLimit)
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return sptrsv_impl(nb, bs, d_row, d_col, diag, d_val, lower != 0, lower != 0, d_b, d_x, ws,
                     S(stream), spin_limit, withhold_row);
}
