// Batched multi-RHS solves: many uneven BSR systems, k right-hand sides each
// (no counterpart in the reference, which solves one system with one
// right-hand side).
//
// The S systems are one block-diagonal BSR matrix (global column indices), so
// the whole preconditioner setup (BILU(0), patterns, pairs, ISAI) runs once on
// the union and every product of a step is one launch over all rows of all
// systems: the apply and the operator become BSR x dense SpMM, with the block
// row tile (rows per warp) picked by an autotuner that times the candidates
// on the batch itself.  Every (system, right-hand side) pair runs its own
// right-preconditioned FGMRES(m) with modified Gram-Schmidt: dot products are
// segmented by system (tiles never cross a system boundary and are reduced
// in tile order, so results are deterministic), Givens rotations run on the
// device, one thread per pair.  A step -- apply, SpMM, j+2 MGS sweeps,
// normalisation, Givens, and the copy of the active-pair count -- is captured
// once as a CUDA graph per (wave, j) and replayed.  The Krylov storage of the
// whole batch can exceed the GPU memory (256 systems of up to 512^2 nodes with
// 32 right-hand sides need ~1.5 TB at m = 30), so systems are packed into
// contiguous waves that fit a memory budget.
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "common.cuh"
#include "gridsync.cuh"

struct bilu_ctx;
extern "C" int bilu_ctx_create(bilu_ctx** ctx, bilu_stream_t stream);
extern "C" int bilu_ctx_destroy(bilu_ctx* ctx);
extern "C" int bilu_ctx_setup(bilu_ctx* c, int nb, int nnzb, int bs, const int* d_row,
                              const int* d_col, const double* d_val, int prec_mask,
                              double* h_times);
extern "C" int bilu_ctx_get(bilu_ctx* c, int which, const void** d_ptr, long long* h_count);

namespace bilu {
namespace {

constexpr int kBT = 256;  // threads per CTA of the row kernels

// ---------------------------------------------------------------- SpMM
// Y[(br - r0)*BS + r][c] = sum_p val[p][r][:] . X[(col[p] - r0)*BS + :][c]
// for block rows br in [r0, r1).  RPW block rows per warp; the 32/RPW lanes
// of a row own right-hand sides lane, lane + 32/RPW, ... (KL per lane).
template <int BS, class VT, class XT, class YT, int RPW>
__global__ void __launch_bounds__(kBT) k_spmm(int r0, int r1, int k, const int* __restrict__ row,
                                              const int* __restrict__ col,
                                              const VT* __restrict__ val,
                                              const XT* __restrict__ X, YT* __restrict__ Y) {
  using AccT = VT;
  constexpr int LPR = 32 / RPW;  // lanes per row
  constexpr int KL = RPW;        // right-hand sides per lane (k <= 32)
  int lane = threadIdx.x & 31;
  int sub = lane / LPR, l = lane - sub * LPR;
  long long br = r0 + ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * RPW + sub;
  if (br >= r1) return;
  AccT acc[BS][KL];
#pragma unroll
  for (int r = 0; r < BS; ++r)
#pragma unroll
    for (int q = 0; q < KL; ++q) acc[r][q] = 0;
  int s = __ldg(row + br), e = __ldg(row + br + 1);
  for (int p = s; p < e; ++p) {
    long long bc = (long long)__ldg(col + p) - r0;
    const VT* blk = val + (long long)p * BS * BS;
#pragma unroll
    for (int kk = 0; kk < BS; ++kk) {
      AccT xv[KL];
#pragma unroll
      for (int q = 0; q < KL; ++q) {
        int c = l + q * LPR;
        xv[q] = c < k ? (AccT)__ldg(X + (bc * BS + kk) * k + c) : (AccT)0;
      }
#pragma unroll
      for (int r = 0; r < BS; ++r) {
        AccT a = __ldg(blk + r * BS + kk);
#pragma unroll
        for (int q = 0; q < KL; ++q) acc[r][q] = fma(a, xv[q], acc[r][q]);
      }
    }
  }
  long long yb = (br - r0) * BS;
#pragma unroll
  for (int q = 0; q < KL; ++q) {
    int c = l + q * LPR;
    if (c < k)
#pragma unroll
      for (int r = 0; r < BS; ++r) Y[(yb + r) * k + c] = (YT)acc[r][q];
  }
}

template <int BS, class VT, class XT, class YT>
int spmm_cfg(int rpw, int r0, int r1, int k, const int* row, const int* col, const VT* val,
             const XT* X, YT* Y, cudaStream_t st) {
  if (r1 <= r0) return BILU_OK;
  long long warps = (r1 - r0 + rpw - 1) / rpw;
  unsigned grid = ceil_div(warps, kBT / 32);
  switch (rpw) {
    case 1: k_spmm<BS, VT, XT, YT, 1><<<grid, kBT, 0, st>>>(r0, r1, k, row, col, val, X, Y); break;
    case 2: k_spmm<BS, VT, XT, YT, 2><<<grid, kBT, 0, st>>>(r0, r1, k, row, col, val, X, Y); break;
    case 4: k_spmm<BS, VT, XT, YT, 4><<<grid, kBT, 0, st>>>(r0, r1, k, row, col, val, X, Y); break;
    default: return BILU_ERR_ARG;
  }
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// ---------------------------------------------------------------- sweeps
// Tile t covers scalar rows [trow[t], trow[t+1]) of system tsys[t] (wave
// local).  One MGS sweep: w -= h_prev[s][c] * vp; partial[t][c] = vn . w
// (or w . w).  Rows are spread over the warps of the CTA, lane = rhs.
__global__ void __launch_bounds__(kBT) k_sweep(int ntiles, int k, const int* __restrict__ trow,
                                               const int* __restrict__ tsys,
                                               const double* __restrict__ vp,
                                               const double* __restrict__ hp,
                                               const double* __restrict__ vn, double* w,
                                               double* __restrict__ partial) {
  __shared__ double red[kBT / 32][32];
  int t = blockIdx.x;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int s = tsys[t];
  double h = (vp && lane < k) ? -__ldg(hp + (long long)s * k + lane) : 0.0;
  double acc = 0.0;
  if (lane < k) {
    for (long long rr = trow[t] + warp; rr < trow[t + 1]; rr += kBT / 32) {
      long long i = rr * k + lane;
      double we = w[i];
      if (vp) {
        we = fma(h, __ldcs(vp + i), we);
        w[i] = we;
      }
      double o = vn ? __ldcs(vn + i) : we;
      acc = fma(o, we, acc);
    }
  }
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0) {
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < kBT / 32; ++q) v += red[q][lane];
    if (lane < k) partial[(long long)t * k + lane] = v;
  }
}

// out[s][c] = sum over the tiles of system s of partial[t][c].  One CTA per
// system, lane = right-hand side: warp w sums the system's tiles w, w + W,
// w + 2W, ... in that order (four loads in flight), then the W warp sums are
// added in warp order.  The order depends only on a tile's index inside its
// system, so the result does not depend on how systems are grouped into
// waves.  (A thread per (system, rhs) walking thousands of tiles took
// ~230 us per call on a 2M-row wave, a quarter of the solve.)
constexpr int kSegWarps = 16;

__global__ void __launch_bounds__(32 * kSegWarps) k_segsum(int S, int k,
                                                            const int* __restrict__ sys_tiles,
                                                            const double* __restrict__ partial,
                                                            double* __restrict__ out) {
  __shared__ double red[kSegWarps][32];
  const int s = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v = 0.0;
  if (s < S && lane < k) {
    const int t1 = sys_tiles[s + 1];
    int t = sys_tiles[s] + warp;
    for (; t + 3 * kSegWarps < t1; t += 4 * kSegWarps) {
      const double a = partial[(long long)t * k + lane];
      const double b = partial[(long long)(t + kSegWarps) * k + lane];
      const double c = partial[(long long)(t + 2 * kSegWarps) * k + lane];
      const double d = partial[(long long)(t + 3 * kSegWarps) * k + lane];
      v += a;
      v += b;
      v += c;
      v += d;
    }
    for (; t < t1; t += kSegWarps) v += partial[(long long)t * k + lane];
  }
  red[warp][lane] = v;
  __syncthreads();
  if (warp == 0 && s < S && lane < k) {
    double r = 0.0;
#pragma unroll
    for (int w = 0; w < kSegWarps; ++w) r += red[w][lane];
    out[(long long)s * k + lane] = r;
  }
}

// y = x / sqrt(nrm2[s][c]) (0 when the norm is 0), with an FP32 copy
__global__ void k_scale_pairs(int ntiles, int k, const int* __restrict__ trow,
                              const int* __restrict__ tsys, const double* __restrict__ x,
                              const double* __restrict__ nrm2, double* __restrict__ y,
                              float* __restrict__ y32) {
  int t = blockIdx.x;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane >= k) return;
  int s = tsys[t];
  double n2 = nrm2[(long long)s * k + lane];
  double a = n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0;
  for (long long rr = trow[t] + warp; rr < trow[t + 1]; rr += kBT / 32) {
    long long i = rr * k + lane;
    double v = x[i] * a;
    y[i] = v;
    if (y32) y32[i] = __double2float_rn(v);
  }
}

// r = b - ax; partial[t][c] = r.r over the tile
__global__ void k_residual_pairs(int ntiles, int k, const int* __restrict__ trow,
                                 const double* __restrict__ b, const double* __restrict__ ax,
                                 double* __restrict__ r, double* __restrict__ partial) {
  __shared__ double red[kBT / 32][32];
  int t = blockIdx.x;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc = 0.0;
  if (lane < k)
    for (long long rr = trow[t] + warp; rr < trow[t + 1]; rr += kBT / 32) {
      long long i = rr * k + lane;
      double v = b[i] - ax[i];
      r[i] = v;
      acc = fma(v, v, acc);
    }
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0) {
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < kBT / 32; ++q) v += red[q][lane];
    if (lane < k) partial[(long long)t * k + lane] = v;
  }
}

// x[i] += sum_{q <= jmax} y[pair][q] * Z_q[i]
__global__ void k_xupdate(int ntiles, int k, int m, int jmax, const int* __restrict__ trow,
                          const int* __restrict__ tsys, const double* __restrict__ Z,
                          long long ldz, const double* __restrict__ y, double* __restrict__ x) {
  int t = blockIdx.x;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane >= k) return;
  int s = tsys[t];
  const double* yp = y + ((long long)s * k + lane) * m;
  for (long long rr = trow[t] + warp; rr < trow[t + 1]; rr += kBT / 32) {
    long long i = rr * k + lane;
    double v = x[i];
    for (int q = 0; q <= jmax; ++q) v = fma(yp[q], Z[q * ldz + i], v);
    x[i] = v;
  }
}

// ---------------------------------------------------------------- pair state
// Per pair (s, c): H[(m+1) x m], cs[m], sn[m], g[m+1], y[m]; status:
// 0 = running in this cycle, 1 = converged in this cycle (jlast fixed),
// 2 = done (true residual below tol).
struct PairState {
  double *H, *cs, *sn, *g, *y, *bnorm, *beta;
  int *status, *jlast, *iters;
  int* active;  // running pairs after the last Givens step
};

__global__ void k_cycle_init(int P, int m, PairState ps, const double* __restrict__ rr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  double beta = sqrt(rr[i]);
  ps.beta[i] = beta;
  for (int q = 0; q <= m; ++q) ps.g[(long long)i * (m + 1) + q] = 0.0;
  ps.g[(long long)i * (m + 1)] = beta;
  if (ps.status[i] != 2) {
    ps.status[i] = 0;
    ps.jlast[i] = -1;
  }
}

// Givens step j of every running pair: hcol[q][pair] (q <= j) from the
// sweeps, hn2[pair] = ||w||^2.
__device__ __forceinline__ void givens_pair(int i, int m, int j, double tol, PairState ps,
                                            const double* hcol, const double* hn2, int P) {
  if (ps.status[i] != 0) return;
  double* H = ps.H + (long long)i * (m + 1) * m;
  double* cs = ps.cs + (long long)i * m;
  double* sn = ps.sn + (long long)i * m;
  double* g = ps.g + (long long)i * (m + 1);
  for (int q = 0; q <= j; ++q) H[q * m + j] = __ldcg(hcol + (long long)q * P + i);
  double hn = sqrt(__ldcg(hn2 + i));
  H[(j + 1) * m + j] = hn;
  for (int q = 0; q < j; ++q) {
    double a = H[q * m + j], b = H[(q + 1) * m + j];
    H[q * m + j] = cs[q] * a + sn[q] * b;
    H[(q + 1) * m + j] = -sn[q] * a + cs[q] * b;
  }
  double a = H[j * m + j], b = H[(j + 1) * m + j];
  double den = sqrt(a * a + b * b);
  cs[j] = den != 0.0 ? a / den : 1.0;
  sn[j] = den != 0.0 ? b / den : 0.0;
  H[j * m + j] = cs[j] * a + sn[j] * b;
  H[(j + 1) * m + j] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  ps.iters[i] += 1;
  ps.jlast[i] = j;
  double res = fabs(g[j + 1]) / ps.bnorm[i];
  if (res <= tol || hn == 0.0 || j == m - 1) ps.status[i] = 1;
  else atomicAdd(ps.active, 1);
}

__global__ void k_givens(int P, int m, int j, double tol, PairState ps,
                         const double* __restrict__ hcol, const double* __restrict__ hn2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  givens_pair(i, m, j, tol, ps, hcol, hn2, P);
}

// Back substitution per pair (y = 0 for done pairs)
__global__ void k_trisolve(int P, int m, PairState ps) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  double* y = ps.y + (long long)i * m;
  for (int q = 0; q < m; ++q) y[q] = 0.0;
  if (ps.status[i] == 2) return;
  int jl = ps.jlast[i];
  const double* H = ps.H + (long long)i * (m + 1) * m;
  const double* g = ps.g + (long long)i * (m + 1);
  for (int q = jl; q >= 0; --q) {
    double v = g[q];
    for (int r = q + 1; r <= jl; ++r) v -= H[q * m + r] * y[r];
    y[q] = v / H[q * m + q];
  }
}

// After the true residual: done when rel. residual <= tol
__global__ void k_check(int P, double tol, PairState ps, const double* __restrict__ rr,
                        double* __restrict__ relres, int* notdone) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  double r = sqrt(rr[i]) / ps.bnorm[i];
  relres[i] = r;
  if (ps.status[i] == 2) return;
  if (r <= tol || rr[i] == 0.0) ps.status[i] = 2;
  else atomicAdd(notdone, 1);
}

// every block (I, J) must stay inside the system of row I (block-diagonal)
__global__ void k_check_blockdiag(int nb, int S, const int* __restrict__ row,
                                  const int* __restrict__ col, const int* __restrict__ sys,
                                  int* bad) {
  int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nb) return;
  int lo = 0, hi = S - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sys[mid] <= I) lo = mid; else hi = mid - 1;
  }
  int a = sys[lo], b = sys[lo + 1];
  for (int p = row[I]; p < row[I + 1]; ++p)
    if (col[p] < a || col[p] >= b) {
      atomicMin(bad, I);
      return;
    }
}

__global__ void k_bnorm(int P, PairState ps, const double* __restrict__ bb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  double b = sqrt(bb[i]);
  ps.bnorm[i] = b > 0.0 ? b : 1.0;
  ps.status[i] = 0;
  ps.iters[i] = 0;
}


// ---------------------------------------------------------------- one launch per step
// The whole Arnoldi step of every pair of a wave in one cooperative launch
// (k_batch_step): the FP32 apply (M_L, then M_U into Z_j), the operator
// SpMM, the j+2 modified Gram-Schmidt sweeps with their per-system sums,
// the normalisation of V_{j+1} and the Givens step of every pair, with a
// counting grid barrier between dependent phases instead of a kernel
// boundary.  Each phase walks its own work list: virtual warps of block
// rows for the SpMMs (the rows-per-warp tile chosen by the autotuner),
// tiles of scalar rows for the sweeps and the normalisation (two tiles at
// a time, one per half of the 16-warp CTA, each reduced over its 8 warps
// exactly as k_sweep does), systems for the segmented sums (16 warps each,
// as k_segsum), pairs for Givens.  The arithmetic of every element and
// every sum is that of the per-phase kernels, so both schedules give the
// same bits; data written earlier in the launch is read through the L2.
constexpr int kStepT = 32 * kSegWarps;  // threads of a k_batch_step CTA (16 warps)
static_assert(kStepT == 2 * kBT, "a step CTA holds two sweep tiles of kBT threads");

struct BatchStepArgs {
  int r0, r1, k, j, m, P, nt, Sw;
  double tol;
  const int *Lrow, *Lcol, *Urow, *Ucol, *Arow, *Acol;
  const float *L32, *U32;
  const double* Aval;
  float *v32, *t32;
  double *V, *Zj, *w, *hcol, *hn2, *part;
  long long vec;
  const int *trow, *tsys, *stile;
  PairState ps;
  GridSync gs;
};

// k_spmm's rows for virtual warp vw, X read through the L2 (an earlier
// phase of the same launch wrote it)
template <int BS, class VT, class XT, class YT, int RPW>
__device__ __forceinline__ void spmm_vwarp(long long vw, int lane, int r0, int r1, int k,
                                           const int* __restrict__ row,
                                           const int* __restrict__ col,
                                           const VT* __restrict__ val, const XT* X, YT* Y) {
  using AccT = VT;
  constexpr int LPR = 32 / RPW;
  constexpr int KL = RPW;
  int sub = lane / LPR, l = lane - sub * LPR;
  long long br = r0 + vw * RPW + sub;
  if (br >= r1) return;
  AccT acc[BS][KL];
#pragma unroll
  for (int r = 0; r < BS; ++r)
#pragma unroll
    for (int q = 0; q < KL; ++q) acc[r][q] = 0;
  int s = __ldg(row + br), e = __ldg(row + br + 1);
  for (int p = s; p < e; ++p) {
    long long bc = (long long)__ldg(col + p) - r0;
    const VT* blk = val + (long long)p * BS * BS;
#pragma unroll
    for (int kk = 0; kk < BS; ++kk) {
      AccT xv[KL];
#pragma unroll
      for (int q = 0; q < KL; ++q) {
        int c = l + q * LPR;
        xv[q] = c < k ? (AccT)__ldcg(X + (bc * BS + kk) * k + c) : (AccT)0;
      }
#pragma unroll
      for (int r = 0; r < BS; ++r) {
        AccT a = __ldg(blk + r * BS + kk);
#pragma unroll
        for (int q = 0; q < KL; ++q) acc[r][q] = fma(a, xv[q], acc[r][q]);
      }
    }
  }
  long long yb = (br - r0) * BS;
#pragma unroll
  for (int q = 0; q < KL; ++q) {
    int c = l + q * LPR;
    if (c < k)
#pragma unroll
      for (int r = 0; r < BS; ++r) Y[(yb + r) * k + c] = (YT)acc[r][q];
  }
}

template <int BS, class VT, class XT, class YT, int RPW>
__device__ __forceinline__ void spmm_phase(int r0, int r1, int k, const int* row, const int* col,
                                           const VT* val, const XT* X, YT* Y) {
  const long long nvw = ((long long)(r1 - r0) + RPW - 1) / RPW;
  const long long total = (long long)gridDim.x * (kStepT / 32);
  const int lane = threadIdx.x & 31;
  for (long long vw = (long long)blockIdx.x * (kStepT / 32) + (threadIdx.x >> 5); vw < nvw;
       vw += total)
    spmm_vwarp<BS, VT, XT, YT, RPW>(vw, lane, r0, r1, k, row, col, val, X, Y);
}

template <int BS, int RPWM, int RPWA>
__global__ void __launch_bounds__(kStepT, BS <= 5 ? 2 : 1) k_batch_step(BatchStepArgs a) {
  __shared__ double red[kStepT / 32][32];
  unsigned passed = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int half = warp >> 3, hw = warp & 7;  // sweep-tile half of the CTA, warp inside it
  const int k = a.k, P = a.P, G = (int)gridDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.ps.active = 0;
  // FP32 apply: t32 = M_L v32, Z_j = M_U t32 (FP64), then w = A Z_j
  spmm_phase<BS, float, float, float, RPWM>(a.r0, a.r1, k, a.Lrow, a.Lcol, a.L32, a.v32, a.t32);
  if (!grid_sync_count(a.gs, passed)) return;
  spmm_phase<BS, float, float, double, RPWM>(a.r0, a.r1, k, a.Urow, a.Ucol, a.U32, a.t32, a.Zj);
  if (!grid_sync_count(a.gs, passed)) return;
  spmm_phase<BS, double, double, double, RPWA>(a.r0, a.r1, k, a.Arow, a.Acol, a.Aval, a.Zj,
                                               a.w);
  if (!grid_sync_count(a.gs, passed)) return;
  for (int i = 0; i <= a.j + 1; ++i) {
    const double* vp = i > 0 ? a.V + a.vec * (i - 1) : nullptr;
    const double* hp = i > 0 ? a.hcol + (long long)(i - 1) * P : nullptr;
    const double* vn = i <= a.j ? a.V + a.vec * i : nullptr;
    double* out = i <= a.j ? a.hcol + (long long)i * P : a.hn2;
    // sweep: tile partials (k_sweep's arithmetic per tile)
    for (int t0 = 2 * blockIdx.x; t0 < a.nt; t0 += 2 * G) {
      const int t = t0 + half;
      double acc = 0.0;
      if (t < a.nt && lane < k) {
        const int sy = a.tsys[t];
        const double h = vp ? -__ldcg(hp + (long long)sy * k + lane) : 0.0;
        // the thread's rows in k_sweep's order, four rows' loads issued
        // before their arithmetic
        const long long re = a.trow[t + 1];
        for (long long rr0 = a.trow[t] + hw; rr0 < re; rr0 += 4 * (kBT / 32)) {
          double we[4], pv[4], ov[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const long long rr = rr0 + u * (kBT / 32);
            const long long q = rr * k + lane;
            const bool ok = rr < re;
            we[u] = ok ? __ldcg(a.w + q) : 0.0;
            pv[u] = (ok && vp) ? __ldcs(vp + q) : 0.0;
            ov[u] = (ok && vn) ? __ldcs(vn + q) : 0.0;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const long long rr = rr0 + u * (kBT / 32);
            if (rr >= re) break;
            const long long q = rr * k + lane;
            if (vp) {
              we[u] = fma(h, pv[u], we[u]);
              a.w[q] = we[u];
            }
            const double o = vn ? ov[u] : we[u];
            acc = fma(o, we[u], acc);
          }
        }
      }
      red[warp][lane] = acc;
      __syncthreads();
      if (hw == 0 && t < a.nt) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < kBT / 32; ++q) v += red[half * 8 + q][lane];
        if (lane < k) a.part[(long long)t * k + lane] = v;
      }
      __syncthreads();
    }
    if (!grid_sync_count(a.gs, passed)) return;
    // per-system sums of the tile partials (k_segsum's order)
    for (int sy = blockIdx.x; sy < a.Sw; sy += G) {
      double v = 0.0;
      if (lane < k) {
        const int t1 = a.stile[sy + 1];
        int t = a.stile[sy] + warp;
        for (; t + 3 * kSegWarps < t1; t += 4 * kSegWarps) {
          const double p0 = __ldcg(a.part + (long long)t * k + lane);
          const double p1 = __ldcg(a.part + (long long)(t + kSegWarps) * k + lane);
          const double p2 = __ldcg(a.part + (long long)(t + 2 * kSegWarps) * k + lane);
          const double p3 = __ldcg(a.part + (long long)(t + 3 * kSegWarps) * k + lane);
          v += p0;
          v += p1;
          v += p2;
          v += p3;
        }
        for (; t < t1; t += kSegWarps) v += __ldcg(a.part + (long long)t * k + lane);
      }
      red[warp][lane] = v;
      __syncthreads();
      if (warp == 0 && lane < k) {
        double r = 0.0;
#pragma unroll
        for (int q = 0; q < kSegWarps; ++q) r += red[q][lane];
        out[(long long)sy * k + lane] = r;
      }
      __syncthreads();
    }
    if (!grid_sync_count(a.gs, passed)) return;
  }
  // V_{j+1} = w / ||w|| (k_scale_pairs) and the Givens step (k_givens)
  double* vnext = a.V + a.vec * (a.j + 1);
  for (int t0 = 2 * blockIdx.x; t0 < a.nt; t0 += 2 * G) {
    const int t = t0 + half;
    if (t >= a.nt || lane >= k) continue;
    const int sy = a.tsys[t];
    const double n2 = __ldcg(a.hn2 + (long long)sy * k + lane);
    const double s = n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0;
    for (long long rr = a.trow[t] + hw; rr < a.trow[t + 1]; rr += kBT / 32) {
      long long q = rr * k + lane;
      double v = __ldcg(a.w + q) * s;
      vnext[q] = v;
      a.v32[q] = __double2float_rn(v);
    }
  }
  for (int pi = blockIdx.x * kStepT + threadIdx.x; pi < P; pi += G * kStepT)
    givens_pair(pi, a.m, a.j, a.tol, a.ps, a.hcol, a.hn2, P);
  grid_exit_count(a.gs);
}

}  // namespace
}  // namespace bilu

using namespace bilu;

struct bilu_batch {
  cudaStream_t st = nullptr;    // caller's stream (setup, ordering of B and X)
  cudaStream_t work = nullptr;  // private non-blocking stream the solve captures on
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  bilu_ctx* ctx = nullptr;
  int S = 0, bs = 0, nb = 0, nnzb = 0;
  std::vector<int> sys;  // S+1 block-row offsets
  const int *Arow = nullptr, *Acol = nullptr, *Lrow = nullptr, *Lcol = nullptr,
            *Urow = nullptr, *Ucol = nullptr;
  const double* Aval = nullptr;
  const float *L32 = nullptr, *U32 = nullptr;
  // rows per warp of the SpMMs (tuned: they do not change any sum's order);
  // scalar rows per tile of the sweeps (fixed: the tiles partition every
  // dot product, so the tile size is part of the arithmetic)
  int rpw_A = 1, rpw_M = 1, tile_rows = 128;
  bool tuned = false;
  // 1: every Arnoldi step is one cooperative launch (k_batch_step); 0: a
  // graph of per-phase kernels.  Both give the same bits.
  int persistent = 1;
  double tune_ms[2][3] = {};
};

namespace {

template <class F>
float time_ms(cudaStream_t st, F f, int reps = 3) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  f();
  cudaEventRecord(a, st);
  for (int i = 0; i < reps; ++i) f();
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

int spmm_A(bilu_batch* B, int rpw, int r0, int r1, int k, const double* X, double* Y) {
  return BILU_DISPATCH_BS(B->bs, spmm_cfg, rpw, r0, r1, k, B->Arow, B->Acol, B->Aval, X, Y,
                          B->work);
}
int spmm_L32(bilu_batch* B, int rpw, int r0, int r1, int k, const float* X, float* Y) {
  return BILU_DISPATCH_BS(B->bs, spmm_cfg, rpw, r0, r1, k, B->Lrow, B->Lcol, B->L32, X, Y, B->work);
}
int spmm_U32(bilu_batch* B, int rpw, int r0, int r1, int k, const float* X, double* Y) {
  return BILU_DISPATCH_BS(B->bs, spmm_cfg, rpw, r0, r1, k, B->Urow, B->Ucol, B->U32, X, Y, B->work);
}

// Autotuner: time every rows-per-warp candidate of the operator SpMM and of
// the FP32 apply on the first wave's rows (3 reps each), keep the fastest.
int autotune(bilu_batch* B, int r0, int r1, int k, double* X, double* Y, float* X32, float* Y32) {
  const int cand[3] = {1, 2, 4};
  float best_a = 1e30f, best_m = 1e30f;
  for (int ci = 0; ci < 3; ++ci) {
    int rpw = cand[ci];
    float ta = time_ms(B->work, [&] { spmm_A(B, rpw, r0, r1, k, X, Y); });
    float tm = time_ms(B->work, [&] {
      spmm_L32(B, rpw, r0, r1, k, X32, Y32);
      spmm_U32(B, rpw, r0, r1, k, Y32, Y);
    });
    BILU_TRY_CUDA(cudaGetLastError());
    B->tune_ms[0][ci] = ta;
    B->tune_ms[1][ci] = tm;
    if (ta < best_a) { best_a = ta; B->rpw_A = rpw; }
    if (tm < best_m) { best_m = tm; B->rpw_M = rpw; }
  }
  B->tuned = true;
  return BILU_OK;
}

template <int BS, int RM, int RA>
int launch_batch_step_t(const BatchStepArgs& a, cudaStream_t st) {
  static int grid = 0;
  const void* fn = (const void*)k_batch_step<BS, RM, RA>;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    BILU_TRY_CUDA(cudaGetDevice(&dev));
    BILU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BILU_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kStepT, 0));
    if (per < 1) return BILU_ERR_UNSUPPORTED;
    grid = per * sms;
  }
  BatchStepArgs arg = a;
  void* args[] = {&arg};
  BILU_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kStepT), args, 0, st));
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

template <int BS, int RM>
int launch_batch_step_a(int ra, const BatchStepArgs& a, cudaStream_t st) {
  switch (ra) {
    case 1: return launch_batch_step_t<BS, RM, 1>(a, st);
    case 2: return launch_batch_step_t<BS, RM, 2>(a, st);
    case 4: return launch_batch_step_t<BS, RM, 4>(a, st);
    default: return BILU_ERR_ARG;
  }
}

template <int BS>
int launch_batch_step_bs(int rm, int ra, const BatchStepArgs& a, cudaStream_t st) {
  switch (rm) {
    case 1: return launch_batch_step_a<BS, 1>(ra, a, st);
    case 2: return launch_batch_step_a<BS, 2>(ra, a, st);
    case 4: return launch_batch_step_a<BS, 4>(ra, a, st);
    default: return BILU_ERR_ARG;
  }
}

int launch_batch_step(int bs, int rm, int ra, const BatchStepArgs& a, cudaStream_t st) {
  return BILU_DISPATCH_BS(bs, launch_batch_step_bs, rm, ra, a, st);
}

}  // namespace

extern "C" int bilu_batch_set_schedule(bilu_batch* B, int persistent) {
  if (!B || persistent < 0 || persistent > 1) return BILU_ERR_ARG;
  B->persistent = persistent;
  return BILU_OK;
}

extern "C" int bilu_batch_create(bilu_batch** b, bilu_stream_t stream) {
  if (!b) return BILU_ERR_ARG;
  bilu_batch* B = new (std::nothrow) bilu_batch();
  if (!B) return BILU_ERR_ARG;
  B->st = S(stream);
  // graph capture is not allowed on the legacy default stream, so the solve
  // runs on a stream of its own, ordered after / before the caller's stream
  cudaError_t e = cudaStreamCreateWithFlags(&B->work, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_out, cudaEventDisableTiming);
  int rc = e == cudaSuccess ? bilu_ctx_create(&B->ctx, stream) : cuda_status(e);
  if (rc != BILU_OK) {
    bilu_batch_destroy(B);
    return rc;
  }
  *b = B;
  return BILU_OK;
}

extern "C" int bilu_batch_destroy(bilu_batch* b) {
  if (!b) return BILU_OK;
  if (b->ctx) bilu_ctx_destroy(b->ctx);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev_out) cudaEventDestroy(b->ev_out);
  if (b->work) cudaStreamDestroy(b->work);
  delete b;
  return BILU_OK;
}

extern "C" int bilu_batch_setup(bilu_batch* B, int S_, const int* h_sys_ptr, int nnzb, int bs,
                                const int* d_row, const int* d_col, const double* d_val,
                                double* h_times) {
  if (!B || S_ < 1 || !h_sys_ptr || h_sys_ptr[0] != 0) return BILU_ERR_ARG;
  for (int s = 0; s < S_; ++s)
    if (h_sys_ptr[s + 1] <= h_sys_ptr[s]) return BILU_ERR_ARG;
  int nb = h_sys_ptr[S_];
  {
    int* d = nullptr;
    BILU_TRY_CUDA(cudaMalloc(&d, sizeof(int) * (S_ + 2)));
    int big = 0x7fffffff, hb = 0;
    cudaMemcpy(d, h_sys_ptr, sizeof(int) * (S_ + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(d + S_ + 1, &big, sizeof(int), cudaMemcpyHostToDevice);
    k_check_blockdiag<<<ceil_div(nb, 256), 256, 0, B->st>>>(nb, S_, d_row, d_col, d, d + S_ + 1);
    cudaError_t e = cudaMemcpyAsync(&hb, d + S_ + 1, sizeof(int), cudaMemcpyDeviceToHost, B->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->st);
    cudaFree(d);
    BILU_TRY_CUDA(e);
    if (hb != big) return BILU_ERR_PATTERN;
  }
  BILU_TRY(bilu_ctx_setup(B->ctx, nb, nnzb, bs, d_row, d_col, d_val, 1 << BILU_FP32, h_times));
  B->S = S_;
  B->bs = bs;
  B->nb = nb;
  B->nnzb = nnzb;
  B->sys.assign(h_sys_ptr, h_sys_ptr + S_ + 1);
  const void* p;
  long long cnt;
  // the handle copies A; LU at 0, M_L 1..3, M_U 4..6, FP32 values 7, 8
  BILU_TRY(bilu_ctx_get(B->ctx, 1, &p, &cnt)); B->Lrow = (const int*)p;
  BILU_TRY(bilu_ctx_get(B->ctx, 2, &p, &cnt)); B->Lcol = (const int*)p;
  BILU_TRY(bilu_ctx_get(B->ctx, 4, &p, &cnt)); B->Urow = (const int*)p;
  BILU_TRY(bilu_ctx_get(B->ctx, 5, &p, &cnt)); B->Ucol = (const int*)p;
  BILU_TRY(bilu_ctx_get(B->ctx, 7, &p, &cnt)); B->L32 = (const float*)p;
  BILU_TRY(bilu_ctx_get(B->ctx, 8, &p, &cnt)); B->U32 = (const float*)p;
  B->Arow = d_row;
  B->Acol = d_col;
  B->Aval = d_val;
  B->tuned = false;
  return BILU_OK;
}

extern "C" int bilu_batch_tuning(bilu_batch* B, int* h_cfg, double* h_ms) {
  if (!B) return BILU_ERR_ARG;
  if (h_cfg) {
    h_cfg[0] = B->rpw_A;
    h_cfg[1] = B->rpw_M;
    h_cfg[2] = B->tile_rows;
  }
  if (h_ms)
    for (int i = 0; i < 6; ++i) h_ms[i] = B->tune_ms[i / 3][i % 3];
  return BILU_OK;
}

namespace {

struct WaveBufs {
  double *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr, *part = nullptr, *hcol = nullptr,
         *hn2 = nullptr, *rr = nullptr, *relres = nullptr;
  float *v32 = nullptr, *t32 = nullptr;
  int *trow = nullptr, *tsys = nullptr, *stile = nullptr, *counters = nullptr;
  int* hpin = nullptr;
  PairState ps{};
  std::vector<void*> owned;
  template <class T>
  int get(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
    if (e != cudaSuccess) return cuda_status(e);
    owned.push_back(*p);
    return BILU_OK;
  }
  ~WaveBufs() {
    for (void* p : owned) cudaFree(p);
    if (hpin) cudaFreeHost(hpin);
  }
};

}  // namespace

namespace {

// Tiles of tile_rows scalar rows over systems [s0, s1), never across a system.
void build_tiles(const bilu_batch* B, int s0, int s1, int tile_rows, std::vector<int>& trow,
                 std::vector<int>& tsys, std::vector<int>& stile) {
  const int r0 = B->sys[s0], bs = B->bs;
  trow.clear();
  tsys.clear();
  stile.assign(s1 - s0 + 1, 0);
  for (int s = s0; s < s1; ++s) {
    long long a = (long long)(B->sys[s] - r0) * bs, e = (long long)(B->sys[s + 1] - r0) * bs;
    for (long long x = a; x < e; x += tile_rows) {
      trow.push_back((int)x);
      tsys.push_back(s - s0);
    }
    stile[s - s0 + 1] = (int)tsys.size();
  }
  trow.push_back((int)((long long)(B->sys[s1] - r0) * bs));
}

}  // namespace

// Solves every system for k right-hand sides (B, X: [n, k] row-major FP64,
// n = nb*bs).  h_iters / h_relres: [S*k] per pair (system-major).  h_stats
// (optional, 4): waves, graph launches, total pair-steps, solve ms.
extern "C" int bilu_batch_solve(bilu_batch* Bt, int k, const double* d_B, double* d_X,
                                int restart, double tol, int maxit, long long mem_budget,
                                int* h_iters, double* h_relres, double* h_stats) {
  if (!Bt || k < 1 || k > 32 || restart < 1 || restart > 30 || maxit < 0 || !d_B || !d_X)
    return BILU_ERR_ARG;
  if (Bt->S == 0) return BILU_ERR_ARG;
  cudaStream_t st = Bt->work;
  BILU_TRY_CUDA(cudaEventRecord(Bt->ev_in, Bt->st));
  BILU_TRY_CUDA(cudaStreamWaitEvent(st, Bt->ev_in, 0));
  const int m = restart, bs = Bt->bs;
  // bytes per scalar row of the wave: V (m+1) + Z (m) + w + r (FP64) and two
  // FP32 vectors, all k wide
  double per_row = (double)k * (8.0 * (2 * m + 3) + 8.0);
  long long budget = mem_budget > 0 ? mem_budget : (long long)64 << 30;
  long long max_rows = std::max<long long>((long long)(budget / per_row), 1);
  // contiguous waves of systems
  std::vector<std::pair<int, int>> waves;
  for (int s = 0; s < Bt->S;) {
    int e = s + 1;
    long long rows = (long long)(Bt->sys[e] - Bt->sys[s]) * bs;
    while (e < Bt->S && rows + (long long)(Bt->sys[e + 1] - Bt->sys[e]) * bs <= max_rows) {
      rows += (long long)(Bt->sys[e + 1] - Bt->sys[e]) * bs;
      ++e;
    }
    waves.push_back({s, e});
    s = e;
  }
  // largest wave sizes
  long long wrows_max = 0, ntile_max = 0;
  int ws_max = 0;
  for (auto& w : waves) {
    long long rows = (long long)(Bt->sys[w.second] - Bt->sys[w.first]) * bs;
    wrows_max = std::max(wrows_max, rows);
    ws_max = std::max(ws_max, w.second - w.first);
    long long nt = 0;
    for (int s = w.first; s < w.second; ++s)
      nt += ((long long)(Bt->sys[s + 1] - Bt->sys[s]) * bs + Bt->tile_rows - 1) / Bt->tile_rows;
    ntile_max = std::max(ntile_max, nt);
  }
  WaveBufs W;
  size_t vec = (size_t)wrows_max * k;
  int P = ws_max * k;
  BILU_TRY(W.get(&W.V, vec * (m + 1)));
  BILU_TRY(W.get(&W.Z, vec * m));
  BILU_TRY(W.get(&W.w, vec));
  BILU_TRY(W.get(&W.r, vec));
  BILU_TRY(W.get(&W.v32, vec));
  BILU_TRY(W.get(&W.t32, vec));
  BILU_TRY(W.get(&W.part, (size_t)ntile_max * k));
  BILU_TRY(W.get(&W.hcol, (size_t)(m + 1) * P));
  BILU_TRY(W.get(&W.hn2, (size_t)P));
  BILU_TRY(W.get(&W.rr, (size_t)P));
  BILU_TRY(W.get(&W.relres, (size_t)P));
  BILU_TRY(W.get(&W.trow, (size_t)ntile_max + 1));
  BILU_TRY(W.get(&W.tsys, (size_t)ntile_max));
  BILU_TRY(W.get(&W.stile, (size_t)ws_max + 1));
  BILU_TRY(W.get(&W.counters, 4));
  unsigned* step_words = nullptr;  // count, exit count, error word of k_batch_step
  BILU_TRY(W.get(&step_words, 4));
  BILU_TRY_CUDA(cudaMemsetAsync(step_words, 0, sizeof(unsigned) * 4, st));
  BILU_TRY(W.get(&W.ps.H, (size_t)P * (m + 1) * m));
  BILU_TRY(W.get(&W.ps.cs, (size_t)P * m));
  BILU_TRY(W.get(&W.ps.sn, (size_t)P * m));
  BILU_TRY(W.get(&W.ps.g, (size_t)P * (m + 1)));
  BILU_TRY(W.get(&W.ps.y, (size_t)P * m));
  BILU_TRY(W.get(&W.ps.bnorm, (size_t)P));
  BILU_TRY(W.get(&W.ps.beta, (size_t)P));
  BILU_TRY(W.get(&W.ps.status, (size_t)P));
  BILU_TRY(W.get(&W.ps.jlast, (size_t)P));
  BILU_TRY(W.get(&W.ps.iters, (size_t)P));
  W.ps.active = W.counters;
  BILU_TRY_CUDA(cudaMallocHost(&W.hpin, sizeof(int) * 4));
  long long graph_launches = 0, pair_steps = 0;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, st);
  for (auto& wv : waves) {
    int s0 = wv.first, s1 = wv.second, Sw = s1 - s0, Pw = Sw * k;
    int r0 = Bt->sys[s0], r1 = Bt->sys[s1];
    long long n_w = (long long)(r1 - r0) * bs;
    std::vector<int> trow, tsys, stile;
    build_tiles(Bt, s0, s1, Bt->tile_rows, trow, tsys, stile);
    int nt = (int)tsys.size();
    BILU_TRY_CUDA(cudaMemcpyAsync(W.trow, trow.data(), sizeof(int) * (nt + 1), cudaMemcpyHostToDevice, st));
    BILU_TRY_CUDA(cudaMemcpyAsync(W.tsys, tsys.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, st));
    BILU_TRY_CUDA(cudaMemcpyAsync(W.stile, stile.data(), sizeof(int) * (Sw + 1), cudaMemcpyHostToDevice, st));
    const double* Bw = d_B + (size_t)(r0)*bs * k;
    double* Xw = d_X + (size_t)(r0)*bs * k;
    unsigned gp = ceil_div(Pw, 128);
    if (!Bt->tuned) BILU_TRY(autotune(Bt, r0, r1, k, W.r, W.w, W.v32, W.t32));
    // x = 0, r = b, ||b||
    BILU_TRY_CUDA(cudaMemsetAsync(Xw, 0, sizeof(double) * n_w * k, st));
    BILU_TRY_CUDA(cudaMemsetAsync(W.w, 0, sizeof(double) * n_w * k, st));
    k_residual_pairs<<<nt, kBT, 0, st>>>(nt, k, W.trow, Bw, W.w, W.r, W.part);
    BILU_LAUNCH_CHECK();
    k_segsum<<<Sw, 32 * kSegWarps, 0, st>>>(Sw, k, W.stile, W.part, W.rr);
    BILU_LAUNCH_CHECK();
    k_bnorm<<<gp, 128, 0, st>>>(Pw, W.ps, W.rr);
    BILU_LAUNCH_CHECK();
    std::vector<cudaGraphExec_t> graphs(m, nullptr);
    int total = 0;
    int notdone = Pw;
    while (notdone > 0 && total < maxit) {
      k_cycle_init<<<gp, 128, 0, st>>>(Pw, m, W.ps, W.rr);
      BILU_LAUNCH_CHECK();
      // V_0 = r / beta
      k_scale_pairs<<<nt, kBT, 0, st>>>(nt, k, W.trow, W.tsys, W.r, W.rr, W.V, W.v32);
      BILU_LAUNCH_CHECK();
      int jmax = -1;
      for (int j = 0; j < m && total < maxit; ++j) {
        if (Bt->persistent) {
          // the whole step in one cooperative launch, then the active count
          // and the launch's barrier error word to the host
          BatchStepArgs a{};
          a.r0 = r0; a.r1 = r1; a.k = k; a.j = j; a.m = m; a.P = Pw; a.nt = nt; a.Sw = Sw;
          a.tol = tol;
          a.Lrow = Bt->Lrow; a.Lcol = Bt->Lcol; a.Urow = Bt->Urow; a.Ucol = Bt->Ucol;
          a.Arow = Bt->Arow; a.Acol = Bt->Acol; a.L32 = Bt->L32; a.U32 = Bt->U32;
          a.Aval = Bt->Aval; a.v32 = W.v32; a.t32 = W.t32; a.V = W.V; a.Zj = W.Z + vec * j;
          a.w = W.w; a.hcol = W.hcol; a.hn2 = W.hn2; a.part = W.part; a.vec = (long long)vec;
          a.trow = W.trow; a.tsys = W.tsys; a.stile = W.stile; a.ps = W.ps;
          a.gs.count = step_words;
          a.gs.gen = step_words + 1;
          a.gs.err = reinterpret_cast<int*>(step_words + 2);
          a.gs.spin = kSpinLimit;
          BILU_TRY(launch_batch_step(bs, Bt->rpw_M, Bt->rpw_A, a, st));
          ++graph_launches;
          BILU_TRY_CUDA(cudaMemcpyAsync(W.hpin, W.counters, sizeof(int), cudaMemcpyDeviceToHost, st));
          BILU_TRY_CUDA(cudaMemcpyAsync(W.hpin + 2, step_words + 2, sizeof(int),
                                        cudaMemcpyDeviceToHost, st));
          BILU_TRY_CUDA(cudaStreamSynchronize(st));
          if (W.hpin[2] != 0) return W.hpin[2];  // a grid barrier of the step timed out
          ++total;
          jmax = j;
          if (W.hpin[0] == 0) break;
          continue;
        }
        if (!graphs[j]) {
          cudaGraph_t g;
          BILU_TRY_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
          int rc = BILU_OK;
          double* Vj = W.V + vec * j;
          double* Zj = W.Z + vec * j;
          rc = rc ? rc : spmm_L32(Bt, Bt->rpw_M, r0, r1, k, W.v32, W.t32);
          rc = rc ? rc : spmm_U32(Bt, Bt->rpw_M, r0, r1, k, W.t32, Zj);
          rc = rc ? rc : spmm_A(Bt, Bt->rpw_A, r0, r1, k, Zj, W.w);
          for (int i = 0; i <= j + 1 && rc == BILU_OK; ++i) {
            const double* vp = i > 0 ? W.V + vec * (i - 1) : nullptr;
            const double* hp = i > 0 ? W.hcol + (size_t)(i - 1) * Pw : nullptr;
            const double* vn = i <= j ? W.V + vec * i : nullptr;
            double* out = i <= j ? W.hcol + (size_t)i * Pw : W.hn2;
            k_sweep<<<nt, kBT, 0, st>>>(nt, k, W.trow, W.tsys, vp, hp, vn, W.w, W.part);
            k_segsum<<<Sw, 32 * kSegWarps, 0, st>>>(Sw, k, W.stile, W.part, out);
          }
          k_scale_pairs<<<nt, kBT, 0, st>>>(nt, k, W.trow, W.tsys, W.w, W.hn2, W.V + vec * (j + 1),
                                            W.v32);
          cudaMemsetAsync(W.counters, 0, sizeof(int), st);
          k_givens<<<gp, 128, 0, st>>>(Pw, m, j, tol, W.ps, W.hcol, W.hn2);
          cudaMemcpyAsync(W.hpin, W.counters, sizeof(int), cudaMemcpyDeviceToHost, st);
          cudaError_t ce = cudaStreamEndCapture(st, &g);
          if (rc != BILU_OK) return rc;
          BILU_TRY_CUDA(ce);
          BILU_TRY_CUDA(cudaGraphInstantiate(&graphs[j], g, 0));
          cudaGraphDestroy(g);
          (void)Vj;
        }
        BILU_TRY_CUDA(cudaGraphLaunch(graphs[j], st));
        ++graph_launches;
        BILU_TRY_CUDA(cudaStreamSynchronize(st));
        ++total;
        jmax = j;
        if (W.hpin[0] == 0) break;
      }
      k_trisolve<<<gp, 128, 0, st>>>(Pw, m, W.ps);
      BILU_LAUNCH_CHECK();
      k_xupdate<<<nt, kBT, 0, st>>>(nt, k, m, jmax, W.trow, W.tsys, W.Z, (long long)vec, W.ps.y, Xw);
      BILU_LAUNCH_CHECK();
      BILU_TRY(spmm_A(Bt, Bt->rpw_A, r0, r1, k, Xw, W.w));
      k_residual_pairs<<<nt, kBT, 0, st>>>(nt, k, W.trow, Bw, W.w, W.r, W.part);
      BILU_LAUNCH_CHECK();
      k_segsum<<<Sw, 32 * kSegWarps, 0, st>>>(Sw, k, W.stile, W.part, W.rr);
      BILU_LAUNCH_CHECK();
      BILU_TRY_CUDA(cudaMemsetAsync(W.counters + 1, 0, sizeof(int), st));
      k_check<<<gp, 128, 0, st>>>(Pw, tol, W.ps, W.rr, W.relres, W.counters + 1);
      BILU_LAUNCH_CHECK();
      BILU_TRY_CUDA(cudaMemcpyAsync(W.hpin + 1, W.counters + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
      BILU_TRY_CUDA(cudaStreamSynchronize(st));
      notdone = W.hpin[1];
    }
    for (auto& g : graphs)
      if (g) cudaGraphExecDestroy(g);
    pair_steps += (long long)total * Pw;
    if (h_iters)
      BILU_TRY_CUDA(cudaMemcpyAsync(h_iters + (size_t)s0 * k, W.ps.iters, sizeof(int) * Pw,
                                    cudaMemcpyDeviceToHost, st));
    if (h_relres)
      BILU_TRY_CUDA(cudaMemcpyAsync(h_relres + (size_t)s0 * k, W.relres, sizeof(double) * Pw,
                                    cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  cudaEventRecord(t1, st);
  cudaEventSynchronize(t1);
  BILU_TRY_CUDA(cudaEventRecord(Bt->ev_out, st));
  BILU_TRY_CUDA(cudaStreamWaitEvent(Bt->st, Bt->ev_out, 0));
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (h_stats) {
    h_stats[0] = (double)waves.size();
    h_stats[1] = (double)graph_launches;
    h_stats[2] = (double)pair_steps;
    h_stats[3] = ms;
  }
  return BILU_OK;
}
