// ISAI setup on the GPU: diagonal-block inverses, dependency pair lists and
// the per-column ISAI-L / ISAI-U solves (FP64, sm_103a).
//
//   build_DinvL/U_from_BSR5_kernel_fix   isai_bsr.h:91,126 (+:33,:61)
//   count/fill_pairs_lower_kernel_v2     isai_bsr.h:1378,1427 (+ scan main.cu:684)
//   isai_lower_* (7 kernels)             isai_bsr.h:288-1376, cacheY_isai.h:159
//   isai_upper_bsr5_warpcol_with_Dinv    isai_bsr.h:161
//
// The reference gives each column a whole warp and runs its merges and block
// lookups on lane 0.  Here a column is a team of bs*bs/EPL lanes that own
// the elements of the current block (EPL elements each): bs=4 packs two
// columns per warp, bs=8 gives each lane two elements of one column.  The
// pair lists are built for M_U as well, so ISAI-U does no binary searches in
// its inner loop.  Products keep the reference's order (sum over k, then
// subtract) and run on the DFMA pipe: DMMA m8n8k4 measured slower than DFMA
// on GB300 (1.05 vs 1.2 TFLOP/s) and a 4x4 block fills 1/8 of its tile.
#include "common.cuh"
#include "scan.cuh"

namespace bilu {

namespace {

template <int BS>
struct Team {
  static constexpr int BS2 = BS * BS;
  static constexpr int EPL = BS2 > 32 ? (BS2 + 31) / 32 : 1;  // elements per lane
  static constexpr int TL = (BS2 + EPL - 1) / EPL;             // lanes per team
  static constexpr int TPW = 32 / TL;                          // teams per warp
  static constexpr int SPAN = 32 / TPW;                        // lane span of a team
};

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

// ---------------------------------------------------------------- Dinv
// Team of BS lanes per block row; lane i holds row i of the work matrix and
// of the identity.  Gauss-Jordan without pivoting, eps 1e-14, retry once
// with 1e-12 added to the diagonal (isai_bsr.h:61-88, :114-120).
template <int BS>
__device__ __forceinline__ bool gauss_jordan(double* M, double* Iv, int i, int base,
                                            unsigned mask) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    double piv = __shfl_sync(mask, M[k], base + k);
    ok = ok && fabs(piv) >= 1e-14;
    double invp = 1.0 / piv;
    if (i == k) {
#pragma unroll
      for (int j = 0; j < BS; ++j) { M[j] *= invp; Iv[j] *= invp; }
    }
    double f = M[k];
#pragma unroll
    for (int j = 0; j < BS; ++j) {
      double rm = __shfl_sync(mask, M[j], base + k);
      double ri = __shfl_sync(mask, Iv[j], base + k);
      if (i != k) {
        M[j] -= f * rm;
        Iv[j] -= f * ri;
      }
    }
  }
  return ok;
}

template <int BS>
__global__ void __launch_bounds__(256) k_dinv(int nb, const int* __restrict__ row,
                                              const int* __restrict__ col,
                                              const double* __restrict__ val, int lower,
                                              double* __restrict__ Dinv, int* fail) {
  constexpr int G = 32 / BS;
  int lane = threadIdx.x & 31;
  int g = lane / BS, i = lane - g * BS;
  long long kk = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * G + g;
  bool active = g < G && kk < nb;
  int k = active ? (int)kk : 0;
  int base = g < G ? g * BS : 0;
  double B[BS], M[BS], Iv[BS];
  int pos = nb > 0 ? find_in_row(col, __ldg(row + k), __ldg(row + k + 1), k) : -1;
#pragma unroll
  for (int j = 0; j < BS; ++j) {
    double v = pos >= 0 ? val[((long long)pos * BS + i) * BS + j] : 0.0;
    if (lower ? (j > i) : (j < i)) v = 0.0;
    if (lower && j == i) v = 1.0;
    B[j] = v;
    M[j] = v;
    Iv[j] = (j == i) ? 1.0 : 0.0;
  }
  unsigned mask = 0xffffffffu;
  bool ok = gauss_jordan<BS>(M, Iv, i, base, mask);
  if (__any_sync(mask, active && !ok)) {
    bool redo = !ok;
    double M2[BS], I2[BS];
#pragma unroll
    for (int j = 0; j < BS; ++j) {
      M2[j] = B[j] + ((j == i) ? 1e-12 : 0.0);
      I2[j] = (j == i) ? 1.0 : 0.0;
    }
    bool ok2 = gauss_jordan<BS>(M2, I2, i, base, mask);
    if (redo) {
#pragma unroll
      for (int j = 0; j < BS; ++j) Iv[j] = I2[j];
      if (active && !ok2) atomicMin(fail, k);
    }
  }
  if (!active) return;
#pragma unroll
  for (int j = 0; j < BS; ++j) Dinv[((long long)k * BS + i) * BS + j] = Iv[j];
}

// Thread per block row (bs 4 and 5: the 2*bs*bs work values fit in
// registers): the same Gauss-Jordan steps as the team version above, in the
// same order, without the redundant per-lane divisions and shuffles.
template <int BS>
__device__ __forceinline__ bool gauss_jordan_t(double (&M)[BS][BS], double (&Iv)[BS][BS]) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    double piv = M[k][k];
    ok = ok && fabs(piv) >= 1e-14;
    double invp = 1.0 / piv;
#pragma unroll
    for (int j = 0; j < BS; ++j) {
      M[k][j] *= invp;
      Iv[k][j] *= invp;
    }
#pragma unroll
    for (int i = 0; i < BS; ++i) {
      if (i == k) continue;
      double f = M[i][k];
#pragma unroll
      for (int j = 0; j < BS; ++j) {
        M[i][j] -= f * M[k][j];
        Iv[i][j] -= f * Iv[k][j];
      }
    }
  }
  return ok;
}

template <int BS>
__global__ void __launch_bounds__(128) k_dinv_t(int nb, const int* __restrict__ row,
                                                const int* __restrict__ col,
                                                const double* __restrict__ val, int lower,
                                                double* __restrict__ Dinv, int* fail) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  int pos = find_in_row(col, __ldg(row + k), __ldg(row + k + 1), k);
  double B[BS][BS], M[BS][BS], Iv[BS][BS];
#pragma unroll
  for (int i = 0; i < BS; ++i)
#pragma unroll
    for (int j = 0; j < BS; ++j) {
      double v = pos >= 0 ? __ldg(val + ((long long)pos * BS + i) * BS + j) : 0.0;
      if (lower ? (j > i) : (j < i)) v = 0.0;
      if (lower && j == i) v = 1.0;
      B[i][j] = v;
      M[i][j] = v;
      Iv[i][j] = (j == i) ? 1.0 : 0.0;
    }
  if (!gauss_jordan_t<BS>(M, Iv)) {
#pragma unroll
    for (int i = 0; i < BS; ++i)
#pragma unroll
      for (int j = 0; j < BS; ++j) {
        M[i][j] = B[i][j] + ((j == i) ? 1e-12 : 0.0);
        Iv[i][j] = (j == i) ? 1.0 : 0.0;
      }
    if (!gauss_jordan_t<BS>(M, Iv)) atomicMin(fail, k);
  }
  double* out = Dinv + (long long)k * BS * BS;
#pragma unroll
  for (int i = 0; i < BS; ++i)
#pragma unroll
    for (int j = 0; j < BS; ++j) out[i * BS + j] = Iv[i][j];
}

// ---------------------------------------------------------------- pairs
// Warp per ISAI column j; lane per entry idx.  lower: pairs p < idx with
// A(t, S_j[p]) stored, ascending p (the reference's merge order); upper:
// pairs p > idx, descending p (the reference's ISAI-U loop order).
template <bool FILL>
__global__ void __launch_bounds__(256) k_pairs(int nb, const int* __restrict__ Arow,
                                               const int* __restrict__ Acol,
                                               const int* __restrict__ Mptr,
                                               const int* __restrict__ Mind, int lower,
                                               int* __restrict__ cnt_or_ptr,
                                               int* __restrict__ PL, int* __restrict__ PS,
                                               int* nmax) {
  int lane = threadIdx.x & 31;
  int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= nb) return;
  int start = Mptr[j], end = Mptr[j + 1], N = end - start;
  if (!FILL && lane == 0) atomicMax(nmax, N);
  for (int idx = lane; idx < N; idx += 32) {
    int t = Mind[start + idx];
    int as = __ldg(Arow + t), ae = __ldg(Arow + t + 1);
    int out = FILL ? cnt_or_ptr[start + idx] : 0;
    int c = 0;
    if (lower) {
      for (int p = 0; p < idx; ++p) {
        int pos = find_in_row(Acol, as, ae, Mind[start + p]);
        if (pos >= 0) {
          if (FILL) { PL[out + c] = p; PS[out + c] = pos; }
          ++c;
        }
      }
    } else {
      for (int p = N - 1; p > idx; --p) {
        int pos = find_in_row(Acol, as, ae, Mind[start + p]);
        if (pos >= 0) {
          if (FILL) { PL[out + c] = p; PS[out + c] = pos; }
          ++c;
        }
      }
    }
    if (!FILL) cnt_or_ptr[start + idx] = c;
  }
}

// ---------------------------------------------------------------- ISAI solve
// Team per column.  Column j of M_L: for idx ascending, rhs = delta_{t,j} I,
// rhs -= A(t,p) Y_p over the pairs, Y_idx = Dinv[t] rhs.  M_U: idx
// descending with the upper pair list.  The first kCache blocks of a column
// stay in shared memory; later ones are re-read from Mval (written by this
// team and ordered by __syncwarp).
template <int BS>
struct IsaiCfg {
  static constexpr int kCache = BS == 8 ? 12 : 24;
  static constexpr int kWarps = BS == 8 ? 4 : 8;
};

template <int BS>
__global__ void __launch_bounds__(256) k_isai(int nb, const double* __restrict__ Aval,
                                              const int* __restrict__ Mptr,
                                              const int* __restrict__ Mind, int lower,
                                              const int* __restrict__ PairPtr,
                                              const int* __restrict__ PairPL,
                                              const int* __restrict__ PairSrc,
                                              const double* __restrict__ Dinv,
                                              double* __restrict__ Mval) {
  using T = Team<BS>;
  constexpr int BS2 = T::BS2, EPL = T::EPL, TL = T::TL, TPW = T::TPW, SPAN = T::SPAN;
  constexpr int CACHE = IsaiCfg<BS>::kCache;
  extern __shared__ double smem[];
  int lane = threadIdx.x & 31;
  int warp = threadIdx.x >> 5;
  int team = lane / SPAN, tl = lane - team * SPAN;
  bool lane_on = team < TPW && tl < TL;
  long long j = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * TPW + team;
  double* sY = smem + ((size_t)warp * TPW + (team < TPW ? team : 0)) * (size_t)(CACHE + 1) * BS2;
  double* sR = sY + (size_t)CACHE * BS2;  // rhs of the current entry
  unsigned wmask = 0xffffffffu;
  bool col_on = team < TPW && j < nb;
  int start = col_on ? Mptr[j] : 0;
  int N = col_on ? Mptr[j + 1] - start : 0;
  // teams of one warp loop in lock-step over the longest column of the warp
  int Nw = N;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) Nw = max(Nw, __shfl_xor_sync(wmask, Nw, o));
  int er[EPL], ec[EPL];
#pragma unroll
  for (int q = 0; q < EPL; ++q) {
    int e = tl * EPL + q;
    er[q] = e / BS;
    ec[q] = e - er[q] * BS;
  }
  for (int step = 0; step < Nw; ++step) {
    bool on = col_on && lane_on && step < N;
    int idx = lower ? step : N - 1 - step;
    int t = 0, qb = 0, qe = 0;
    if (col_on && step < N) {
      t = Mind[start + idx];
      qb = PairPtr[start + idx];
      qe = PairPtr[start + idx + 1];
    }
    double rhs[EPL];
#pragma unroll
    for (int q = 0; q < EPL; ++q) rhs[q] = (on && t == j && er[q] == ec[q]) ? 1.0 : 0.0;
    for (int qq = qb; qq < qe; ++qq) {
      int pl = PairPL[qq];
      const double* Ab = Aval + (long long)PairSrc[qq] * BS2;
      const double* Yp = pl < CACHE ? sY + (size_t)pl * BS2 : Mval + (long long)(start + pl) * BS2;
      if (on) {
#pragma unroll
        for (int q = 0; q < EPL; ++q) {
          if (tl * EPL + q >= BS2) continue;
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < BS; ++k) s = fma(__ldg(Ab + er[q] * BS + k), Yp[k * BS + ec[q]], s);
          rhs[q] -= s;
        }
      }
    }
    // rhs block to shared memory, then Y = Dinv[t] * rhs
    if (on) {
#pragma unroll
      for (int q = 0; q < EPL; ++q)
        if (tl * EPL + q < BS2) sR[tl * EPL + q] = rhs[q];
    }
    __syncwarp();
    double y[EPL];
    if (on) {
      const double* Di = Dinv + (long long)t * BS2;
#pragma unroll
      for (int q = 0; q < EPL; ++q) {
        double s = 0.0;
        if (tl * EPL + q < BS2) {
#pragma unroll
          for (int k = 0; k < BS; ++k) s = fma(__ldg(Di + er[q] * BS + k), sR[k * BS + ec[q]], s);
        }
        y[q] = s;
      }
#pragma unroll
      for (int q = 0; q < EPL; ++q) {
        int e = tl * EPL + q;
        if (e >= BS2) continue;
        Mval[(long long)(start + idx) * BS2 + e] = y[q];
        if (idx < CACHE) sY[(size_t)idx * BS2 + e] = y[q];
      }
    }
    __syncwarp();
  }
}

template <int BS>
int launch_dinv(int nb, const int* row, const int* col, const double* val, int lower,
                double* Dinv, int* d_fail, cudaStream_t st) {
  if (nb == 0) return BILU_OK;
  if constexpr (BS <= 5) {
    k_dinv_t<BS><<<ceil_div(nb, 128), 128, 0, st>>>(nb, row, col, val, lower, Dinv, d_fail);
  } else {
    constexpr int G = 32 / BS;
    long long warps = (nb + G - 1) / G;
    k_dinv<BS><<<ceil_div(warps, 8), 256, 0, st>>>(nb, row, col, val, lower, Dinv, d_fail);
  }
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

template <int BS>
int launch_isai(int nb, const double* Aval, const int* Mptr, const int* Mind, int lower,
                const int* pp, const int* pl, const int* ps, const double* Dinv, double* Mval,
                cudaStream_t st) {
  if (nb == 0) return BILU_OK;
  using T = Team<BS>;
  constexpr int W = IsaiCfg<BS>::kWarps;
  size_t smem = (size_t)W * T::TPW * (IsaiCfg<BS>::kCache + 1) * T::BS2 * sizeof(double);
  static bool attr_set = false;
  if (!attr_set) {
    BILU_TRY_CUDA(cudaFuncSetAttribute(k_isai<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr_set = true;
  }
  long long warps = (nb + T::TPW - 1) / T::TPW;
  k_isai<BS><<<ceil_div(warps, W), 32 * W, smem, st>>>(nb, Aval, Mptr, Mind, lower, pp, pl, ps,
                                                       Dinv, Mval);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

}  // namespace

int dinv_impl(int nb, int bs, const int* row, const int* col, const double* val, int lower,
              double* Dinv, int* d_fail, cudaStream_t st) {
  return BILU_DISPATCH_BS(bs, launch_dinv, nb, row, col, val, lower, Dinv, d_fail, st);
}

size_t pairs_ws(long long mnnz) { return carve_size(sizeof(int)) + scan_ws_bytes(mnnz + 1); }

int pairs_ptr_impl(int nb, const int* Arow, const int* Acol, const int* Mptr, const int* Mind,
                   int lower, int* PairPtr, int mnnz, int* h_total, int* h_nmax, Carver& ws,
                   cudaStream_t st) {
  int* nmax = ws.take<int>(1);
  if (!nmax) return BILU_ERR_WORKSPACE;
  BILU_TRY_CUDA(cudaMemsetAsync(nmax, 0, sizeof(int), st));
  if (nb > 0) {
    k_pairs<false><<<ceil_div(nb, 8), 256, 0, st>>>(nb, Arow, Acol, Mptr, Mind, lower, PairPtr,
                                                    nullptr, nullptr, nmax);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY(scan_exclusive(PairPtr, PairPtr, mnnz, h_total, ws, st));
  if (h_nmax) {
    BILU_TRY_CUDA(cudaMemcpyAsync(h_nmax, nmax, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  return BILU_OK;
}

int pairs_fill_impl(int nb, const int* Arow, const int* Acol, const int* Mptr, const int* Mind,
                    int lower, const int* PairPtr, int* PL, int* PS, cudaStream_t st) {
  if (nb == 0) return BILU_OK;
  k_pairs<true><<<ceil_div(nb, 8), 256, 0, st>>>(nb, Arow, Acol, Mptr, Mind, lower,
                                                 const_cast<int*>(PairPtr), PL, PS, nullptr);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int isai_impl(int nb, int bs, const double* Aval, const int* Mptr, const int* Mind, int lower,
              const int* pp, const int* pl, const int* ps, const double* Dinv, double* Mval,
              cudaStream_t st) {
  return BILU_DISPATCH_BS(bs, launch_isai, nb, Aval, Mptr, Mind, lower, pp, pl, ps, Dinv, Mval,
                          st);
}

}  // namespace bilu

using namespace bilu;

extern "C" int bilu_build_dinv(int nb, int bs, const int* d_Arow, const int* d_Acol,
                               const double* d_Aval, int lower, double* d_Dinv,
                               bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_Arow || !d_Acol || !d_Aval || !d_Dinv))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return dinv_impl(nb, bs, d_Arow, d_Acol, d_Aval, lower != 0, d_Dinv, nullptr, S(stream));
}

extern "C" size_t bilu_pairs_ws_bytes(int mnnz) { return pairs_ws(mnnz); }

extern "C" int bilu_pairs_ptr(int nb, const int* d_Arow, const int* d_Acol, const int* d_Mptr,
                              const int* d_Mind, int lower, int* d_PairPtr, int* h_total,
                              int* h_nmax, void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || !d_PairPtr) return BILU_ERR_ARG;
  int mnnz = 0;
  if (nb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&mnnz, d_Mptr + nb, sizeof(int), cudaMemcpyDeviceToHost,
                                  S(stream)));
    BILU_TRY_CUDA(cudaStreamSynchronize(S(stream)));
  }
  Carver ws(d_ws, ws_bytes);
  return pairs_ptr_impl(nb, d_Arow, d_Acol, d_Mptr, d_Mind, lower != 0, d_PairPtr, mnnz, h_total,
                        h_nmax, ws, S(stream));
}

extern "C" int bilu_pairs_fill(int nb, const int* d_Arow, const int* d_Acol, const int* d_Mptr,
                               const int* d_Mind, int lower, const int* d_PairPtr,
                               int* d_PairPLocal, int* d_PairSrc, bilu_stream_t stream) {
  if (nb < 0) return BILU_ERR_ARG;
  return pairs_fill_impl(nb, d_Arow, d_Acol, d_Mptr, d_Mind, lower != 0, d_PairPtr, d_PairPLocal,
                         d_PairSrc, S(stream));
}

extern "C" int bilu_isai_compute(int nb, int bs, const double* d_Aval, const int* d_Mptr,
                                 const int* d_Mind, int lower, const int* d_PairPtr,
                                 const int* d_PairPLocal, const int* d_PairSrc,
                                 const double* d_Dinv, double* d_Mval, bilu_stream_t stream) {
  if (nb < 0) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  return isai_impl(nb, bs, d_Aval, d_Mptr, d_Mind, lower != 0, d_PairPtr, d_PairPLocal,
                   d_PairSrc, d_Dinv, d_Mval, S(stream));
}
