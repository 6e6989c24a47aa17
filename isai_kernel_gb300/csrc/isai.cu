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
// Inverse of each masked diagonal block (the unit lower triangle of the
// packed factor, or its upper triangle) by the reference's Gauss-Jordan
// without pivoting: eps 1e-14 on the pivots, one retry with 1e-12 added to
// the diagonal (isai_bsr.h:61-88, :114-120).  On a triangular block most
// Gauss-Jordan operations are exact no-ops (products with structural zeros,
// scalings by a unit pivot).  A thread per block performs only the others,
// each element receiving them in the Gauss-Jordan order:
//   lower: every pivot is 1 and the multiplier of row i at step k stays
//     L[i][k], so X[i][j] = 0 - L[i][j] X[j][j] - ... - L[i][i-1] X[i-1][j]
//     (k ascending; X[k][j] is final by step k);
//   upper: row k is untouched until step k, where it is scaled by
//     r_k = 1 / u_kk into S[k][j] = u_kj r_k; row i's scaled entries
//     m_j = u_ij r_i take m_j -= m_k S[k][j] for k = i+1, i+2, ..., and
//     X[i][k] = -(m_k r_k), X[i][i] = r_i.  The pivots it tests are the
//     u_kk themselves.
template <int BS>
__device__ __forceinline__ void dinv_lower(const double (&T)[BS][BS], double* __restrict__ out) {
  // fixed trip counts with guards (triangular bounds are not always unrolled)
#pragma unroll
  for (int j = 0; j < BS; ++j) {
    double x[BS];
#pragma unroll
    for (int i = 0; i < BS; ++i) {
      double s = i == j ? 1.0 : 0.0;
#pragma unroll
      for (int k = 0; k < BS; ++k)
        if (k >= j && k < i) s -= T[i][k] * x[k];
      x[i] = s;
    }
#pragma unroll
    for (int i = 0; i < BS; ++i) out[i * BS + j] = x[i];
  }
}

template <int BS>
__device__ __forceinline__ bool dinv_pivots_ok(const double (&T)[BS][BS], double shift) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < BS; ++k) ok = ok && fabs(T[k][k] + shift) >= 1e-14;
  return ok;
}

template <int BS>
__device__ __forceinline__ void dinv_upper(const double (&T)[BS][BS], double shift,
                                           double* __restrict__ out) {
  double r[BS], S[BS][BS];
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    r[k] = 1.0 / (T[k][k] + shift);
#pragma unroll
    for (int j = k + 1; j < BS; ++j) S[k][j] = T[k][j] * r[k];
  }
#pragma unroll
  for (int i = 0; i < BS; ++i) {
    double m[BS];
#pragma unroll
    for (int j = i + 1; j < BS; ++j) m[j] = S[i][j];
#pragma unroll
    for (int j = 0; j < i; ++j) out[i * BS + j] = 0.0;
    out[i * BS + i] = r[i];
#pragma unroll
    for (int k = i + 1; k < BS; ++k) {
      const double f = m[k];
      out[i * BS + k] = -(f * r[k]);
#pragma unroll
      for (int j = k + 1; j < BS; ++j) m[j] -= f * S[k][j];
    }
  }
}

template <int BS, bool LOWER>
__global__ void __launch_bounds__(128) k_dinv_tri(int nb, const int* __restrict__ row,
                                                  const int* __restrict__ col,
                                                  const double* __restrict__ val,
                                                  double* __restrict__ Dinv, int* fail) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int pos = find_in_row(col, __ldg(row + k), __ldg(row + k + 1), k);
  double T[BS][BS];
#pragma unroll
  for (int i = 0; i < BS; ++i)
#pragma unroll
    for (int j = 0; j < BS; ++j) {
      const bool stored = LOWER ? j < i : j >= i;
      T[i][j] = stored ? (pos >= 0 ? __ldg(val + ((long long)pos * BS + i) * BS + j) : 0.0)
                       : (LOWER && i == j ? 1.0 : 0.0);
    }
  double* out = Dinv + (long long)k * BS * BS;
  if (LOWER) {
    dinv_lower<BS>(T, out);  // unit pivots: never retried
    return;
  }
  double shift = 0.0;
  if (!dinv_pivots_ok<BS>(T, 0.0)) {
    shift = 1e-12;
    if (!dinv_pivots_ok<BS>(T, shift)) atomicMin(fail, k);
  }
  dinv_upper<BS>(T, shift, out);
}
// ---------------------------------------------------------------- pairs
// Thread per ISAI entry (t = S_j[idx] of column j, the column found by
// binary search over the column pointers, so a column of a few entries does
// not leave most of a warp idle).  lower: pairs p < idx with A(t, S_j[p])
// stored, ascending p (the reference's merge order); upper: pairs p > idx,
// descending p (the reference's ISAI-U loop order).
template <bool FILL>
__global__ void __launch_bounds__(256) k_pairs(int nb, long long mnnz,
                                               const int* __restrict__ Arow,
                                               const int* __restrict__ Acol,
                                               const int* __restrict__ Mptr,
                                               const int* __restrict__ Mind, int lower,
                                               int* __restrict__ cnt_or_ptr,
                                               int* __restrict__ PL, int* __restrict__ PS,
                                               int* nmax) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= mnnz) return;
  int lo = 0, hi = nb - 1;  // last column starting at or before q
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(Mptr + mid) <= q) lo = mid; else hi = mid - 1;
  }
  const int start = __ldg(Mptr + lo), N = __ldg(Mptr + lo + 1) - start;
  const int idx = (int)(q - start);
  if (!FILL && idx == 0) atomicMax(nmax, N);
  const int t = __ldg(Mind + q);
  const int as = __ldg(Arow + t), ae = __ldg(Arow + t + 1);
  const int out = FILL ? cnt_or_ptr[q] : 0;
  int c = 0;
  if (lower) {
    for (int p = 0; p < idx; ++p) {
      const int pos = find_in_row(Acol, as, ae, __ldg(Mind + start + p));
      if (pos >= 0) {
        if (FILL) { PL[out + c] = p; PS[out + c] = pos; }
        ++c;
      }
    }
  } else {
    for (int p = N - 1; p > idx; --p) {
      const int pos = find_in_row(Acol, as, ae, __ldg(Mind + start + p));
      if (pos >= 0) {
        if (FILL) { PL[out + c] = p; PS[out + c] = pos; }
        ++c;
      }
    }
  }
  if (!FILL) cnt_or_ptr[q] = c;
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
      // an entry without pairs has rhs = delta_{t,j} I: Dinv[t] I is Dinv[t]
      // exactly (every other product is a zero), so it is copied
      const bool copy = qb == qe;
#pragma unroll
      for (int q = 0; q < EPL; ++q) {
        double s = 0.0;
        if (tl * EPL + q < BS2) {
          if (copy) {
            s = t == j ? __ldg(Di + er[q] * BS + ec[q]) : 0.0;
          } else {
#pragma unroll
            for (int k = 0; k < BS; ++k)
              s = fma(__ldg(Di + er[q] * BS + k), sR[k * BS + ec[q]], s);
          }
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
  if (lower)
    k_dinv_tri<BS, true><<<ceil_div(nb, 128), 128, 0, st>>>(nb, row, col, val, Dinv, d_fail);
  else
    k_dinv_tri<BS, false><<<ceil_div(nb, 128), 128, 0, st>>>(nb, row, col, val, Dinv, d_fail);
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
    k_pairs<false><<<ceil_div(std::max(mnnz, 1), 256), 256, 0, st>>>(
        nb, mnnz, Arow, Acol, Mptr, Mind, lower, PairPtr, nullptr, nullptr, nmax);
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
                    int lower, const int* PairPtr, int mnnz, int* PL, int* PS, cudaStream_t st) {
  if (nb == 0 || mnnz == 0) return BILU_OK;
  k_pairs<true><<<ceil_div(mnnz, 256), 256, 0, st>>>(nb, mnnz, Arow, Acol, Mptr, Mind, lower,
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
  int mnnz = 0;
  if (nb > 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(&mnnz, d_Mptr + nb, sizeof(int), cudaMemcpyDeviceToHost,
                                  S(stream)));
    BILU_TRY_CUDA(cudaStreamSynchronize(S(stream)));
  }
  return pairs_fill_impl(nb, d_Arow, d_Acol, d_Mptr, d_Mind, lower != 0, d_PairPtr, mnnz,
                         d_PairPLocal, d_PairSrc, S(stream));
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
