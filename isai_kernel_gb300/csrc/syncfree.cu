// BILU(0) and block triangular solves on the dependency DAG (sm_103a):
//
//   bsrilu02_inplace (bsrilu.h:20, cuSPARSE bsrilu02)   -> k_bilu0_levels
//   spTrSolveL / spTrSolveU (cape_sptrsv.h:8,55)         -> k_sptrsv_levels,
//                                                            k_sptrsv (sync-free)
//
// Level schedule (default): a breadth-first sweep (k_bfs_levels) groups the
// block rows by dependency level; one cooperative launch then processes a
// level with a group of bs lanes per row and meets at a bounded grid barrier.
//
// Sync-free schedule (the reference's design, kept for the solve): a warp
// owns one block row at a time.  Rows are handed out by an atomic ticket
// counter in level order, so every row a warp waits on was taken by a warp
// that is already running (the reference maps rows to threads statically and
// relies on scheduling order).  A finished row publishes its flag with
// st.release; waiters poll with relaxed loads, take one acquire fence when
// the flag is set, and read the producer's data through L2 (ld.cg).
//
// Every wait is bounded: after kSpinLimit polls the waiter sets the error
// word to BILU_ERR_TIMEOUT, and all other waiters see the error word and
// leave, so no launch hangs.
#include <climits>

#include <algorithm>

#include "common.cuh"
#include "gridsync.cuh"
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
  // reciprocal pivots 1 / u_rr of the block rows (nb x bs): written by the
  // factorisation, read by upper solves instead of dividing (null: divide)
  double* rdiag = nullptr;
  // per lower position pk of the factor: how many blocks dependency K
  // updates in row I (null: not counted, every dependency searches)
  const int* nmatch = nullptr;
};

// Warp-wide wait until flags[K] != 0.  Returns false if the launch aborted.
__device__ __forceinline__ bool warp_wait(const int* flag, int* err, long long spin) {
  long long n = 0;
  unsigned ns = 32;
  while (true) {
    int v = ld_relaxed(flag);
    if (__all_sync(FULL, v != 0)) {
      fence_acquire();
      return true;
    }
    if (__any_sync(FULL, ld_relaxed(err) != 0)) return false;
    if (++n > spin) {
      if ((threadIdx.x & 31) == 0) atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    backoff(ns);
  }
}

// Single-lane wait (lanes of a warp may wait on different rows).
__device__ __forceinline__ bool lane_wait(const int* flag, int* err, long long spin) {
  long long n = 0;
  unsigned ns = 32;
  while (ld_relaxed(flag) == 0) {
    if (ld_relaxed(err) != 0) return false;
    if (++n > spin) {
      atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    backoff(ns);
  }
  fence_acquire();
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

// ------------------------------------------------------------------ SpTRSV
// Block-row solve on a packed factor.  LOWER: x_I = b_I - sum_{K<I} B_IK x_K
// then the diagonal block's lower part; otherwise the upper part and J > I
// in reverse ticket order.  UNIT: the diagonal block contributes its strict
// triangle and no division (unit diagonal).  Lane (slot, r) accumulates row
// r of blocks slot, slot+G, ...; slots are summed by shuffles.
// Structural part of one block row of a triangular solve: everything that
// does not depend on x (the row, its diagonal position, the first pass of
// blocks with their column indices).  The level schedule loads it for the
// next level before the barrier, so only the x reads follow the barrier.
template <int BS>
struct RowPre {
  int I, dI, ps, pe;  // warp-uniform; I < 0: no row
  int K;              // this lane's block column in the first pass, or -1
  double a[BS];       // row r of that block
  double dq[BS];      // lanes q < BS: row q of the diagonal block
  double bq;          // lanes q < BS: b_q
};

// 1 / d for scalar row (lane % BS) of block row I: the factorisation's
// stored reciprocal when there is one (the same correctly rounded
// quotient), else the division.
template <int BS>
__device__ __forceinline__ double recip_pivot(const double* rdiag, int I, double d) {
  if (rdiag) return __ldg(rdiag + (long long)I * BS + (threadIdx.x & 31) % BS);
  return 1.0 / d;
}

template <int BS, bool LOWER, bool UNIT>
__device__ __forceinline__ void sptrsv_prefetch(int I, const int* __restrict__ row,
                                                const int* __restrict__ col,
                                                const int* __restrict__ diag,
                                                const double* __restrict__ val,
                                                const double* __restrict__ b, RowPre<BS>& p) {
  constexpr int G = 32 / BS;
  const int lane = threadIdx.x & 31, slot = lane / BS, r = lane - slot * BS;
  p.I = I;
  p.K = -1;
  if (I < 0) return;
  int rs = __ldg(row + I), re = __ldg(row + I + 1), dI = __ldg(diag + I);
  p.dI = dI;
  p.ps = LOWER ? rs : dI + 1;
  p.pe = LOWER ? dI : re;
  int q = p.ps + slot;
  if (slot < G && q < p.pe) {
    p.K = __ldg(col + q);
    const double* blk = val + (long long)q * BS * BS + r * BS;
#pragma unroll
    for (int c = 0; c < BS; ++c) p.a[c] = __ldg(blk + c);
  }
  // the diagonal block row and b do not depend on x
  p.bq = 0.0;
  if (lane < BS) {
    const double* D = val + (long long)dI * BS * BS + lane * BS;
#pragma unroll
    for (int c = 0; c < BS; ++c) p.dq[c] = __ldg(D + c);
    p.bq = __ldg(b + (long long)I * BS + lane);
  } else {
#pragma unroll
    for (int c = 0; c < BS; ++c) p.dq[c] = 1.0;
  }
}

// The x-dependent part of the row, one warp.  Lane (slot, r) accumulates
// row r of blocks slot, slot+G, ...; slots are summed by shuffles.  The
// diagonal block is solved by substitution spread over lanes 0..BS-1 (lane
// q holds row q of the block): step c finalises x_c on lane c (times the
// pivot reciprocal unless UNIT) and broadcasts it; LOWER runs c ascending,
// otherwise descending, so every x_q subtracts its terms in the oracle's
// order.  WAIT: the rows read may still be in progress (sync-free
// schedule); PUBLISH: lane 0 stores x_I and releases the row's flag.
// Returns false if the launch aborted.
template <int BS, bool LOWER, bool UNIT, bool WAIT, bool PUBLISH>
__device__ __forceinline__ bool sptrsv_finish(const RowPre<BS>& p, const int* __restrict__ col,
                                              const double* __restrict__ val, double* x,
                                              const SyncState& ss) {
  constexpr int BS2 = BS * BS;
  constexpr int G = 32 / BS;
  const int lane = threadIdx.x & 31, slot = lane / BS, r = lane - slot * BS;
  // Blocks are summed in row order: each block's partial starts from zero
  // and the partials of a pass are added in slot order, so the total is
  // the same as a sequential sum over the row's blocks (the level schedule
  // sums that way and gives bit-identical x).
  double tot = 0.0, rq = 1.0;
  bool ok = true;
  {
    double d = p.dq[0];  // pivot of row `lane` (lanes < BS), one division per lane
#pragma unroll
    for (int c = 1; c < BS; ++c)
      if (c == lane) d = p.dq[c];
    double sp = 0.0;
    if (p.K >= 0) {
      if (WAIT) ok = lane_wait(ss.flags + p.K, ss.err, ss.spin);
      if (ok) {
        const double* xk = x + (long long)p.K * BS;
        double xv[BS];
#pragma unroll
        for (int c = 0; c < BS; ++c) xv[c] = __ldcg(xk + c);
        if (!UNIT) rq = recip_pivot<BS>(ss.rdiag, p.I, d);  // overlaps the x reads
#pragma unroll
        for (int c = 0; c < BS; ++c) sp = fma(p.a[c], xv[c], sp);
      }
    } else if (!UNIT) {
      rq = recip_pivot<BS>(ss.rdiag, p.I, d);
    }
    if (WAIT && __any_sync(FULL, !ok)) return false;
#pragma unroll
    for (int g = 0; g < G; ++g) tot += __shfl_sync(FULL, sp, g * BS + r);
  }
  for (int p0 = p.ps + G; p0 < p.pe; p0 += G) {  // rows with more than G blocks
    int q = p0 + slot;
    double sp = 0.0;
    if (slot < G && q < p.pe) {
      int K = __ldg(col + q);
      if (WAIT) ok = lane_wait(ss.flags + K, ss.err, ss.spin);
      if (ok) {
        const double* blk = val + (long long)q * BS2 + r * BS;
        const double* xk = x + (long long)K * BS;
#pragma unroll
        for (int c = 0; c < BS; ++c) sp = fma(__ldg(blk + c), __ldcg(xk + c), sp);
      }
    }
    if (WAIT && __any_sync(FULL, !ok)) return false;
#pragma unroll
    for (int g = 0; g < G; ++g) tot += __shfl_sync(FULL, sp, g * BS + r);
  }
  double v = p.bq - tot, xv = 0.0;
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const int c = LOWER ? k : BS - 1 - k;
    double mine = (UNIT || lane != c) ? v : v * rq;
    double xc = __shfl_sync(FULL, mine, c);
    if (lane == c) xv = xc;
    if (LOWER ? (lane > c && lane < BS) : (lane < c)) v -= p.dq[c] * xc;
  }
  if (PUBLISH) {
    // lane 0 stores the row and releases its flag (st.release orders its own
    // stores before the flag)
    double xs[BS];
#pragma unroll
    for (int c = 0; c < BS; ++c) xs[c] = __shfl_sync(FULL, xv, c);
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < BS; ++c) x[(long long)p.I * BS + c] = xs[c];
      if (p.I != ss.withhold) st_release(ss.flags + p.I, 1);
    }
  } else if (lane < BS) {
    x[(long long)p.I * BS + lane] = xv;
  }
  return true;
}

// Block-row solve on a packed factor.  LOWER: x_I = b_I - sum_{K<I} B_IK x_K
// then the diagonal block's lower part; otherwise the upper part and J > I
// in reverse ticket order.  UNIT: the diagonal block contributes its strict
// triangle and no division (unit diagonal).  Lane (slot, r) accumulates row
// r of blocks slot, slot+G, ...; slots are summed by shuffles.
// One block row of the solve, executed by one warp.  WAIT: the rows it
// reads may still be in progress and are waited for through their flags;
// otherwise they are final (level schedule).  x_I is stored by lane 0.
// Returns false if the launch aborted.
template <int BS, bool LOWER, bool UNIT, bool WAIT>
__device__ __forceinline__ bool sptrsv_row(int I, const int* __restrict__ row,
                                           const int* __restrict__ col,
                                           const int* __restrict__ diag,
                                           const double* __restrict__ val,
                                           const double* __restrict__ b, double* x,
                                           const SyncState& ss) {
  constexpr int BS2 = BS * BS;
  constexpr int G = 32 / BS;
  int lane = threadIdx.x & 31;
  int slot = lane / BS, r = lane - slot * BS;
  int rs = __ldg(row + I), re = __ldg(row + I + 1), dI = __ldg(diag + I);
  int ps = LOWER ? rs : dI + 1, pe = LOWER ? dI : re;
  double s = 0.0;
  bool ok = true;
  for (int p0 = ps; p0 < pe; p0 += G) {
    int p = p0 + slot;
    if (slot < G && p < pe && ok) {
      int K = __ldg(col + p);
      if (WAIT) ok = lane_wait(ss.flags + K, ss.err, ss.spin);
      if (ok) {
        const double* blk = val + (long long)p * BS2 + r * BS;
        const double* xk = x + (long long)K * BS;
#pragma unroll
        for (int c = 0; c < BS; ++c) s = fma(__ldg(blk + c), __ldcg(xk + c), s);
      }
    }
  }
  if (WAIT && __any_sync(FULL, !ok)) return false;
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
  }
  return true;
}

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
  int lane = threadIdx.x & 31;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ss.ticket, 1);
    t = __shfl_sync(FULL, t, 0);
    if (t >= nb) return;
    int I = ss.order ? __ldg(ss.order + t) : (LOWER ? t : nb - 1 - t);
    RowPre<BS> p;
    sptrsv_prefetch<BS, LOWER, UNIT>(I, row, col, diag, val, b, p);
    if (!sptrsv_finish<BS, LOWER, UNIT, true, true>(p, col, val, x, ss)) return;
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
      unsigned ns = 32;
      int v;
      while ((v = ld_relaxed(f)) == 0) {
        if (ld_relaxed(err) != 0) return;
        if (++n > spin) {
          atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
          return;
        }
        backoff(ns);
      }
      lv = max(lv, v);  // the level value itself is the only datum read
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

// ------------------------------------------------------------------ level schedule
// The dependency DAG is cut into levels (level 0: rows without dependencies;
// level l+1: rows whose dependencies all sit in levels <= l).  A level
// scheduled kernel is one cooperative launch (all CTAs co-resident) that
// processes the rows of a level with one warp each and then meets at a
// grid-wide barrier; no per-row flags are polled.

// Dependencies of row I: lower -> columns in [row[I], diag[I]); upper ->
// columns in (diag[I], row[I+1]).  cnt[K] += 1 per dependent of K.
__global__ void k_dep_count(int nb, const int* __restrict__ row, const int* __restrict__ col,
                            const int* __restrict__ diag, int lower, int* __restrict__ cnt,
                            int* __restrict__ indeg, int* maxdeg) {
  int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nb) return;
  int ps = lower ? row[I] : diag[I] + 1, pe = lower ? diag[I] : row[I + 1];
  indeg[I] = pe - ps;
  if (pe - ps > 0) atomicMax(maxdeg, pe - ps);
  for (int p = ps; p < pe; ++p) atomicAdd(cnt + col[p], 1);
}

// Successor lists: sidx[sptr[K] ...] = rows that depend on K (any order).
__global__ void k_dep_fill(int nb, const int* __restrict__ row, const int* __restrict__ col,
                           const int* __restrict__ diag, int lower, const int* __restrict__ sptr,
                           int* __restrict__ cursor, int* __restrict__ sidx) {
  int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nb) return;
  int ps = lower ? row[I] : diag[I] + 1, pe = lower ? diag[I] : row[I + 1];
  for (int p = ps; p < pe; ++p) {
    int K = col[p];
    sidx[sptr[K] + atomicAdd(cursor + K, 1)] = I;
  }
}

// Appends the rows of the warp's ready lanes to order[base0 + ...] with one
// atomic on the level's append counter per warp (ballot + prefix count).
// Called by all 32 lanes.
__device__ __forceinline__ void warp_append(bool ready, int J, int* order, int base0,
                                            int* count) {
  const unsigned m = __ballot_sync(FULL, ready);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(FULL, base, leader);
  if (ready) order[base0 + base + __popc(m & ((1u << lane) - 1u))] = J;
}

// Breadth-first level sweep (Kahn's algorithm, one level per barrier):
// order[] receives the rows level by level, lvl_ptr[l] the start of level l
// (lvl_ptr[nlev] = nb), *nlev the number of levels.  Warps take 32
// consecutive frontier rows, walk their successor lists in step (one slot
// per lane and round), decrement in-degrees and append the rows that reach
// zero with one atomic per warp.  The rows inside a level come in append
// order (k_sort_levels orders them afterwards); the level sizes do not
// depend on it.
//
// Every CTA must see the same frontier: after the barrier that closes
// level l, each CTA reads how many rows level l appended, while the CTAs
// that left the barrier first are already appending level l + 1's rows.
// So the levels count their appends in three rotating counters (cnt[l % 3];
// the rows of the initial frontier in cnt[2]): the one a CTA reads after
// barrier l is not written again until level l + 3, and CTA 0 clears the
// counter of level l + 1 while it works on level l, after every CTA has
// read it at level l - 2 (barrier l - 1 orders the reads before the clear,
// barrier l the clear before the appends).  Rows go to absolute positions
// e + count, e being the end of the current frontier, which every CTA knows.
__global__ void __launch_bounds__(256) k_bfs_levels(int nb, const int* __restrict__ sptr,
                                                    const int* __restrict__ sidx, int* indeg,
                                                    int* order, int* lvl_ptr, int* cnt,
                                                    int* nlev, GridSync gs) {
  __shared__ int end_s;
  unsigned passed = 0;
  const int lane = threadIdx.x & 31;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long wbase = tid - lane;  // first position of this warp
  const long long nthr = (long long)gridDim.x * blockDim.x;
  for (long long I0 = wbase; I0 < nb; I0 += nthr) {
    const long long I = I0 + lane;
    warp_append(I < nb && indeg[I] == 0, (int)I, order, 0, cnt + 2);
  }
  if (!grid_sync_count(gs, passed)) return;
  if (threadIdx.x == 0) end_s = ld_relaxed(cnt + 2);
  __syncthreads();
  int s = 0, e = end_s;
  if (tid == 0) {
    lvl_ptr[0] = 0;
    lvl_ptr[1] = e;
  }
  for (int l = 0;; ++l) {
    if (s == e) {
      if (tid == 0) *nlev = l;
      grid_exit_count(gs);
      return;
    }
    if (tid == 0) atomicExch(cnt + (l + 1) % 3, 0);
    int* count = cnt + l % 3;
    for (long long q0 = s + wbase; q0 < e; q0 += nthr) {
      const long long q = q0 + lane;
      const int I = q < e ? __ldcg(order + q) : -1;
      int p = I >= 0 ? __ldg(sptr + I) : 0;
      const int pe = I >= 0 ? __ldg(sptr + I + 1) : 0;
      while (__any_sync(FULL, p < pe)) {
        bool ready = false;
        int J = -1;
        if (p < pe) {
          J = __ldg(sidx + p);
          ready = atomicSub(indeg + J, 1) == 1;
          ++p;
        }
        warp_append(ready, J, order, e, count);
      }
    }
    if (!grid_sync_count(gs, passed)) return;
    if (threadIdx.x == 0) end_s = e + ld_relaxed(count);
    __syncthreads();
    s = e;
    e = end_s;
    if (tid == 0) lvl_ptr[l + 2] = e;
  }
}

constexpr int kLvlThreads = 256;

// Warp rank for level work.  Consecutive ranks sit in different CTAs (the
// CTAs of a co-resident launch are spread over the SMs), so a level narrower
// than the grid is spread over every SM instead of filling the first CTAs'
// warps while the other SMs wait at the barrier.  Within a CTA, which warp
// serves which round of ranks is rotated by the CTA's slot on its SM, so
// that the CTAs sharing an SM start on different sub-partitions: each of
// the four has its own FP64 unit, about 80 cycles per warp instruction
// whatever the number of active lanes.  The slot comes from a per-SM
// counter that is never reset (consecutive CTAs on one SM get consecutive
// values); any rotation is a permutation of the CTA's warps, so only the
// spread, not the set of ranks, depends on it.  Called by every thread of
// the CTA before any of them returns.
__device__ unsigned g_sm_slot[1024];

__device__ __forceinline__ int spread_warp(int per_sm) {
  __shared__ int rot_s;
  const int nwc = (int)(blockDim.x >> 5);
  if (threadIdx.x == 0) {
    unsigned sm;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    const int c = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
    const int k = (int)(atomicAdd(&g_sm_slot[sm & 1023u], 1u) % (unsigned)c);
    rot_s = (k * (4 / c)) % nwc;  // per_sm 2: warps 0 and 2 open the rounds
  }
  __syncthreads();
  const int round = ((int)(threadIdx.x >> 5) - rot_s + nwc) % nwc;
  return (int)(round * gridDim.x + blockIdx.x);
}
// rows with more dependencies than this make the level kernels give each
// row a whole warp instead of a bs-lane group
constexpr int kLongRow = 32;
// Level analysis recommendations (measured on GB300, stencil and power-law
// systems).  Solves: the level order (flow kernel) when no row has more than
// kFlowMaxDeps dependencies, whatever the level width (it was 4-10x faster
// than the sync-free kernel on 2D and 3D stencils down to 32 rows per
// level), the sync-free kernel otherwise (a lane group walks a long row's
// dependencies one after the other).  BILU(0): the level order (a barrier
// per level) when a level holds at least kFactorLevelWidth rows on average
// and no row has more than kLongRow dependencies, sync-free otherwise.
constexpr int kFlowMaxDeps = 8;
constexpr int kFactorLevelWidth = 4096;

// Rows of the flow schedule: a group of BS lanes per block row (32/BS rows
// per warp; lane r of a group owns scalar row r).  On GB300 an FP64 warp
// instruction costs the same whatever the number of active lanes, so packing
// rows is what makes the per-row FP64 work small; rows of one level are
// independent, so groups of a warp never wait on each other.
//
// A row's critical path is its x reads (rows of earlier levels) and a short
// FP64 chain; everything else is loaded ahead in three stages.  While one
// row is solved, a group holds: the index of its row after next (read from
// the level order), the row pointers and diagonal position of its next row
// (issued before the current row's arithmetic), and, issued right after it,
// the next row's first D column indices and blocks, its diagonal row and b.
// The x reads of those D blocks are then independent of each other.
// T: the arithmetic and storage type of the solve (double, or float for
// the FP32-stored factor of the mixed exact-ILU apply).
template <int BS, class T>
struct GRowPre {
  // blocks held in registers (bs 8: one, within the register budget)
  static constexpr int D = BS <= 5 ? 16 / BS : 1;
  int I, ps, pe;   // I < 0: no row for this group
  int K[D];        // columns of the first D dependencies (-1 past the row)
  T a[D][BS];      // row r of those blocks
  T dq[BS];        // row r of the diagonal block
  T bq;            // b_r
  T rq;            // 1 / pivot of row r, when the factorisation stored it
};

// structural words of row I: dependency range and diagonal position
struct GRowMeta {
  int rs, re, dI;
};

__device__ __forceinline__ void grow_meta(int I, const int* __restrict__ row,
                                          const int* __restrict__ diag, GRowMeta& m) {
  m.rs = m.re = m.dI = 0;
  if (I < 0) return;
  m.rs = __ldg(row + I);
  m.re = __ldg(row + I + 1);
  m.dI = __ldg(diag + I);
}

template <int BS, bool LOWER, class T>
__device__ __forceinline__ void grow_load(int I, const GRowMeta& m, const int* __restrict__ col,
                                          const T* __restrict__ val, const T* __restrict__ b,
                                          const T* __restrict__ rdiag, GRowPre<BS, T>& p) {
  constexpr int BS2 = BS * BS, D = GRowPre<BS, T>::D;
  const int r = (threadIdx.x & 31) % BS;
  p.I = I;
  p.ps = LOWER ? m.rs : m.dI + 1;
  p.pe = LOWER ? m.dI : m.re;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const int q = p.ps + j;
    const bool has = I >= 0 && q < p.pe;
    p.K[j] = has ? __ldg(col + q) : -1;
    const T* blk = val + (long long)(has ? q : 0) * BS2 + r * BS;
#pragma unroll
    for (int c = 0; c < BS; ++c) p.a[j][c] = has ? __ldg(blk + c) : T(0);
  }
  if (I < 0) return;
  const T* Dg = val + (long long)m.dI * BS2 + r * BS;
#pragma unroll
  for (int c = 0; c < BS; ++c) p.dq[c] = __ldg(Dg + c);
  p.bq = __ldg(b + (long long)I * BS + r);
  p.rq = (!LOWER && rdiag) ? __ldg(rdiag + (long long)I * BS + r) : T(0);
}

template <int BS, bool LOWER, class T>
__device__ __forceinline__ void grow_prefetch(int I, const int* __restrict__ row,
                                              const int* __restrict__ col,
                                              const int* __restrict__ diag,
                                              const T* __restrict__ val, const T* __restrict__ b,
                                              const T* __restrict__ rdiag, GRowPre<BS, T>& p) {
  GRowMeta m;
  grow_meta(I, row, diag, m);
  grow_load<BS, LOWER, T>(I, m, col, val, b, rdiag, p);
}

// Level-scheduled solve for rows with long dependency lists (more than
// kLongRow blocks): a warp per row, the slots of the warp summing the row's
// blocks as in the sync-free kernel (bit-identical x), a counting grid
// barrier after each level.  The first row of a warp's next level is
// loaded before the barrier.
template <int BS, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(kLvlThreads, 2) k_sptrsv_levels(
    const int* __restrict__ row, const int* __restrict__ col, const int* __restrict__ diag,
    const double* __restrict__ val, const double* __restrict__ b, double* x,
    const int* __restrict__ order, const int* __restrict__ lvl_ptr, const int* __restrict__ nlev_p,
    SyncState ss, GridSync gs) {
  unsigned passed = 0;
  const int warp = spread_warp(gs.per_sm);
  const int nw = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const int nlev = __ldg(nlev_p);
  if (nlev <= 0) return;
  RowPre<BS> wp;
  {
    int t = __ldg(lvl_ptr) + warp;
    sptrsv_prefetch<BS, LOWER, UNIT>(t < __ldg(lvl_ptr + 1) ? __ldg(order + t) : -1, row, col,
                                     diag, val, b, wp);
  }
  for (int l = 0; l < nlev; ++l) {
    const int s = __ldg(lvl_ptr + l), e = __ldg(lvl_ptr + l + 1);
    if (wp.I >= 0) sptrsv_finish<BS, LOWER, UNIT, false, false>(wp, col, val, x, ss);
    for (int t = s + warp + nw; t < e; t += nw) {
      RowPre<BS> q;
      sptrsv_prefetch<BS, LOWER, UNIT>(__ldg(order + t), row, col, diag, val, b, q);
      sptrsv_finish<BS, LOWER, UNIT, false, false>(q, col, val, x, ss);
    }
    if (l + 1 < nlev) {
      int t = e + warp;
      sptrsv_prefetch<BS, LOWER, UNIT>(t < __ldg(lvl_ptr + l + 2) ? __ldg(order + t) : -1, row,
                                       col, diag, val, b, wp);
      if (!grid_sync_count(gs, passed)) return;
    }
  }
  grid_exit_count(gs);
}

// ------------------------------------------------------------------ flow schedule
// Level-order solve without grid barriers.  Every group keeps the rows the
// level schedule gives it (the same static assignment and the same
// arithmetic as k_sptrsv_levels), but instead of meeting the whole grid at
// a barrier after each level it waits only for the x entries its row reads.
// x is self-flagging: before the launch every entry holds a signalling-NaN
// pattern (XBits::kPending); a row's entries are written once, each with a
// single 64-bit (FP32 solve: 32-bit) store, and floating-point arithmetic
// only ever yields quiet NaNs, so an entry that no longer reads the pattern
// holds its final value and no flag, fence or barrier is needed.  Each dependent entry is read with a strong
// (L2) load; a pending one is polled with bounded back-off.  All warps are
// co-resident (cooperative launch) and each processes its rows in level
// order, so every wait ends: rows of level 0 wait for nothing, rows of
// level l only for rows of lower levels.  The solve then advances as a
// wavefront at the latency of one dependency chain per level rather than
// at that of the slowest CTA plus a grid barrier.
// Bit patterns of x entries: kPending (a signalling NaN) and the quiet NaN
// stored instead of a result that happened to carry the pending pattern.
template <class T>
struct XBits;
template <>
struct XBits<double> {
  using U = unsigned long long;
  static constexpr U kPending = 0x7FF0A5A5A5A5A5A5ull;
  static constexpr U kQuiet = 0x7FF8000000000000ull;
};
template <>
struct XBits<float> {
  using U = unsigned;
  static constexpr U kPending = 0x7FA5A5A5u;
  static constexpr U kQuiet = 0x7FC00000u;
};
constexpr int kFlowSpin = 64;  // polling rounds without sleeping

__device__ __forceinline__ unsigned long long ld_strong_bits(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ unsigned ld_strong_bits(const float* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double from_bits(unsigned long long u, double) {
  return __longlong_as_double((long long)u);
}
__device__ __forceinline__ float from_bits(unsigned u, float) { return __uint_as_float(u); }

// Stores a computed entry; a value with the pending pattern (impossible
// for an arithmetic result) would be stored as the canonical quiet NaN.
__device__ __forceinline__ void st_strong(double* p, double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  if (u == XBits<double>::kPending) u = XBits<double>::kQuiet;
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(u));
}
__device__ __forceinline__ void st_strong(float* p, float v) {
  unsigned u = __float_as_uint(v);
  if (u == XBits<float>::kPending) u = XBits<float>::kQuiet;
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(u));
}

// Re-reads the entries of u[] that are still pending (x entries of rows of
// earlier levels that other warps are computing) until none is: the first
// kFlowSpin rounds back to back (most waits end within a few hundred
// nanoseconds, and a sleep, however short it is asked to be, was measured to
// cost more than that on GB300), then with bounded back-off.  u[j * BS + c] is entry c of block row K[j] (absent
// dependencies have K[j] < 0 and u = 0, never pending).  The addresses are
// rebuilt from K each round (through an opaque move, so the compiler does
// not keep D * BS addresses live across the loop).  Per lane, no warp
// collectives (groups of a warp wait for different rows).  false: the
// launch aborted.
template <int BS, int D, class T>
__device__ __forceinline__ bool poll_pending(typename XBits<T>::U (&u)[D * BS], const int (&K)[D],
                                             const T* x, const SyncState& ss) {
  constexpr typename XBits<T>::U kP = XBits<T>::kPending;
  bool pend = false;
#pragma unroll
  for (int i = 0; i < D * BS; ++i) pend |= u[i] == kP;
  long long n = 0;
  unsigned ns = 32;
  while (pend) {
    if (n >= kFlowSpin) backoff(ns);
    pend = false;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      int k;
      asm volatile("mov.b32 %0, %1;" : "=r"(k) : "r"(K[j]));
      const T* xk = x + (long long)k * BS;
#pragma unroll
      for (int c = 0; c < BS; ++c) {
        if (u[j * BS + c] == kP) {
          u[j * BS + c] = ld_strong_bits(xk + c);
          pend |= u[j * BS + c] == kP;
        }
      }
    }
    if (!pend) break;
    if (++n > ss.spin) {
      atomicCAS(ss.err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    if ((n & 31) == 0 && ld_relaxed(ss.err) != 0) return false;
  }
  return true;
}

// grow_finish with waits on the entries read; the same operations in the
// same order, in T.  y64 (optional): x is also stored there as FP64 (the
// FP32 solve's output in the precision its consumer wants).  Called by all
// 32 lanes; false in every lane if the launch aborted.
template <int BS, bool LOWER, bool UNIT, class T>
__device__ __forceinline__ bool grow_finish_flow(const GRowPre<BS, T>& p,
                                                 const int* __restrict__ col,
                                                 const T* __restrict__ val, T* x, double* y64,
                                                 bool have_rq, const SyncState& ss) {
  constexpr int BS2 = BS * BS, D = GRowPre<BS, T>::D;
  using U = typename XBits<T>::U;
  const int lane = threadIdx.x & 31, r = lane % BS, gb = lane - r;
  T tot = T(0), rq = T(1);
  bool ok = true;
  if (p.I >= 0) {
    T d = p.dq[0];
#pragma unroll
    for (int c = 1; c < BS; ++c)
      if (c == r) d = p.dq[c];
    // entries of absent dependencies read as 0 (never pending)
    U u[D * BS];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const T* xk = x + (long long)(p.K[j] >= 0 ? p.K[j] : 0) * BS;
#pragma unroll
      for (int c = 0; c < BS; ++c) u[j * BS + c] = p.K[j] >= 0 ? ld_strong_bits(xk + c) : U(0);
    }
    if (!UNIT) rq = have_rq ? p.rq : T(1) / d;  // overlaps the x reads
    ok = poll_pending<BS, D, T>(u, p.K, x, ss);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      if (p.K[j] >= 0) {
        T sp = T(0);
#pragma unroll
        for (int c = 0; c < BS; ++c) sp = fma(p.a[j][c], from_bits(u[j * BS + c], T()), sp);
        tot += sp;
      }
    }
    for (int q = p.ps + D; ok && q < p.pe; ++q) {
      const int K = __ldg(col + q);
      const T* blk = val + (long long)q * BS2 + r * BS;
      const T* xq = x + (long long)K * BS;
      U uq[BS];
#pragma unroll
      for (int c = 0; c < BS; ++c) uq[c] = ld_strong_bits(xq + c);
      const int Kq[1] = {K};
      ok = poll_pending<BS, 1, T>(uq, Kq, x, ss);
      T sp = T(0);
#pragma unroll
      for (int c = 0; c < BS; ++c) sp = fma(__ldg(blk + c), from_bits(uq[c], T()), sp);
      tot += sp;
    }
  }
  if (__any_sync(FULL, !ok)) return false;
  T v = p.bq - tot, xr = T(0);
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const int c = LOWER ? k : BS - 1 - k;
    T mine = (UNIT || r != c) ? v : v * rq;
    T xc = __shfl_sync(FULL, mine, (gb + c) & 31);
    if (r == c) xr = xc;
    if (LOWER ? (r > c) : (r < c)) v -= p.dq[c] * xc;
  }
  if (p.I >= 0 && p.I != ss.withhold) {
    st_strong(x + (long long)p.I * BS + r, xr);
    if (y64) y64[(long long)p.I * BS + r] = (double)xr;
  }
  return true;
}

// Row cursor of a warp in the flow kernel: level l and the position t0 of
// group 0's row in the level order.  Pass 0 of every level is visited, also
// where the warp has no row (a cheap skip); further passes of a wide level
// follow while group 0's position is inside the level.
struct RowCursor {
  int l;
  long long t0;
};

__device__ __forceinline__ void cursor_next(RowCursor& c, int nlev, long long first,
                                            long long ngrp, const int* __restrict__ lvl_ptr) {
  if (c.l >= nlev) return;
  c.t0 += ngrp;
  if (c.t0 >= __ldg(lvl_ptr + c.l + 1)) {
    ++c.l;
    c.t0 = c.l < nlev ? __ldg(lvl_ptr + c.l) + first : 0;
  }
}

__device__ __forceinline__ int cursor_row(const RowCursor& c, int g, bool active, int nlev,
                                          const int* __restrict__ order,
                                          const int* __restrict__ lvl_ptr) {
  if (!active || c.l >= nlev) return -1;
  const long long t = c.t0 + g;
  return t < __ldg(lvl_ptr + c.l + 1) ? __ldg(order + t) : -1;
}

// One row per group and iteration.  The rows ahead of the cursor are staged
// so that nothing but x is read on a row's critical path: the next row's
// blocks, diagonal row and b are loaded before the current row waits, the
// structure of the row after it (row pointers, diagonal position) and the
// index of the one after that one step earlier still.  Two staged rows
// need about 180 registers a thread, so one 256-thread CTA runs per SM (two
// warps a sub-partition; more warps only queue on its FP64 unit).
template <int BS, bool LOWER, bool UNIT, class T>
__global__ void __launch_bounds__(kLvlThreads, 1) k_sptrsv_flow(
    const int* __restrict__ row, const int* __restrict__ col, const int* __restrict__ diag,
    const T* __restrict__ val, const T* __restrict__ b, T* x, double* y64,
    const T* __restrict__ rdiag_in, const int* __restrict__ order,
    const int* __restrict__ lvl_ptr, const int* __restrict__ nlev_p, SyncState ss, int per_sm) {
  constexpr int G = 32 / BS;
  const int g = (threadIdx.x & 31) / BS;
  const int warp = spread_warp(per_sm);
  const int nw = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const long long ngrp = (long long)nw * G;
  const long long first = (long long)warp * G;
  const int nlev = __ldg(nlev_p);
  if (nlev <= 0) return;
  const bool active = g < G;
  const T* rdiag = LOWER ? nullptr : rdiag_in;
  RowCursor c0{0, __ldg(lvl_ptr) + first};
  RowCursor c1 = c0;
  cursor_next(c1, nlev, first, ngrp, lvl_ptr);
  RowCursor c2 = c1;
  cursor_next(c2, nlev, first, ngrp, lvl_ptr);
  RowCursor c3 = c2;
  cursor_next(c3, nlev, first, ngrp, lvl_ptr);
  GRowPre<BS, T> pre;
  grow_prefetch<BS, LOWER, T>(cursor_row(c0, g, active, nlev, order, lvl_ptr), row, col, diag, val,
                           b, rdiag, pre);
  int I1 = cursor_row(c1, g, active, nlev, order, lvl_ptr);
  GRowMeta m1;
  grow_meta(I1, row, diag, m1);
  int I2 = cursor_row(c2, g, active, nlev, order, lvl_ptr);
  while (c0.l < nlev) {
    // loads for the rows ahead first: they do not depend on x
    GRowPre<BS, T> nxt;
    if (c1.l < nlev) grow_load<BS, LOWER, T>(I1, m1, col, val, b, rdiag, nxt);
    GRowMeta m2;
    grow_meta(I2, row, diag, m2);
    const int I3 = cursor_row(c3, g, active, nlev, order, lvl_ptr);
    if (!grow_finish_flow<BS, LOWER, UNIT, T>(pre, col, val, x, y64, rdiag != nullptr, ss))
      return;
    pre = nxt;
    m1 = m2;
    I1 = I2;
    I2 = I3;
    c0 = c1;
    c1 = c2;
    c2 = c3;
    cursor_next(c3, nlev, first, ngrp, lvl_ptr);
  }
}

template <class T>
__global__ void k_fill_pending(typename XBits<T>::U* x, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = XBits<T>::kPending;
}

// ------------------------------------------------------------------ BILU(0)
// Scalar ILU(0) on the block pattern in IKJ order, blockwise:
//   for K < I in row I:  L_IK = A_IK U_KK^-1 (row-wise forward elimination),
//                        A_IJ -= L_IK U_KJ for J > K present in rows I and K;
//   then LU of the diagonal block (no pivoting) and U_IJ = L_II^-1 A_IJ.
// Each element sees the same sequence of a -= l*u updates as the scalar IKJ
// loop, with ascending k.  Multipliers are formed as a * (1 / u_kk): each
// row stores the reciprocals of its BS pivots once (SyncState::rdiag) and
// the rows below it multiply by them, so a row costs BS FP64 divisions
// instead of BS per dependency plus BS(BS-1)/2 (a division is a chain of
// FP64 instructions, each ~80 cycles of a sub-partition's FP64 unit on
// GB300).  The factor differs from the divided one by rounding only.
//
// One block row with a group of BS lanes (level schedule: rows of one level
// are independent, so groups of a warp never wait on each other; the
// group's shuffles and ballots use its own lane mask).  Lane r of the group
// owns scalar row r of L_IK and of the updates, and column r of the
// diagonal LU and of the U blocks.  Phase 2 takes its candidates from the
// shorter of the two column lists (power-law hub rows hold thousands of
// blocks), BS at a time, each lane binary-searching one in the other list;
// every block is updated once per K, so the update order of each element
// does not depend on which list is scanned.
// LU without pivoting of a diagonal block, right-looking, in the registers
// of a group of BS lanes: lane c holds column c (dc[q] = D[q][c]) on entry
// and the packed L\U column on exit.  Step k takes the reciprocal of the
// final pivot u_kk on lane k, scales the rest of column k into the
// multipliers l_qk = d_qk * (1 / u_kk), broadcasts them and updates the
// columns right of it.  Each element receives its updates in ascending k,
// as in the scalar IKJ loop.  Returns 1 / u_cc on lane c (the reciprocal
// pivots that later rows and the upper solves multiply by).
template <int BS>
__device__ __forceinline__ double bilu0_diag_lu(double (&dc)[BS], int c, unsigned gmask, int gb) {
  double rp = 0.0;
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const double rk = 1.0 / dc[k];  // meaningful on lane k
    if (c == k) rp = rk;
#pragma unroll
    for (int q = k + 1; q < BS; ++q) {
      const double l = __shfl_sync(gmask, dc[q] * rk, gb + k);
      if (c == k) dc[q] = l;
      else if (c > k) dc[q] -= l * dc[k];
    }
  }
  return rp;
}

// The same LU by a whole warp: lane (c, j) holds rows j + m PL of column c
// (PL lanes per column, so BS 8 keeps two rows a lane instead of eight on
// a lane per column).  Step k broadcasts the reciprocal pivot from the lane
// holding u_kk and row k of each column from the lane holding it; slots
// whose rows are all <= k are skipped at compile time.  Every element
// receives the operations of bilu0_diag_lu in the same order.  On the lane
// (c, c % PL): rp = 1 / u_cc and piv = u_cc.  Lanes outside the block take
// part in the shuffles only.
template <int BS, int PL>
__device__ __forceinline__ void bilu0_diag_lu_warp(double (&d)[(BS + PL - 1) / PL], int c, int j,
                                                   double& rp, double& piv) {
  constexpr int PC = (BS + PL - 1) / PL;
  rp = 0.0;
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const int mk = k / PL, jk = k - mk * PL;
    // only the pivot's lane divides a block entry (a zero elsewhere would
    // send its lane down the division's slow path)
    const bool at_pivot = c == k && j == jk;
    const double rk = __shfl_sync(FULL, 1.0 / (at_pivot ? d[mk] : 1.0), k * PL + jk);
    if (at_pivot) rp = rk;
    const double dkc = __shfl_sync(FULL, d[mk], (c * PL + jk) & 31);  // d[k][c]
#pragma unroll
    for (int m = 0; m < PC; ++m) {
      if (m * PL + PL - 1 <= k) continue;  // every row of slot m is final
      const int q = j + m * PL;
      const double l = __shfl_sync(FULL, d[m] * rk, k * PL + j);  // l_qk from column k
      if (q > k && q < BS) {
        if (c == k) d[m] = l;
        else if (c > k && c < BS) d[m] -= l * dkc;
      }
    }
  }
  piv = d[0];
#pragma unroll
  for (int m = 1; m < PC; ++m)
    if (m == c / PL) piv = d[m];
}

// Structure of a block row and of its first dependency (pattern only: read
// ahead of the values, before the level's barrier).
struct BRowPre {
  int I;               // < 0: no row
  int rs, re, dI;      // row pointers and diagonal position
  int K, dK, ke;       // first dependency: column, its diagonal position, its row end
  int m0, m1;          // its match list [m0, m1) when the lists were built
};

__device__ __forceinline__ void brow_prefetch(int I, const int* __restrict__ row,
                                              const int* __restrict__ col,
                                              const int* __restrict__ diag,
                                              const int* __restrict__ mptr, BRowPre& p) {
  p.I = I;
  p.rs = p.re = p.dI = p.K = p.dK = p.ke = p.m0 = p.m1 = 0;
  if (I < 0) return;
  p.rs = __ldg(row + I);
  p.re = __ldg(row + I + 1);
  p.dI = __ldg(diag + I);
  if (p.rs < p.dI) {
    p.K = __ldg(col + p.rs);
    p.dK = __ldg(diag + p.K);
    p.ke = __ldg(row + p.K + 1);
    if (mptr) {
      p.m0 = __ldg(mptr + p.rs);
      p.m1 = __ldg(mptr + p.rs + 1);
    }
  }
}

// mptr / mpair (optional): the match lists of k_bilu0_match_fill, which
// take the searches of phase 2 out of the row's dependency chain; the
// updates and their arithmetic are the same either way.
template <int BS>
__device__ __forceinline__ void bilu0_grow(const BRowPre& pr, const int* __restrict__ row,
                                           const int* __restrict__ col,
                                           const int* __restrict__ diag, double* val,
                                           const SyncState& ss, unsigned gmask, int r, int gb,
                                           const int* __restrict__ mptr,
                                           const int2* __restrict__ mpair) {
  constexpr int BS2 = BS * BS;
  const int I = pr.I, rs = pr.rs, re = pr.re, dI = pr.dI;
  // structure of the next dependency, loaded one step ahead
  int Kn = pr.K, dKn = pr.dK, ken = pr.ke;
  int ms = pr.m0, men = pr.m1;
  for (int pk = rs; pk < dI; ++pk) {
    const int K = Kn, dK = dKn, ke = ken;
    const int me = men;
    if (pk + 1 < dI) {
      Kn = __ldg(col + pk + 1);
      dKn = __ldg(diag + Kn);
      ken = __ldg(row + Kn + 1);
      if (mptr) men = __ldg(mptr + pk + 2);
    }
    // the first match's positions load beside phase 1's operands
    int2 mfirst = make_int2(0, 0);
    if (mptr && ms < me) mfirst = __ldg(mpair + ms);
    double* L = val + (long long)pk * BS2;
    const double* Ukk = val + (long long)dK * BS2;
    const double* rK = ss.rdiag + (long long)K * BS;  // 1 / pivots of U_KK
    // phase 1: row r of L_IK = A_IK U_KK^-1 (forward elimination)
    double a[BS];
#pragma unroll
    for (int c = 0; c < BS; ++c) a[c] = L[r * BS + c];
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      a[k] = a[k] * __ldcg(rK + k);
#pragma unroll
      for (int c = k + 1; c < BS; ++c) a[c] -= a[k] * __ldcg(Ukk + k * BS + c);
    }
#pragma unroll
    for (int c = 0; c < BS; ++c) L[r * BS + c] = a[c];
    // phase 2: A_IJ -= L_IK U_KJ for J > K in rows I and K
    if (mptr) {
      for (int q = ms; q < me; ++q) {
        const int2 m = q == ms ? mfirst : __ldg(mpair + q);
        double* Aij = val + (long long)m.x * BS2 + r * BS;
        const double* Ukj = val + (long long)m.y * BS2;
#pragma unroll
        for (int c = 0; c < BS; ++c) {
          double v = Aij[c];
#pragma unroll
          for (int k = 0; k < BS; ++k) v -= a[k] * __ldcg(Ukj + k * BS + c);
          Aij[c] = v;
        }
      }
      ms = me;
      continue;
    }
    // without match lists the shorter column list supplies the candidates,
    // BS at a time, searched for in the other
    const bool from_i = (re - pk - 1) <= (ke - dK - 1);
    const int cs = from_i ? pk + 1 : dK + 1, ce = from_i ? re : ke;
    const int ss_ = from_i ? dK + 1 : pk + 1, se = from_i ? ke : re;
    for (int c0 = cs; c0 < ce; c0 += BS) {
      int pc = c0 + r, other = -1;
      if (pc < ce) other = find_in_row(col, ss_, se, __ldg(col + pc));
      unsigned found = (__ballot_sync(gmask, other >= 0) >> gb) & ((1u << BS) - 1u);
      while (found) {
        const int bit = __ffs(found) - 1;
        found &= found - 1;
        const int o = __shfl_sync(gmask, other, gb + bit);
        const int pj = from_i ? c0 + bit : o, pos = from_i ? o : c0 + bit;
        double* Aij = val + (long long)pj * BS2 + r * BS;
        const double* Ukj = val + (long long)pos * BS2;
#pragma unroll
        for (int c = 0; c < BS; ++c) {
          double v = Aij[c];
#pragma unroll
          for (int k = 0; k < BS; ++k) v -= a[k] * __ldcg(Ukj + k * BS + c);
          Aij[c] = v;
        }
      }
    }
  }
  __syncwarp(gmask);
  // diagonal block, lane c = r owns column c: bilu0_diag_lu
  double* D = val + (long long)dI * BS2;
  double dc[BS];
#pragma unroll
  for (int q = 0; q < BS; ++q) dc[q] = D[q * BS + r];
  const double rp = bilu0_diag_lu<BS>(dc, r, gmask, gb);
  double piv = dc[0];  // this lane's diagonal element of U_II
#pragma unroll
  for (int q = 1; q < BS; ++q)
    if (q == r) piv = dc[q];
  if (piv == 0.0) atomicMin(ss.zp, I);
#pragma unroll
  for (int q = 0; q < BS; ++q) D[q * BS + r] = dc[q];
  ss.rdiag[(long long)I * BS + r] = rp;
  __syncwarp(gmask);
  // U blocks right of the diagonal: U_IJ = L_II^-1 A_IJ, lane per column
  for (int pj = dI + 1; pj < re; ++pj) {
    double* U = val + (long long)pj * BS2;
    double u[BS];
#pragma unroll
    for (int q = 0; q < BS; ++q) u[q] = U[q * BS + r];
#pragma unroll
    for (int q = 1; q < BS; ++q)
#pragma unroll
      for (int k = 0; k < q; ++k) u[q] -= D[q * BS + k] * u[k];
#pragma unroll
    for (int q = 1; q < BS; ++q) U[q * BS + r] = u[q];
  }
}

// One block row with a whole warp (the sync-free factorisation, used for
// matrices with long rows or narrow levels).  WAIT: the rows K it reads may
// still be in progress and are waited for through their flags.  Phase 1 by
// the whole warp (PL lanes per row of L_IK), or for runs of dependencies
// without updates by a lane group each; phase 2 with teams of lanes per
// updated block; the diagonal LU by the whole warp; U blocks with 32/BS
// blocks per pass.  The same operations per element as bilu0_grow.
// Returns false if the launch aborted.
// Column index p of row I (rs = first position of the row): from the
// shared-memory copy when the row was staged there.
__device__ __forceinline__ int row_col(const int* __restrict__ col, const int* stage, int rs,
                                       int p) {
  return stage ? stage[p - rs] : __ldg(col + p);
}

// Binary search for key among positions [s, e) of row I (staged or not).
__device__ __forceinline__ int find_in_row_staged(const int* __restrict__ col, const int* stage,
                                                  int rs, int s, int e, int key) {
  int lo = s, hi = e - 1;
  while (lo <= hi) {
    int m = (lo + hi) >> 1;
    int v = row_col(col, stage, rs, m);
    if (v == key) return m;
    if (v < key) lo = m + 1; else hi = m - 1;
  }
  return -1;
}

constexpr int kRowStage = 2048;  // column indices of a long row kept in shared memory

__device__ __forceinline__ unsigned dynamic_smem_bytes() {
  unsigned v;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
  return v;
}

// Wait of a group of lanes (gmask) on one flag: the group's lanes read the
// same word; bounded like warp_wait.
__device__ __forceinline__ bool group_wait(const int* flag, int* err, long long spin,
                                           unsigned gmask, bool leader) {
  long long n = 0;
  unsigned ns = 32;
  while (true) {
    const int v = ld_relaxed(flag);
    if (__all_sync(gmask, v != 0)) {
      fence_acquire();
      return true;
    }
    if (__any_sync(gmask, ld_relaxed(err) != 0)) return false;
    if (++n > spin) {
      if (leader) atomicCAS(err, 0, (int)BILU_ERR_TIMEOUT);
      return false;
    }
    backoff(ns);
  }
}

// Phase 1 of a run of dependencies of row I: positions pk, pk+1, ... (at
// most 32 / BS of them, all before the diagonal) whose match count is 0,
// so that none of them updates a block another one reads.  Group q of BS
// lanes takes position pk + q, waits for its row K and computes
// L_IK = A_IK U_KK^-1 with lane r owning row r, the same operations per
// element in the same order as the warp-wide step.  A hub row of a
// power-law matrix has about a thousand such dependencies, which one warp
// would otherwise take one after another on the critical path.  Returns
// how many positions were taken (0 if fewer than two qualify), -1 if a
// wait gave up.
template <int BS, bool WAIT>
__device__ __forceinline__ int bilu0_run_phase1(int pk, int dI, int rs,
                                                const int* __restrict__ col, const int* stage,
                                                const int* __restrict__ diag, double* val,
                                                const SyncState& ss) {
  constexpr int G = 32 / BS, BS2 = BS * BS;
  const int lane = threadIdx.x & 31, q = lane / BS, r = lane - q * BS;
  const int p = pk + q;
  const bool mine = q < G && p < dI && __ldg(ss.nmatch + p) == 0;
  const unsigned lead = __ballot_sync(FULL, mine && r == 0);
  int take = 0;  // the run of qualifying groups from group 0
  while (take < G && ((lead >> (take * BS)) & 1u)) ++take;
  if (take < 2) return 0;
  bool ok = true;
  if (q < take) {
    const unsigned gmask = ((1u << BS) - 1u) << (q * BS);
    const int K = row_col(col, stage, rs, p);
    const int dK = __ldg(diag + K);
    if (WAIT) ok = group_wait(ss.flags + K, ss.err, ss.spin, gmask, r == 0);
    if (ok) {
      double* L = val + (long long)p * BS2;
      const double* Ukk = val + (long long)dK * BS2;
      const double* rK = ss.rdiag + (long long)K * BS;
      double a[BS];
#pragma unroll
      for (int c = 0; c < BS; ++c) a[c] = L[r * BS + c];
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        a[k] = a[k] * __ldcg(rK + k);
#pragma unroll
        for (int c = k + 1; c < BS; ++c) a[c] -= a[k] * __ldcg(Ukk + k * BS + c);
      }
#pragma unroll
      for (int c = 0; c < BS; ++c) L[r * BS + c] = a[c];
    }
  }
  if (!__all_sync(FULL, ok)) return -1;
  __syncwarp();
  return take;
}

template <int BS, bool WAIT>
__device__ __forceinline__ bool bilu0_wrow(int I, const int* __restrict__ row,
                                          const int* __restrict__ col,
                                          const int* __restrict__ diag, double* val,
                                          const SyncState& ss, int* stage_buf) {
  constexpr int BS2 = BS * BS;
  constexpr int EPL = BS2 > 32 ? 2 : 1;
  constexpr int TL = BS2 / EPL + (BS2 % EPL ? 1 : 0);
  constexpr int TPW = 32 / TL;         // blocks updated per pass in phase 2
  constexpr int SPAN = 32 / TPW;
  constexpr int GU = 32 / BS;          // U blocks per pass (lane = column)
  constexpr int PL = 32 / BS < BS ? 32 / BS : BS;  // phase 1: lanes per row
  constexpr int PC = (BS + PL - 1) / PL;           // phase 1: columns per lane
  int lane = threadIdx.x & 31;
  int team = lane / SPAN, tl = lane - team * SPAN;
  bool team_on = team < TPW && tl < TL;
  const int pr = lane / PL, pj = lane - pr * PL;
  const bool p_on = pr < BS;
  int rs = __ldg(row + I), re = __ldg(row + I + 1), dI = __ldg(diag + I);
  // a hub row searches its own column list once per K: keep it in shared
  // memory (one L2 round trip per search step otherwise)
  const int* stage = nullptr;
  if (stage_buf && re - rs > 64 && re - rs <= kRowStage) {
    for (int t = lane; t < re - rs; t += 32) stage_buf[t] = __ldg(col + rs + t);
    __syncwarp();
    stage = stage_buf;
  }
  for (int pk = rs; pk < dI; ++pk) {
    // a run of dependencies that update no block beyond their own L_IK
    // (match count 0) is independent inside the row: a lane group each
    if (ss.nmatch && dI - pk >= 2) {
      const int took = bilu0_run_phase1<BS, WAIT>(pk, dI, rs, col, stage, diag, val, ss);
      if (took < 0) return false;
      if (took > 0) {
        pk += took - 1;
        continue;
      }
    }
    const int K = row_col(col, stage, rs, pk);
    const int dK = __ldg(diag + K), ke = __ldg(row + K + 1);
    const int nm = ss.nmatch ? __ldg(ss.nmatch + pk) : 1;
    // sync-free schedule: row K may still be in progress
    if (WAIT && !warp_wait(ss.flags + K, ss.err, ss.spin)) return false;
    double* L = val + (long long)pk * BS2;
    const double* Ukk = val + (long long)dK * BS2;
    const double* rK = ss.rdiag + (long long)K * BS;  // 1 / pivots of U_KK
    // phase 1: row pr of L_IK = A_IK U_KK^-1 on the PL lanes of row pr,
    // lane (pr, pj) holding columns pj + m PL.  Step k scales column k by
    // the reciprocal pivot, broadcasts it along the row and updates the
    // columns right of it; slots whose columns are all <= k are skipped
    // at compile time.  Per element the same operations in the same order
    // as a lane per row, with half the FP64 instructions at BS 8 (18 per
    // dependency instead of 36).
    {
      // every operand is loaded up front, unpredicated (clamped columns):
      // loads under the lane predicates of the steps would wait one L2
      // round trip per step
      double a[PC], rkv[PC], u[BS][PC];
#pragma unroll
      for (int m = 0; m < PC; ++m) {
        const int c = pj + m * PL, cc = c < BS ? c : BS - 1;
        a[m] = (p_on && c < BS) ? L[pr * BS + c] : 0.0;
        rkv[m] = __ldcg(rK + cc);
#pragma unroll
        for (int k = 0; k < BS; ++k)
          u[k][m] = m * PL + PL - 1 <= k ? 0.0 : __ldcg(Ukk + k * BS + cc);
      }
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        const int mk = k / PL, jk = k - mk * PL;
        if (pj == jk) a[mk] = a[mk] * rkv[mk];
        const double ak = __shfl_sync(FULL, a[mk], (pr * PL + jk) & 31);
#pragma unroll
        for (int m = 0; m < PC; ++m) {
          if (m * PL + PL - 1 <= k) continue;  // every column of slot m is final
          const int c = pj + m * PL;
          if (c > k && c < BS) a[m] -= ak * u[k][m];
        }
      }
#pragma unroll
      for (int m = 0; m < PC; ++m) {
        const int c = pj + m * PL;
        if (p_on && c < BS) L[pr * BS + c] = a[m];
      }
    }
    __syncwarp();
    // phase 2: A_IJ -= L_IK U_KJ for J > K in rows I and K.  The shorter
    // of the two column lists supplies the candidates, 32 at a time, each
    // lane binary-searching one of them in the other list (hub rows of
    // power-law matrices hold thousands of blocks); then the teams update
    // the matched blocks.  Every block is updated once per K, so the
    // update order of each element is the same either way.  A dependency
    // counted as updating no block skips the searches.
    if (nm != 0) {
      const bool from_i = (re - pk - 1) <= (ke - dK - 1);
      const int cs = from_i ? pk + 1 : dK + 1, ce = from_i ? re : ke;
      const int ss_ = from_i ? dK + 1 : pk + 1, se = from_i ? ke : re;
      for (int c0 = cs; c0 < ce; c0 += 32) {
        int pc = c0 + lane, other = -1;
        if (pc < ce) {
          // candidates from row I come from the staged copy, searches in row
          // I run on it too; row K is read from global memory
          const int key = from_i ? row_col(col, stage, rs, pc) : __ldg(col + pc);
          other = from_i ? find_in_row(col, ss_, se, key)
                         : find_in_row_staged(col, stage, rs, ss_, se, key);
        }
        unsigned found = __ballot_sync(FULL, other >= 0);
        while (found) {
          // the next TPW matches go to the TPW teams
          int src = -1;
#pragma unroll
          for (int t = 0; t < TPW; ++t) {
            int bit = found ? __ffs(found) - 1 : -1;
            if (bit >= 0) found &= found - 1;
            if (t == team) src = bit;
          }
          int o = __shfl_sync(FULL, other, src < 0 ? 0 : src);
          if (team_on && src >= 0) {
            int pj = from_i ? c0 + src : o;
            int pos = from_i ? o : c0 + src;
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
      }
    }
    __syncwarp();
  }
  // diagonal block: lane (c, j) = (lane / PL, lane % PL) holds rows
  // j + m PL of column c
  double* D = val + (long long)dI * BS2;
  {
    const int c = pr, j = pj;
    double d[PC];
#pragma unroll
    for (int m = 0; m < PC; ++m) {
      const int q = j + m * PL;
      d[m] = (c < BS && q < BS) ? D[q * BS + c] : 1.0;
    }
    double rp, piv;
    bilu0_diag_lu_warp<BS, PL>(d, c, j, rp, piv);
#pragma unroll
    for (int m = 0; m < PC; ++m) {
      const int q = j + m * PL;
      if (c < BS && q < BS) D[q * BS + c] = d[m];
    }
    if (c < BS && j == c % PL) {
      if (piv == 0.0) atomicMin(ss.zp, I);
      ss.rdiag[(long long)I * BS + c] = rp;
    }
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
  return true;
}


template <int BS>
__global__ void __launch_bounds__(kLvlThreads, 2) k_bilu0_levels(
    const int* __restrict__ row, const int* __restrict__ col, const int* __restrict__ diag,
    double* val, const int* __restrict__ order, const int* __restrict__ lvl_ptr,
    const int* __restrict__ nlev_p, SyncState ss, GridSync gs, const int* __restrict__ mptr,
    const int2* __restrict__ mpair) {
  constexpr int G = 32 / BS;
  unsigned passed = 0;
  const int lane = threadIdx.x & 31, g = lane / BS, r = lane - g * BS, gb = g * BS;
  const unsigned gmask = g < G ? (((1u << BS) - 1u) << gb) : 0u;
  const int warp = spread_warp(gs.per_sm);
  const int nw = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const long long ngrp = (long long)nw * G;
  const long long mygrp = (long long)warp * G + g;
  const int nlev = __ldg(nlev_p);
  // (matrices with long rows or narrow levels take the sync-free kernel)
  // each group's first row of the next level is staged before the barrier
  BRowPre pre;
  {
    const long long t = __ldg(lvl_ptr) + mygrp;
    brow_prefetch(g < G && nlev > 0 && t < __ldg(lvl_ptr + 1) ? __ldg(order + t) : -1, row, col,
                  diag, mptr, pre);
  }
  for (int l = 0; l < nlev; ++l) {
    const int s = __ldg(lvl_ptr + l), e = __ldg(lvl_ptr + l + 1);
    if (pre.I >= 0) bilu0_grow<BS>(pre, row, col, diag, val, ss, gmask, r, gb, mptr, mpair);
    if (g < G)
      for (long long t = s + mygrp + ngrp; t < e; t += ngrp) {
        BRowPre q;
        brow_prefetch(__ldg(order + t), row, col, diag, mptr, q);
        bilu0_grow<BS>(q, row, col, diag, val, ss, gmask, r, gb, mptr, mpair);
      }
    if (l + 1 < nlev) {
      const long long t = e + mygrp;
      brow_prefetch(g < G && t < __ldg(lvl_ptr + l + 2) ? __ldg(order + t) : -1, row, col, diag,
                    mptr, pre);
      if (!grid_sync_count(gs, passed)) return;
    }
  }
  grid_exit_count(gs);
}


int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

int occupancy_per_sm(const void* fn, int threads, size_t smem = 0) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess ||
      per < 1)
    per = 1;
  return per;
}

int occupancy_grid(const void* fn, int threads, size_t smem = 0) {
  return sm_count() * occupancy_per_sm(fn, threads, smem);
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

// For every lower position pk = (I, K) of the pattern: the number of blocks
// J > K present in both rows, i.e. the blocks dependency K updates in row I
// (0 at the other positions).  Structure only and free of dependencies; the
// same shorter-list searches as the factorisation.  On graphs with few
// triangles most counts are 0, and the sync-free factorisation then skips
// those searches inside its dependency chains.
//
// Pass 1: a thread per position (its block row found by binary search over
// the row pointers, so that the thousand dependencies of a hub row spread
// over many warps), counting lists of up to kMatchSerial candidates; a
// longer list (two hub rows) is marked -1.  Pass 2: a warp per 32
// positions takes the marked ones, 32 candidates at a time.
constexpr int kMatchSerial = 32;

struct MatchLists {
  int cs, ce, s, e;  // candidates [cs, ce) searched for in positions [s, e)
  bool from_i;       // the candidates are row I's positions (else row K's)
};

__device__ __forceinline__ MatchLists match_lists(long long pk, int nb,
                                                  const int* __restrict__ row,
                                                  const int* __restrict__ col,
                                                  const int* __restrict__ diag, int& I) {
  int lo = 0, hi = nb - 1;  // last block row starting at or before pk
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(row + mid) <= pk) lo = mid; else hi = mid - 1;
  }
  I = lo;
  MatchLists m{0, 0, 0, 0, true};
  if (pk >= __ldg(diag + I)) return m;  // diagonal or upper position
  const int re = __ldg(row + I + 1);
  const int K = __ldg(col + pk), dK = __ldg(diag + K), ke = __ldg(row + K + 1);
  const bool from_i = (re - pk - 1) <= (ke - dK - 1);
  m.cs = from_i ? (int)pk + 1 : dK + 1;
  m.ce = from_i ? re : ke;
  m.s = from_i ? dK + 1 : (int)pk + 1;
  m.e = from_i ? ke : re;
  m.from_i = from_i;
  return m;
}

__global__ void __launch_bounds__(256) k_bilu0_nmatch(int nb, long long nnzb,
                                                      const int* __restrict__ row,
                                                      const int* __restrict__ col,
                                                      const int* __restrict__ diag,
                                                      int* __restrict__ nmatch) {
  const long long pk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pk >= nnzb) return;
  int I;
  const MatchLists m = match_lists(pk, nb, row, col, diag, I);
  if (m.ce - m.cs > kMatchSerial) {
    nmatch[pk] = -1;
    return;
  }
  int n = 0;
  for (int c = m.cs; c < m.ce; ++c) n += find_in_row(col, m.s, m.e, __ldg(col + c)) >= 0;
  nmatch[pk] = n;
}

__global__ void __launch_bounds__(256) k_bilu0_nmatch_long(int nb, long long nnzb,
                                                           const int* __restrict__ row,
                                                           const int* __restrict__ col,
                                                           const int* __restrict__ diag,
                                                           int* __restrict__ nmatch) {
  const long long p0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll;
  const int lane = threadIdx.x & 31;
  if (p0 >= nnzb) return;
  unsigned todo = __ballot_sync(FULL, p0 + lane < nnzb && nmatch[p0 + lane] < 0);
  while (todo) {
    const long long pk = p0 + __ffs(todo) - 1;
    todo &= todo - 1;
    int I;
    const MatchLists m = match_lists(pk, nb, row, col, diag, I);
    int n = 0;
    for (int c0 = m.cs; c0 < m.ce; c0 += 32) {
      const int c = c0 + lane;
      const bool hit = c < m.ce && find_in_row(col, m.s, m.e, __ldg(col + c)) >= 0;
      n += __popc(__ballot_sync(FULL, hit));
    }
    if (lane == 0) nmatch[pk] = n;
  }
}

// Total of the match counts in 64 bits (the caller decides from it whether
// the lists fit before their int32 scan).
__global__ void __launch_bounds__(256) k_match_total(long long n, const int* __restrict__ cnt,
                                                     unsigned long long* __restrict__ total) {
  unsigned long long s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += (unsigned)max(__ldg(cnt + i), 0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

// The match lists themselves for the level-order factorisation: a thread
// per lower position writes, in its candidates' order, the pairs (position
// of A_IJ in row I, position of U_KJ in row K) that the factorisation would
// otherwise find by searching inside its dependency chain.
__global__ void __launch_bounds__(256) k_bilu0_match_fill(int nb, long long nnzb,
                                                          const int* __restrict__ row,
                                                          const int* __restrict__ col,
                                                          const int* __restrict__ diag,
                                                          const int* __restrict__ mptr,
                                                          int2* __restrict__ mpair) {
  const long long pk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (pk >= nnzb) return;
  int out = __ldg(mptr + pk);
  const int end = __ldg(mptr + pk + 1);
  if (out >= end) return;
  int I;
  const MatchLists m = match_lists(pk, nb, row, col, diag, I);
  if (m.ce - m.cs > kMatchSerial) return;  // k_bilu0_match_fill_long
  for (int c = m.cs; c < m.ce && out < end; ++c) {
    const int o = find_in_row(col, m.s, m.e, __ldg(col + c));
    if (o >= 0) mpair[out++] = m.from_i ? make_int2(c, o) : make_int2(o, c);
  }
}

// The positions with more than kMatchSerial candidates (two hub rows): a
// warp per 32 positions takes them one at a time, 32 candidates per pass,
// and writes the matches of a pass in candidate order.
__global__ void __launch_bounds__(256) k_bilu0_match_fill_long(int nb, long long nnzb,
                                                               const int* __restrict__ row,
                                                               const int* __restrict__ col,
                                                               const int* __restrict__ diag,
                                                               const int* __restrict__ mptr,
                                                               int2* __restrict__ mpair) {
  const long long p0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll;
  const int lane = threadIdx.x & 31;
  if (p0 >= nnzb) return;  // the whole warp
  bool mine = false;
  if (p0 + lane < nnzb && __ldg(mptr + p0 + lane + 1) > __ldg(mptr + p0 + lane)) {
    int I;
    const MatchLists m = match_lists(p0 + lane, nb, row, col, diag, I);
    mine = m.ce - m.cs > kMatchSerial;
  }
  unsigned todo = __ballot_sync(FULL, mine);
  while (todo) {
    const long long pk = p0 + __ffs(todo) - 1;
    todo &= todo - 1;
    int I;
    const MatchLists m = match_lists(pk, nb, row, col, diag, I);
    int out = __ldg(mptr + pk);
    const int end = __ldg(mptr + pk + 1);
    for (int c0 = m.cs; c0 < m.ce; c0 += 32) {
      const int c = c0 + lane;
      const int o = c < m.ce ? find_in_row(col, m.s, m.e, __ldg(col + c)) : -1;
      const unsigned hit = __ballot_sync(FULL, o >= 0);
      const int at = out + __popc(hit & ((1u << lane) - 1u));
      if (o >= 0 && at < end) mpair[at] = m.from_i ? make_int2(c, o) : make_int2(o, c);
      out += __popc(hit);
    }
  }
}

// Sync-free BILU(0) (matrices with narrow levels or long rows): block rows
// taken by atomic tickets in level order, a warp per row, bounded waits on
// the rows it reads, the row's flag released when it is final.  Hub rows of
// a power-law matrix then no longer hold up a whole level.
template <int BS>
__global__ void __launch_bounds__(kLvlThreads, 3) k_bilu0_syncfree(
    int nb, const int* __restrict__ row, const int* __restrict__ col,
    const int* __restrict__ diag, double* val, SyncState ss) {
  extern __shared__ int stage_smem[];
  const bool staged = dynamic_smem_bytes() >= (blockDim.x >> 5) * kRowStage * sizeof(int);
  int* stage = staged ? stage_smem + (threadIdx.x >> 5) * kRowStage : nullptr;
  const int lane = threadIdx.x & 31;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ss.ticket, 1);
    t = __shfl_sync(FULL, t, 0);
    if (t >= nb) return;
    const int I = __ldg(ss.order + t);
    if (__any_sync(FULL, ld_relaxed(ss.err) != 0)) return;
    if (!bilu0_wrow<BS, true>(I, row, col, diag, val, ss, stage)) return;
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(ss.flags + I, 1);
  }
}

// Rows of each level in ascending index order.  The order inside a level
// is free (its rows are independent); sorted, the rows a warp takes at
// consecutive levels of a structured problem depend on rows of a few
// neighbouring warps instead of rows all over the previous level, which
// the flow schedule turns into shorter waits.  One CTA per level, bitonic
// sort in shared memory; a level wider than kSortCap keeps its breadth-first
// order (only the speed depends on it).
constexpr int kSortCap = 16384;

__global__ void __launch_bounds__(512) k_sort_levels(int* order, const int* __restrict__ lvl_ptr) {
  extern __shared__ int sbuf[];
  const int l = blockIdx.x;
  const int s = __ldg(lvl_ptr + l), n = __ldg(lvl_ptr + l + 1) - s;
  if (n <= 1 || n > kSortCap) return;
  int m2 = 1;
  while (m2 < n) m2 <<= 1;
  for (int t = threadIdx.x; t < m2; t += blockDim.x) sbuf[t] = t < n ? order[s + t] : INT_MAX;
  __syncthreads();
  for (int k = 2; k <= m2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < m2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const int a = sbuf[t], c = sbuf[u];
          if ((a > c) == ((t & k) == 0)) {
            sbuf[t] = c;
            sbuf[u] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) order[s + t] = sbuf[t];
}

// ---------------------------------------------------------------- level schedule (host)
int coop_grid(const void* fn, int threads, size_t smem = 0) {
  return occupancy_grid(fn, threads, smem);
}

// misc words of a level-scheduled launch: count, gen, err, spare
int grid_sync_init(GridSync& gs, Carver& ws, cudaStream_t st) {
  unsigned* misc = ws.take<unsigned>(4);
  if (!misc) return BILU_ERR_WORKSPACE;
  BILU_TRY_CUDA(cudaMemsetAsync(misc, 0, sizeof(unsigned) * 4, st));
  gs.count = misc;
  gs.gen = misc + 1;
  gs.err = (int*)(misc + 2);
  gs.spin = kSpinLimit;
  return BILU_OK;
}

int grid_sync_finish(const GridSync& gs, cudaStream_t st) {
  int herr = 0;
  BILU_TRY_CUDA(cudaMemcpyAsync(&herr, gs.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  return herr;
}

int launch_coop(const void* fn, int grid, int threads, void** args, cudaStream_t st,
                size_t smem = 0) {
  BILU_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3((unsigned)threads),
                                            args, smem, st));
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// Level analysis of the lower (or upper) dependency DAG: successor lists by
// counting sort, then the breadth-first level sweep.  order[nb],
// lvl_ptr[nb+2] and *nlev_d on the device; *h_nlev on the host.
int build_levels(int nb, const int* row, const int* col, const int* diag, int lower,
                 long long ndeps_max, int* order, int* lvl_ptr, int* nlev_d, int* h_nlev,
                 Carver& ws, cudaStream_t st, int* h_sched = nullptr, int* h_maxdeg = nullptr,
                 int* h_fsched = nullptr) {
  int* sptr = ws.take<int>((size_t)nb + 1);
  int* cursor = ws.take<int>((size_t)nb + 1);
  int* indeg = ws.take<int>((size_t)nb + 1);
  int* sidx = ws.take<int>((size_t)std::max(ndeps_max, 1ll));
  // tail[1]: the largest dependency count (k_dep_count); tail[4..6]: the
  // breadth-first sweep's append counters
  int* tail = ws.take<int>(8);
  if (!sptr || !cursor || !indeg || !sidx || !tail) return BILU_ERR_WORKSPACE;
  GridSync gs;
  BILU_TRY(grid_sync_init(gs, ws, st));
  BILU_TRY_CUDA(cudaMemsetAsync(sptr, 0, sizeof(int) * ((size_t)nb + 1), st));
  BILU_TRY_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * ((size_t)nb + 1), st));
  BILU_TRY_CUDA(cudaMemsetAsync(tail, 0, sizeof(int) * 8, st));
  BILU_TRY_CUDA(cudaMemsetAsync(nlev_d, 0, sizeof(int) * 4, st));
  BILU_TRY_CUDA(cudaMemsetAsync(lvl_ptr, 0, sizeof(int) * ((size_t)nb + 2), st));
  if (nb == 0) {
    if (h_nlev) *h_nlev = 0;
    if (h_maxdeg) *h_maxdeg = 0;
    return BILU_OK;
  }
  k_dep_count<<<ceil_div(nb, 256), 256, 0, st>>>(nb, row, col, diag, lower, sptr, indeg,
                                                  tail + 1);
  BILU_LAUNCH_CHECK();
  int total = 0;
  BILU_TRY(scan_exclusive(sptr, sptr, nb, &total, ws, st));
  if (total > ndeps_max) return BILU_ERR_WORKSPACE;
  k_dep_fill<<<ceil_div(nb, 256), 256, 0, st>>>(nb, row, col, diag, lower, sptr, cursor, sidx);
  BILU_LAUNCH_CHECK();
  // two CTAs per SM at most: a level's frontier is small, the barrier's
  // cost grows with the number of CTAs
  int grid = std::min<long long>(std::min(coop_grid((const void*)k_bfs_levels, 256),
                                          2 * sm_count()),
                                 ceil_div(nb, 256));
  int* cnt = tail + 4;
  void* args[] = {&nb, &sptr, &sidx, &indeg, &order, &lvl_ptr, &cnt, &nlev_d, &gs};
  BILU_TRY(launch_coop((const void*)k_bfs_levels, grid, 256, args, st));
  int herr = grid_sync_finish(gs, st);
  if (herr != 0) return herr;
  int h[2] = {0, 0};
  BILU_TRY_CUDA(cudaMemcpyAsync(&h[0], nlev_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  BILU_TRY_CUDA(cudaMemcpyAsync(&h[1], lvl_ptr + h[0], sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (h[1] != nb) return BILU_ERR_PATTERN;  // a row was never reached
  if (h_nlev) *h_nlev = h[0];
  if (h[0] > 0) {
    static bool attr_set = false;
    if (!attr_set) {
      BILU_TRY_CUDA(cudaFuncSetAttribute((const void*)k_sort_levels,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kSortCap * sizeof(int))));
      attr_set = true;
    }
    k_sort_levels<<<(unsigned)h[0], 512, kSortCap * sizeof(int), st>>>(order, lvl_ptr);
    BILU_LAUNCH_CHECK();
  }
  // nlev_d[1] = the largest dependency count (picks warp or group rows);
  // nlev_d[2] = the recommended schedule (0 level, 1 sync-free)
  BILU_TRY_CUDA(cudaMemcpyAsync(nlev_d + 1, tail + 1, sizeof(int), cudaMemcpyDeviceToDevice, st));
  int maxdeg = 0;
  BILU_TRY_CUDA(cudaMemcpy(&maxdeg, tail + 1, sizeof(int), cudaMemcpyDeviceToHost));
  // nlev_d[2] = the recommended solve schedule, nlev_d[3] the recommended
  // factorisation schedule (0 level order, 1 sync-free)
  int sched[2] = {maxdeg > kFlowMaxDeps ? 1 : 0,
                  ((long long)nb < (long long)kFactorLevelWidth * h[0] || maxdeg > kLongRow) ? 1
                                                                                            : 0};
  BILU_TRY_CUDA(cudaMemcpy(nlev_d + 2, sched, sizeof(sched), cudaMemcpyHostToDevice));
  if (h_sched) *h_sched = sched[0];
  if (h_fsched) *h_fsched = sched[1];
  if (h_maxdeg) *h_maxdeg = maxdeg;
  return BILU_OK;
}

template <int BS>
int launch_sptrsv_levels(int nb, const int* row, const int* col, const int* diag,
                         const double* val, int lower, int unit, const double* b, double* x,
                         const int* order, const int* lvl_ptr, const int* nlev_d, int nlev,
                         SyncState ss, GridSync gs, cudaStream_t st) {
  const void* fn = lower ? (unit ? (const void*)k_sptrsv_levels<BS, true, true>
                                 : (const void*)k_sptrsv_levels<BS, true, false>)
                         : (unit ? (const void*)k_sptrsv_levels<BS, false, true>
                                 : (const void*)k_sptrsv_levels<BS, false, false>);
  // no more lane groups than rows; fewer CTAs make the barrier cheaper
  int grid = std::min<long long>(coop_grid(fn, kLvlThreads),
                                 ceil_div(nb, (kLvlThreads / 32) * (32 / BS)));
  gs.per_sm = std::max(1, std::min(occupancy_per_sm(fn, kLvlThreads), (int)ceil_div(grid, sm_count())));
  (void)nlev;
  void* args[] = {&row, &col, &diag, &val, &b, &x, &order, &lvl_ptr, &nlev_d, &ss, &gs};
  return launch_coop(fn, grid, kLvlThreads, args, st);
}

// Flow-scheduled solve: x is filled with the pending pattern on the stream,
// then one cooperative launch (every warp resident, so every wait ends).
// rdiag: reciprocal pivots for the upper solve (null: divide); y64: an
// FP64 copy of x (null: none).
template <int BS, class T>
int launch_sptrsv_flow_t(int nb, const int* row, const int* col, const int* diag, const T* val,
                         int lower, int unit, const T* b, T* x, double* y64, const T* rdiag,
                         const int* order, const int* lvl_ptr, const int* nlev_d, SyncState ss,
                         cudaStream_t st) {
  const void* fn = lower ? (unit ? (const void*)k_sptrsv_flow<BS, true, true, T>
                                 : (const void*)k_sptrsv_flow<BS, true, false, T>)
                         : (unit ? (const void*)k_sptrsv_flow<BS, false, true, T>
                                 : (const void*)k_sptrsv_flow<BS, false, false, T>);
  int grid = std::min<long long>(coop_grid(fn, kLvlThreads),
                                 ceil_div(nb, (kLvlThreads / 32) * (32 / BS)));
  int per_sm = std::max(1, std::min(occupancy_per_sm(fn, kLvlThreads), (int)ceil_div(grid, sm_count())));
  const long long n = (long long)nb * BS;
  k_fill_pending<T><<<(unsigned)std::min<long long>(ceil_div(n, 256), (long long)sm_count() * 16),
                      256, 0, st>>>((typename XBits<T>::U*)x, n);
  BILU_LAUNCH_CHECK();
  void* args[] = {&row, &col,   &diag,    &val,     &b,      &x,  &y64,
                  &rdiag, &order, &lvl_ptr, &nlev_d, &ss, &per_sm};
  return launch_coop(fn, grid, kLvlThreads, args, st);
}

template <int BS>
int launch_sptrsv_flow(int nb, const int* row, const int* col, const int* diag,
                       const double* val, int lower, int unit, const double* b, double* x,
                       const int* order, const int* lvl_ptr, const int* nlev_d, SyncState ss,
                       cudaStream_t st) {
  return launch_sptrsv_flow_t<BS, double>(nb, row, col, diag, val, lower, unit, b, x, nullptr,
                                          ss.rdiag, order, lvl_ptr, nlev_d, ss, st);
}

template <int BS>
int launch_sptrsv_flow_f32(int nb, const int* row, const int* col, const int* diag,
                           const float* val, int lower, int unit, const float* b, float* x,
                           double* y64, const float* rdiag, const int* order, const int* lvl_ptr,
                           const int* nlev_d, SyncState ss, cudaStream_t st) {
  return launch_sptrsv_flow_t<BS, float>(nb, row, col, diag, val, lower, unit, b, x, y64, rdiag,
                                         order, lvl_ptr, nlev_d, ss, st);
}

template <int BS>
int launch_bilu0_syncfree(int nb, const int* row, const int* col, const int* diag, double* val,
                          SyncState ss, cudaStream_t st) {
  const void* fn = (const void*)k_bilu0_syncfree<BS>;
  const size_t smem = (size_t)(kLvlThreads / 32) * kRowStage * sizeof(int);
  static bool attr_set = false;
  if (!attr_set) {
    BILU_TRY_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr_set = true;
  }
  // every warp resident at once is not required (tickets), but more warps
  // than rows would only spin
  int grid = std::min<long long>(occupancy_grid(fn, kLvlThreads, smem),
                                 ceil_div(nb, kLvlThreads / 32));
  k_bilu0_syncfree<BS><<<grid, kLvlThreads, smem, st>>>(nb, row, col, diag, val, ss);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

template <int BS>
int launch_bilu0_levels(int nb, const int* row, const int* col, const int* diag, double* val,
                        const int* order, const int* lvl_ptr, const int* nlev_d, SyncState ss,
                        GridSync gs, const int* mptr, const int2* mpair, cudaStream_t st) {
  const void* fn = (const void*)k_bilu0_levels<BS>;
  int grid = std::min<long long>(coop_grid(fn, kLvlThreads),
                                 ceil_div(nb, (kLvlThreads / 32) * (32 / BS)));
  gs.per_sm = std::max(1, std::min(occupancy_per_sm(fn, kLvlThreads), (int)ceil_div(grid, sm_count())));
  void* args[] = {&row, &col, &diag, &val, &order, &lvl_ptr, &nlev_d, &ss, &gs, &mptr, &mpair};
  return launch_coop(fn, grid, kLvlThreads, args, st);
}

}  // namespace

size_t syncfree_ws(int nb) {
  // flags + order + (levels, counts, misc, scan) + sync misc + error words
  return carve_size(sizeof(int) * ((size_t)nb + 1)) * 4 + carve_size(sizeof(int) * 4) * 2 +
         carve_size(sizeof(int) * 2) + scan_ws_bytes(nb + 1);
}

// Level analysis scratch (successor lists of up to ndeps dependencies).
size_t levels_ws(int nb, long long ndeps) {
  return carve_size(sizeof(int) * ((size_t)nb + 1)) * 3 +
         carve_size(sizeof(int) * (size_t)std::max(ndeps, 1ll)) + carve_size(sizeof(int) * 8) +
         carve_size(sizeof(unsigned) * 4) + scan_ws_bytes(nb + 1);
}

// Level-scheduled factor / solve scratch: the analysis output (order,
// lvl_ptr, nlev), the analysis scratch, and the error / barrier words.
size_t level_sched_ws(int nb, long long nnzb) {
  return carve_size(sizeof(int) * ((size_t)nb + 1)) + carve_size(sizeof(int) * ((size_t)nb + 2)) +
         carve_size(sizeof(int) * 2) + levels_ws(nb, std::max(nnzb - nb, 0ll)) +
         carve_size(sizeof(int) * 4) + carve_size(sizeof(unsigned) * 4);
}

// BILU(0) scratch: the level-scheduled one plus the sync-free schedule's
// per-position match counts.
size_t bilu0_ws(int nb, long long nnzb) {
  return level_sched_ws(nb, nnzb) + carve_size(sizeof(int) * (size_t)std::max(nnzb, 1ll));
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

namespace {

// error and zero-pivot words without per-row flags (level schedule)
int sync_init_words(SyncState& ss, Carver& ws, cudaStream_t st) {
  int* misc = ws.take<int>(4);
  if (!misc) return BILU_ERR_WORKSPACE;
  ss = SyncState{nullptr, misc, misc + 1, misc + 2, kSpinLimit, -1, nullptr};
  int init[4] = {0, 0, INT_MAX, 0};
  BILU_TRY_CUDA(cudaMemcpyAsync(misc, init, sizeof(init), cudaMemcpyHostToDevice, st));
  return BILU_OK;
}

}  // namespace

// BILU(0) in place, level scheduled (one cooperative launch, one grid
// barrier per dependency level of the lower DAG) or sync-free.  rdiag
// (nb x bs) receives the reciprocal pivots; null: carved from ws.  keep
// (optional): where the level analysis of the lower DAG is built and kept.
// Level analysis of BILU(0)'s lower DAG into keep (order, lvl, nlev on the
// device; level count, schedules and largest dependency count on the host).
// Structure only: it may run before the values are on the device.
int bilu0_analyze(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                  LevelOut& keep, Carver& ws, cudaStream_t st) {
  if (!keep.order || !keep.lvl || !keep.nlev) return BILU_ERR_WORKSPACE;
  return build_levels(nb, row, col, diag, 1, std::max(nnzb - nb, 0ll), keep.order, keep.lvl,
                      keep.nlev, &keep.h_nlev, ws, st, &keep.h_sched, &keep.h_maxdeg,
                      &keep.h_fsched);
}

// BILU(0)'s match lists from the pattern alone (a structure step, before
// the values): mptr (nnzb + 1 ints) receives the per-position counts and
// *h_total their sum; when the sum is at most cap, mptr is turned into
// their exclusive scan for bilu0_match_fill, else it is left as counts and
// the lists are not to be built.  Synchronises the stream once.
int bilu0_match_count(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                      int* mptr, long long cap, long long* h_total, Carver& ws,
                      cudaStream_t st) {
  *h_total = 0;
  if (nb < 1 || nnzb < 1) return BILU_OK;
  unsigned long long* tot = ws.take<unsigned long long>(1);
  if (!tot) return BILU_ERR_WORKSPACE;
  const unsigned grid = ceil_div(nnzb, 256);
  k_bilu0_nmatch<<<grid, 256, 0, st>>>(nb, nnzb, row, col, diag, mptr);
  BILU_LAUNCH_CHECK();
  k_bilu0_nmatch_long<<<grid, 256, 0, st>>>(nb, nnzb, row, col, diag, mptr);
  BILU_LAUNCH_CHECK();
  BILU_TRY_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), st));
  k_match_total<<<std::min(grid, 1024u), 256, 0, st>>>(nnzb, mptr, tot);
  BILU_LAUNCH_CHECK();
  unsigned long long h = 0;
  BILU_TRY_CUDA(cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  *h_total = (long long)std::min<unsigned long long>(h, (unsigned long long)LLONG_MAX);
  if (*h_total > cap || *h_total > (long long)INT_MAX) return BILU_OK;
  return scan_exclusive(mptr, mptr, nnzb, nullptr, ws, st);
}

// The lists themselves, into mpair (mptr[nnzb] pairs) after bilu0_match_count.
int bilu0_match_fill(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                     const int* mptr, int2* mpair, cudaStream_t st) {
  if (nb < 1 || nnzb < 1) return BILU_OK;
  k_bilu0_match_fill<<<ceil_div(nnzb, 256), 256, 0, st>>>(nb, nnzb, row, col, diag, mptr,
                                                          mpair);
  BILU_LAUNCH_CHECK();
  k_bilu0_match_fill_long<<<ceil_div(nnzb, 256), 256, 0, st>>>(nb, nnzb, row, col, diag, mptr,
                                                               mpair);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

// BILU(0) on an analysis from bilu0_analyze (with the match lists when
// keep has them and the level-order kernel runs).
int bilu0_factor(int nb, long long nnzb, int bs, const int* row, const int* col,
                 const int* diag, double* val, int* h_zp, Carver& ws, cudaStream_t st,
                 int schedule, double* rdiag, const LevelOut& keep) {
  int* order = keep.order;
  int* lvl = keep.lvl;
  int* nlev_d = keep.nlev;
  if (!rdiag) rdiag = ws.take<double>((size_t)nb * bs + 1);
  if (!order || !lvl || !nlev_d || !rdiag) return BILU_ERR_WORKSPACE;
  int sched = keep.h_fsched;
  if (schedule == 0 || schedule == 1) sched = schedule;  // caller's choice
  if (sched == 1) {
    // narrow levels or long rows: sync-free, tickets in level order
    int* nmatch = ws.take<int>((size_t)std::max(nnzb, 1ll));
    if (!nmatch) return BILU_ERR_WORKSPACE;
    SyncState ss;
    BILU_TRY(sync_init(ss, nb, ws, st));
    ss.order = order;
    ss.rdiag = rdiag;
    ss.nmatch = nmatch;
    if (nb > 0) {
      const unsigned grid = ceil_div(std::max(nnzb, 1ll), 256);
      k_bilu0_nmatch<<<grid, 256, 0, st>>>(nb, nnzb, row, col, diag, nmatch);
      BILU_LAUNCH_CHECK();
      k_bilu0_nmatch_long<<<grid, 256, 0, st>>>(nb, nnzb, row, col, diag, nmatch);
      BILU_LAUNCH_CHECK();
      BILU_TRY(BILU_DISPATCH_BS(bs, launch_bilu0_syncfree, nb, row, col, diag, val, ss, st));
    }
    return sync_finish(ss, h_zp, st);
  }
  SyncState ss;
  BILU_TRY(sync_init_words(ss, ws, st));
  ss.rdiag = rdiag;
  GridSync gs;
  BILU_TRY(grid_sync_init(gs, ws, st));
  if (nb > 0)
    BILU_TRY(BILU_DISPATCH_BS(bs, launch_bilu0_levels, nb, row, col, diag, val, order, lvl,
                              nlev_d, ss, gs, keep.mptr, keep.mpair, st));
  int herr = grid_sync_finish(gs, st);
  if (herr != 0) return herr;
  return sync_finish(ss, h_zp, st);
}

// Analysis and factorisation; the analysis goes to keep when its arrays are
// given, else to the workspace.
int bilu0_impl(int nb, long long nnzb, int bs, const int* row, const int* col, const int* diag,
               double* val, int* h_zp, Carver& ws, cudaStream_t st, int schedule,
               double* rdiag, LevelOut* keep) {
  const bool kept = keep && keep->order && keep->lvl && keep->nlev;
  LevelOut local;
  LevelOut& k = kept ? *keep : local;
  if (!kept) {
    k.order = ws.take<int>((size_t)nb + 1);
    k.lvl = ws.take<int>((size_t)nb + 2);
    k.nlev = ws.take<int>(4);
    if (!k.order || !k.lvl || !k.nlev) return BILU_ERR_WORKSPACE;
  }
  {
    Carver w2 = ws;
    BILU_TRY(bilu0_analyze(nb, nnzb, row, col, diag, k, w2, st));
  }
  return bilu0_factor(nb, nnzb, bs, row, col, diag, val, h_zp, ws, st, schedule, rdiag, k);
}

// Sync-free solve (dynamic tickets over the level order, per-row flags).
// Needs only nb-sized scratch (no successor lists): used by the
// allocation-free entry point and the timeout test hook.
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

// Level-scheduled solve with a level analysis (order, lvl_ptr, nlev_d):
// the flow kernel (waits on the x entries read) when no row has more than
// kLongRow dependencies (maxdeg, from the analysis), else the barrier
// kernel with a warp per row.  x must not alias b (the flow kernel marks x
// pending before it starts).
int sptrsv_levels(int nb, int bs, const int* row, const int* col, const int* diag,
                  const int* order, const int* lvl, const int* nlev_d, const double* val,
                  int lower, int unit, const double* b, double* x, Carver& ws, cudaStream_t st,
                  int maxdeg) {
  SyncState ss;
  BILU_TRY(sync_init_words(ss, ws, st));
  GridSync gs;
  BILU_TRY(grid_sync_init(gs, ws, st));
  ss.err = gs.err;  // one error word for either kernel
  if (nb > 0) {
    if (maxdeg <= kLongRow)
      BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv_flow, nb, row, col, diag, val, lower, unit, b,
                                x, order, lvl, nlev_d, ss, st));
    else
      BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv_levels, nb, row, col, diag, val, lower, unit,
                                b, x, order, lvl, nlev_d, 0, ss, gs, st));
  }
  return grid_sync_finish(gs, st);
}

// Sync-free solve on a level order (ticket order = order[]).
int sptrsv_syncfree_ordered(int nb, int bs, const int* row, const int* col, const int* diag,
                            const int* order, const double* val, int lower, int unit,
                            const double* b, double* x, Carver& ws, cudaStream_t st) {
  SyncState ss;
  BILU_TRY(sync_init(ss, nb, ws, st));
  ss.order = order;
  if (nb > 0)
    BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv, nb, row, col, diag, val, lower, unit, b, x, ss,
                              st));
  return sync_finish(ss, nullptr, st);
}

// One-shot solve: level analysis, then the schedule it recommends.
int sptrsv_level_impl(int nb, long long nnzb, int bs, const int* row, const int* col,
                      const int* diag, const double* val, int lower, int unit, const double* b,
                      double* x, Carver& ws, cudaStream_t st) {
  int* order = ws.take<int>((size_t)nb + 1);
  int* lvl = ws.take<int>((size_t)nb + 2);
  int* nlev_d = ws.take<int>(4);
  if (!order || !lvl || !nlev_d) return BILU_ERR_WORKSPACE;
  int sched = 0, maxdeg = 0;
  {
    Carver w2 = ws;
    BILU_TRY(build_levels(nb, row, col, diag, lower, std::max(nnzb - nb, 0ll), order, lvl,
                          nlev_d, nullptr, w2, st, &sched, &maxdeg));
  }
  if (sched == 1)
    return sptrsv_syncfree_ordered(nb, bs, row, col, diag, order, val, lower, unit, b, x, ws, st);
  return sptrsv_levels(nb, bs, row, col, diag, order, lvl, nlev_d, val, lower, unit, b, x, ws,
                       st, maxdeg);
}

// Level analysis into caller-owned arrays (order[nb+1], lvl[nb+2], nlev[2]).
int level_analysis(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                   int lower, int* order, int* lvl, int* nlev_d, int* h_nlev, Carver& ws,
                   cudaStream_t st, int* h_sched, int* h_maxdeg) {
  return build_levels(nb, row, col, diag, lower, std::max(nnzb - nb, 0ll), order, lvl, nlev_d,
                      h_nlev, ws, st, h_sched, h_maxdeg);
}

// Launch-only sync-free solve for use inside a solver: flags and ticket
// (nb + 1 and 1 ints, caller-owned) are cleared on the stream before the
// launch; failures land in *err for a later check.
int sptrsv_syncfree_async(int nb, int bs, const int* row, const int* col, const int* diag,
                          const int* order, const double* val, int lower, int unit,
                          const double* b, double* x, int* flags, int* ticket, int* err,
                          cudaStream_t st, const double* rdiag) {
  if (nb == 0) return BILU_OK;
  BILU_TRY_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * ((size_t)nb + 1), st));
  BILU_TRY_CUDA(cudaMemsetAsync(ticket, 0, sizeof(int), st));
  SyncState ss{flags, ticket, err, err, kSpinLimit, -1, order, const_cast<double*>(rdiag)};
  return BILU_DISPATCH_BS(bs, launch_sptrsv, nb, row, col, diag, val, lower, unit, b, x, ss, st);
}

// Launch-only level-scheduled solve for use inside a solver: no host
// synchronisation.  words: [0] barrier count, [1] exit count (both 0
// between launches), [2] error word (0 or a bilu_status, read by the caller
// later), [3] zero-pivot word.
int sptrsv_levels_async(int nb, int bs, const int* row, const int* col, const int* diag,
                        const int* order, const int* lvl, const int* nlev_d, const double* val,
                        int lower, int unit, const double* b, double* x, unsigned* words,
                        cudaStream_t st, const double* rdiag, int maxdeg) {
  if (nb == 0) return BILU_OK;
  int* w = (int*)words;
  SyncState ss{nullptr, nullptr, w + 2, w + 3, kSpinLimit, -1, nullptr,
               const_cast<double*>(rdiag)};
  if (maxdeg <= kLongRow)
    return BILU_DISPATCH_BS(bs, launch_sptrsv_flow, nb, row, col, diag, val, lower, unit, b, x,
                            order, lvl, nlev_d, ss, st);
  GridSync gs{words, words + 1, w + 2, kSpinLimit};
  return BILU_DISPATCH_BS(bs, launch_sptrsv_levels, nb, row, col, diag, val, lower, unit, b, x,
                          order, lvl, nlev_d, 0, ss, gs, st);
}

// Launch-only FP32 level-order solve for the mixed exact-ILU apply: FP32
// factor values, b and x (x32 must not be b32), FP32 reciprocal pivots for
// the upper solve, an optional FP64 copy of x (y64).  Only the flow kernel
// has an FP32 form: patterns with rows of more than kLongRow dependencies
// return BILU_ERR_UNSUPPORTED.  words as sptrsv_levels_async.
int sptrsv_flow_f32_async(int nb, int bs, const int* row, const int* col, const int* diag,
                          const int* order, const int* lvl, const int* nlev_d, const float* val,
                          int lower, int unit, const float* b32, float* x32, double* y64,
                          unsigned* words, cudaStream_t st, const float* rdiag32, int maxdeg) {
  if (nb == 0) return BILU_OK;
  if (maxdeg > kLongRow) return BILU_ERR_UNSUPPORTED;
  int* w = (int*)words;
  SyncState ss{nullptr, nullptr, w + 2, w + 3, kSpinLimit, -1, nullptr, nullptr};
  return BILU_DISPATCH_BS(bs, launch_sptrsv_flow_f32, nb, row, col, diag, val, lower, unit, b32,
                          x32, y64, rdiag32, order, lvl, nlev_d, ss, st);
}

}  // namespace bilu

using namespace bilu;

namespace {

// analysis record: diag[nb+1] | order[nb+1] | lvl_ptr[nb+2] | nlev[4]
struct AnalysisView {
  int *diag, *order, *lvl, *nlev;
  AnalysisView(void* p, int nb) {
    Carver c(p, (size_t)-1 / 2);
    diag = c.take<int>((size_t)nb + 1);
    order = c.take<int>((size_t)nb + 1);
    lvl = c.take<int>((size_t)nb + 2);
    nlev = c.take<int>(4);  // levels, largest dependency count, solve and factor schedules
  }
};

// The analysis record's four words on the host (a synchronising read).
int read_analysis_words(int nb, const AnalysisView& a, int* h, cudaStream_t st) {
  if (nb == 0) return BILU_OK;
  BILU_TRY_CUDA(cudaMemcpyAsync(h, a.nlev, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  return BILU_OK;
}

}  // namespace

extern "C" size_t bilu_sptrsv_analysis_bytes(int nb) {
  if (nb < 0) return 0;
  return 2 * carve_size(sizeof(int) * ((size_t)nb + 1)) +
         carve_size(sizeof(int) * ((size_t)nb + 2)) + carve_size(sizeof(int) * 4);
}

extern "C" size_t bilu_sptrsv_analysis_ws_bytes(int nb, int nnzb) {
  if (nb < 0 || nnzb < 0) return 0;
  return levels_ws(nb, std::max((long long)nnzb - nb, 0ll)) + carve_size(sizeof(int) * 2);
}

extern "C" size_t bilu_sptrsv_solve_ws_bytes(int nb) {
  if (nb < 0) return 0;
  return syncfree_ws(nb);
}

extern "C" int bilu_sptrsv_analysis(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                                    int lower, void* d_info, void* d_ws, size_t ws_bytes,
                                    bilu_stream_t stream) {
  if (nb < 0 || nnzb < nb || !d_info || (nb > 0 && (!d_row || !d_col))) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  AnalysisView a(d_info, nb);
  Carver ws(d_ws, ws_bytes);
  BILU_TRY(diag_positions(nb, d_row, d_col, a.diag, nullptr, ws, S(stream)));
  return build_levels(nb, d_row, d_col, a.diag, lower != 0, (long long)nnzb - nb, a.order, a.lvl,
                      a.nlev, nullptr, ws, S(stream));
}

extern "C" int bilu_sptrsv_solve(int nb, int bs, const int* d_row, const int* d_col,
                                 const double* d_val, int lower, int unit, const void* d_info,
                                 const double* d_b, double* d_x, void* d_ws, size_t ws_bytes,
                                 bilu_stream_t stream) {
  if (nb < 0 || !d_info || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)) ||
      (nb > 0 && (const void*)d_b == (const void*)d_x))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  AnalysisView a(const_cast<void*>(d_info), nb);
  Carver ws(d_ws, ws_bytes);
  int h[4] = {0, 0, 0, 0};  // levels, largest dependency count, solve / factor schedule
  BILU_TRY(read_analysis_words(nb, a, h, S(stream)));
  if (h[2] == 1)
    return sptrsv_syncfree_ordered(nb, bs, d_row, d_col, a.diag, a.order, d_val, lower != 0,
                                   unit != 0, d_b, d_x, ws, S(stream));
  return sptrsv_levels(nb, bs, d_row, d_col, a.diag, a.order, a.lvl, a.nlev, d_val, lower != 0,
                       unit != 0, d_b, d_x, ws, S(stream), h[1]);
}

extern "C" int bilu_sptrsv_solve_level(int nb, int bs, const int* d_row, const int* d_col,
                                       const double* d_val, int lower, int unit,
                                       const void* d_info, const double* d_b, double* d_x,
                                       void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || !d_info || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)) ||
      (nb > 0 && (const void*)d_b == (const void*)d_x))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  AnalysisView a(const_cast<void*>(d_info), nb);
  Carver ws(d_ws, ws_bytes);
  int h[4] = {0, 0, 0, 0};
  BILU_TRY(read_analysis_words(nb, a, h, S(stream)));
  return sptrsv_levels(nb, bs, d_row, d_col, a.diag, a.order, a.lvl, a.nlev, d_val, lower != 0,
                       unit != 0, d_b, d_x, ws, S(stream), h[1]);
}

extern "C" int bilu_sptrsv_solve_syncfree(int nb, int bs, const int* d_row, const int* d_col,
                                          const double* d_val, int lower, int unit,
                                          const void* d_info, const double* d_b, double* d_x,
                                          void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || !d_info || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)) ||
      (nb > 0 && (const void*)d_b == (const void*)d_x))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  AnalysisView a(const_cast<void*>(d_info), nb);
  Carver ws(d_ws, ws_bytes);
  return sptrsv_syncfree_ordered(nb, bs, d_row, d_col, a.diag, a.order, d_val, lower != 0,
                                 unit != 0, d_b, d_x, ws, S(stream));
}

extern "C" size_t bilu_bsrilu0_ws_bytes(int nb, int nnzb) {
  if (nb < 0 || nnzb < 0) return 0;
  // diag, bad-row word, reciprocal pivots (largest block size), level scratch
  return carve_size(sizeof(int) * ((size_t)nb + 1)) + carve_size(sizeof(int) * 2) +
         carve_size(sizeof(double) * ((size_t)nb * 8 + 1)) + bilu0_ws(nb, nnzb);
}

extern "C" int bilu_bsrilu0(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                            double* d_val, int* h_info, void* d_ws, size_t ws_bytes,
                            bilu_stream_t stream) {
  return bilu_bsrilu0_ex(nb, nnzb, bs, d_row, d_col, d_val, -1, h_info, d_ws, ws_bytes, stream);
}

extern "C" int bilu_bsrilu0_ex(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                               double* d_val, int schedule, int* h_info, void* d_ws,
                               size_t ws_bytes, bilu_stream_t stream) {
  if (h_info) *h_info = -1;
  if (nb < 0 || nnzb < 0 || (nb > 0 && (!d_row || !d_col || !d_val))) return BILU_ERR_ARG;
  if (schedule < -1 || schedule > 1) return BILU_ERR_ARG;
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
  return bilu0_impl(nb, nnzb, bs, d_row, d_col, diag, d_val, h_info, ws, S(stream), schedule,
                    nullptr, nullptr);
}

extern "C" size_t bilu_sptrsv_ws_bytes(int nb, int nnzb) {
  if (nb < 0 || nnzb < 0) return 0;
  return carve_size(sizeof(int) * ((size_t)nb + 1)) + carve_size(sizeof(int) * 2) +
         level_sched_ws(nb, nnzb);
}

extern "C" int bilu_sptrsv(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                           const double* d_val, int lower, const double* d_b, double* d_x,
                           void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  return bilu_sptrsv_ex(nb, nnzb, bs, d_row, d_col, d_val, lower, lower, d_b, d_x, d_ws, ws_bytes,
                        stream);
}

extern "C" int bilu_sptrsv_ex(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                              const double* d_val, int lower, int unit, const double* d_b,
                              double* d_x, void* d_ws, size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 0 || nnzb < nb || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x)) ||
      (nb > 0 && (const void*)d_b == (const void*)d_x))
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return sptrsv_level_impl(nb, nnzb, bs, d_row, d_col, diag, d_val, lower != 0, unit != 0, d_b,
                           d_x, ws, S(stream));
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

// Test hook: the flow (level-order) solve with block row `withhold_row`
// never storing its x entries and a spin budget of spin_limit polls, so the
// rows that read them give up and the call returns BILU_ERR_TIMEOUT (the
// others see the error word and leave).  Every wait is bounded; the launch
// ends by itself and the context stays usable.  Patterns with rows of more
// than 32 dependencies take the barrier kernel and are refused here.
extern "C" int bilu_debug_sptrsv_withhold_flow(int nb, int nnzb, int bs, const int* d_row,
                                               const int* d_col, const double* d_val, int lower,
                                               const double* d_b, double* d_x, int withhold_row,
                                               long long spin_limit, void* d_ws,
                                               size_t ws_bytes, bilu_stream_t stream) {
  if (nb < 1 || nnzb < nb || !d_row || !d_col || !d_val || !d_b || !d_x || d_b == d_x ||
      spin_limit < 1 || spin_limit > kSpinLimit)
    return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  Carver ws(d_ws, ws_bytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  int* order = ws.take<int>((size_t)nb + 1);
  int* lvl = ws.take<int>((size_t)nb + 2);
  int* nlev_d = ws.take<int>(4);
  if (!diag || !order || !lvl || !nlev_d) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, st));
  int maxdeg = 0;
  {
    Carver w2 = ws;
    BILU_TRY(build_levels(nb, d_row, d_col, diag, lower != 0, (long long)nnzb - nb, order, lvl,
                          nlev_d, nullptr, w2, st, nullptr, &maxdeg));
  }
  if (maxdeg > kLongRow) return BILU_ERR_UNSUPPORTED;
  SyncState ss;
  BILU_TRY(sync_init_words(ss, ws, st));
  GridSync gs;
  BILU_TRY(grid_sync_init(gs, ws, st));
  ss.err = gs.err;
  ss.spin = spin_limit;
  ss.withhold = withhold_row;
  BILU_TRY(BILU_DISPATCH_BS(bs, launch_sptrsv_flow, nb, d_row, d_col, diag, d_val, lower != 0,
                            lower != 0, d_b, d_x, order, lvl, nlev_d, ss, st));
  return grid_sync_finish(gs, st);
}
