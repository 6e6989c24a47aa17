// Grid-wide synchronisation for cooperative launches (sm_103a): bounded
// polling with back-off and a counting grid barrier.  Shared by the level
// kernels (BILU(0), triangular solves, level analysis) and the Krylov
// solver's orthogonalisation kernels.
#pragma once

#include "common.cuh"

namespace bilu {

// Exponential back-off between polls (32 ns doubling to 256 ns): waiters that
// spin at full rate flood the L2 with flag reads and slow the rows they wait
// for.
__device__ __forceinline__ void backoff(unsigned& ns) {
  __nanosleep(ns);
  ns = ns < 256u ? ns * 2u : 256u;
}

// Acquire side of the flag handshake.  Flags are polled with relaxed loads
// (an acquire load per poll would invalidate L1 on every iteration of every
// spinning warp); once the release store is observed, one acquire fence
// orders the reads of the producer's data after it.
__device__ __forceinline__ void fence_acquire() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

struct GridSync {
  unsigned* count;  // arrivals since the launch started
  unsigned* gen;    // CTAs that have left the kernel (grid_exit_count)
  int* err;         // 0 or a bilu_status; set on a barrier timeout
  long long spin;   // polls before a waiting CTA gives up
  int per_sm = 1;   // CTAs of the launch resident on one SM
};

__device__ __forceinline__ unsigned ld_relaxed_u(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned atom_add_acq_rel_u(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v)
               : "memory");
  return old;
}

// Counting grid barrier.  After __syncthreads, thread 0 of each CTA arrives
// with an acquire-release atomic (release: the CTA's writes, ordered before
// it by the CTA barrier, become visible with it); the arrival count grows
// through the launch (barrier b is complete when it reaches
// (b + 1) x gridDim.x) and every CTA polls the count itself with relaxed
// loads and back-off, then takes one acquire fence, so the release reaches
// the waiting CTAs with the last arrival's atomic.  (On GB300 an
// acquire-release arrival costs ~0.9 us less than a fence + relaxed atomic
// at 304 CTAs, and polling the count ~0.7 us less than a generation word
// that the last arriver writes after its atomic returns.)  `passed` counts the
// barriers this CTA has passed (thread 0's copy is the one used).  The
// comparison is modulo 2^32.  g.gen counts CTAs that have left the kernel
// (grid_exit_count); both words are 0 between launches.
__device__ __forceinline__ bool grid_sync_count(const GridSync& g, unsigned& passed) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned target = (passed + 1u) * gridDim.x;
    unsigned v = atom_add_acq_rel_u(g.count, 1u) + 1u;
    long long n = 0;
    unsigned ns = 32;
    while ((int)(v - target) < 0) {
      if (ld_relaxed(g.err) != 0) { ok = 0; break; }
      if (++n > g.spin) {
        atomicCAS(g.err, 0, (int)BILU_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      backoff(ns);
      v = ld_relaxed_u(g.count);
    }
    fence_acquire();
    passed += 1u;
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// End of a launch that used grid_sync_count: a CTA arrives here only after
// passing every barrier, so when the last one arrives no CTA polls the
// count any more and both words can go back to 0 for the next launch.  (A
// launch that aborted skips this; its error word is set and the caller
// clears the words before the next solve.)
__device__ __forceinline__ void grid_exit_count(const GridSync& g) {
  if (threadIdx.x == 0 && atomicAdd(g.gen, 1u) == gridDim.x - 1u) {
    atomicExch(g.count, 0u);
    atomicExch(g.gen, 0u);
  }
}

}  // namespace bilu
