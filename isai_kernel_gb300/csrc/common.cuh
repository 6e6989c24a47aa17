// Shared helpers for the sm_103a kernels of libbilu_isai.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bilu_isai.h"

namespace bilu {

// Last CUDA error seen by a host entry point of this thread.
extern thread_local int g_last_cuda_error;
// Kernel launches issued by this library (all threads), for accounting.
extern unsigned long long g_launches;

inline int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return BILU_OK;
  g_last_cuda_error = (int)e;
  return BILU_ERR_CUDA;
}

#define BILU_TRY_CUDA(call)                          \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return ::bilu::cuda_status(e_); \
  } while (0)

#define BILU_TRY(call)               \
  do {                               \
    int st_ = (call);                \
    if (st_ != BILU_OK) return st_;  \
  } while (0)

#define BILU_LAUNCH_CHECK()                                    \
  do {                                                         \
    __atomic_fetch_add(&::bilu::g_launches, 1ull, __ATOMIC_RELAXED); \
    BILU_TRY_CUDA(cudaGetLastError());                         \
  } while (0)

inline cudaStream_t S(bilu_stream_t s) { return (cudaStream_t)s; }

inline bool bs_supported(int bs) { return bs == 4 || bs == 5 || bs == 8; }

// Dispatch a templated launcher over the built block sizes.
#define BILU_DISPATCH_BS(bs, FN, ...)                 \
  ((bs) == 4   ? FN<4>(__VA_ARGS__)                    \
   : (bs) == 5 ? FN<5>(__VA_ARGS__)                    \
   : (bs) == 8 ? FN<8>(__VA_ARGS__)                    \
               : BILU_ERR_UNSUPPORTED)

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Workspace carving: aligned sub-allocations from a caller buffer.
struct Carver {
  char* base;
  size_t cap, used;
  Carver(void* p, size_t n) : base((char*)p), cap(n), used(0) {}
  template <class T>
  T* take(size_t count) {
    size_t off = (used + 255) & ~(size_t)255;
    size_t need = off + count * sizeof(T);
    if (need > cap || (base == nullptr && count > 0)) return nullptr;
    used = need;
    return (T*)(base + off);
  }
};
inline size_t carve_size(size_t bytes) { return ((bytes + 255) & ~(size_t)255) + 256; }

// ---------------------------------------------------------------- device
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v, unsigned mask = 0xffffffffu) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// Streaming (evict-first) 16-byte loads for values read exactly once.
__device__ __forceinline__ double2 ld_stream(const double2* p) {
  double2 v;
  asm volatile("ld.global.cs.v2.f64 {%0,%1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ float4 ld_stream(const float4* p) {
  float4 v;
  asm volatile("ld.global.cs.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
  double v;
  asm volatile("ld.global.cs.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float v;
  asm volatile("ld.global.cs.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// Bounded spin budget for sync-free kernels: after this many polls of a
// dependency flag the waiter records BILU_ERR_TIMEOUT and returns.
// Polls back off up to 256 ns, so the budget bounds a wait at a few seconds.
constexpr long long kSpinLimit = 1ll << 22;

// Caller-owned home for the level analysis of the lower DAG that BILU(0)
// computes (order[nb+1], lvl_ptr[nb+2], nlev[4]), so that lower triangular
// solves on the factor can reuse it; the host words are filled on return.
struct LevelOut {
  int *order = nullptr, *lvl = nullptr, *nlev = nullptr;
  int h_nlev = 0, h_sched = 0, h_maxdeg = 0;  // levels, solve schedule, largest dependency count
  int h_fsched = 0;                           // recommended factorisation schedule
  // optional match lists of BILU(0)'s updates (bilu0_match_count / _fill):
  // positions mptr[p] .. mptr[p+1] of mpair for block position p
  const int* mptr = nullptr;
  const int2* mpair = nullptr;
};

}  // namespace bilu
