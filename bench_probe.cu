// Pipe-throughput and synchronisation probes for bench.py (measurement
// tooling, built into bench_probe.so beside bench.py; not part of
// libbilu_isai.so).  The first probe sets the compute roofline of the FP64
// kernels: DFMA, DMMA (mma.sync.m8n8k4.f64, the reference's tensor path) and
// FFMA rates of the current GPU, from register-only kernels with one store
// per thread.  The second measures what the level-order kernels are bound
// by: the FP64 issue interval of one SM sub-partition, the store-to-load
// visibility between two SMs and the latency of an L2 hit.  Every wait in
// it is bounded.
//
// Return codes: 0 ok, -1 bad argument, -4 a wait gave up, -5 CUDA error,
// -8 unsupported device.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace probe {

constexpr int kOk = 0, kErrArg = -1, kErrTimeout = -4, kErrCuda = -5, kErrUnsupported = -8;

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? kOk : kErrCuda; }

#define PROBE_TRY_CUDA(call)                 \
  do {                                       \
    if ((call) != cudaSuccess) return kErrCuda; \
  } while (0)

namespace {

constexpr int kProbeIters = 4096;

__global__ void k_probe_dfma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_ffma(float* out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, b);
  float s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_probe_dmma(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = c[0][0] + c[1][1] + c[2][0] + c[3][1];
}

// FP64 issue interval: each warp runs 8 independent DFMA chains on lanes
// < active; thread 0 of each warp records its cycles (clock64).
__global__ void k_probe_dfma_issue(int iters, int active, long long* cyc, double* sink) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = 1.0 + 1e-9 * (threadIdx.x + i);
  const long long t0 = clock64();
  if ((int)(threadIdx.x & 31) < active) {
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int i = 0; i < 8; ++i) x[i] = fma(x[i], 0.999999, 1e-7);
  }
  __syncwarp();
  const long long t1 = clock64();
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if ((threadIdx.x & 31) == 0) cyc[blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)] = t1 - t0;
  if (s == 12345.0) sink[0] = s;  // keeps the chains
}

__device__ __forceinline__ unsigned probe_ld(const unsigned* p, int mode) {
  unsigned v;
  if (mode == 0) asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
  else asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ void probe_st(unsigned* p, unsigned v, int mode) {
  if (mode == 0) asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v));
  else asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v));
}

// Ping-pong between CTA 0 and CTA b (one 32-thread CTA per SM, cooperative
// launch so both are resident): each round one side stores the round number
// and the other polls for it.  out[0] = CTA 0's cycles for all rounds
// (-1 if a wait gave up), out[1..2] = the two SM ids.
__global__ void k_probe_pingpong(int b, int rounds, int mode, unsigned* X, unsigned* Y,
                                 long long* out) {
  if (threadIdx.x != 0 || (blockIdx.x != 0 && (int)blockIdx.x != b)) return;
  unsigned sm;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
  const long long lim = 1ll << 22;
  if (blockIdx.x == 0) {
    out[1] = sm;
    const long long t0 = clock64();
    for (int i = 1; i <= rounds; ++i) {
      probe_st(X, (unsigned)i, mode);
      long long n = 0;
      while (probe_ld(Y, mode) != (unsigned)i)
        if (++n > lim) {
          out[0] = -1;
          return;
        }
    }
    out[0] = clock64() - t0;
  } else {
    out[2] = sm;
    for (int i = 1; i <= rounds; ++i) {
      long long n = 0;
      while (probe_ld(X, mode) != (unsigned)i)
        if (++n > lim) return;
      probe_st(Y, (unsigned)i, mode);
    }
  }
}

// Dependent chain of L2-hit loads (one thread).
__global__ void k_probe_chain(const unsigned* p, int n, long long* out) {
  unsigned i = 0;
  const long long t0 = clock64();
  for (int k = 0; k < n; ++k) asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(i) : "l"(p + i));
  out[0] = clock64() - t0;
  out[1] = i;
}

}  // namespace
}  // namespace probe

using namespace probe;

// h_out[0..2] = DFMA, DMMA, FFMA throughput in TFLOP/s (best of two runs).
extern "C" int probe_rates(double* h_out) {
  if (!h_out) return kErrArg;
  int dev = 0, sms = 0;
  PROBE_TRY_CUDA(cudaGetDevice(&dev));
  PROBE_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = sms * 8, block = 256;
  const double threads = (double)grid * block;
  double* buf = nullptr;
  PROBE_TRY_CUDA(cudaMalloc(&buf, sizeof(double) * (size_t)grid * block));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best[3] = {0, 0, 0};
  int rc = kOk;
  for (int rep = 0; rep < 2 && rc == kOk; ++rep) {
    float ms = 0;
    k_probe_dfma<<<grid, block>>>(buf, 64, 1.0000001, 1e-9);
    cudaEventRecord(e0);
    k_probe_dfma<<<grid, block>>>(buf, kProbeIters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    best[0] = std::max(best[0], 2.0 * 8 * kProbeIters * threads / (ms * 1e9));
    k_probe_dmma<<<grid, block>>>(buf, 16);
    cudaEventRecord(e0);
    k_probe_dmma<<<grid, block>>>(buf, kProbeIters / 4);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    best[1] = std::max(best[1], 2.0 * 8 * 8 * 4 * 4 * (kProbeIters / 4) * (threads / 32) / (ms * 1e9));
    k_probe_ffma<<<grid, block>>>((float*)buf, 64, 1.0000001f, 1e-9f);
    cudaEventRecord(e0);
    k_probe_ffma<<<grid, block>>>((float*)buf, kProbeIters * 8, 1.0000001f, 1e-9f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    best[2] = std::max(best[2], 2.0 * 8 * kProbeIters * 8 * threads / (ms * 1e9));
    rc = cuda_status(cudaGetLastError());
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  for (int i = 0; i < 3; ++i) h_out[i] = best[i];
  return rc;
}

// h_out[0..3]: SM cycles per DFMA warp instruction per SM with 1, 4 and 16
// warps per SM (8 independent chains each) and with 4 warps of which only
// 4 lanes work; h_out[4..5]: one-way store -> load latency in cycles
// between two SMs (relaxed stores and loads), smallest and largest over
// four SM pairs; h_out[6]: the same with st.release / ld.acquire (first
// pair); h_out[7]: cycles of a dependent L2-hit load.
extern "C" int probe_sync(double* h_out) {
  if (!h_out) return kErrArg;
  int dev = 0, sms = 0;
  PROBE_TRY_CUDA(cudaGetDevice(&dev));
  PROBE_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (sms < 2) return kErrUnsupported;
  long long* cyc = nullptr;
  unsigned* words = nullptr;
  double* sink = nullptr;
  const size_t nchain = 1 << 20;
  PROBE_TRY_CUDA(cudaMalloc(&cyc, sizeof(long long) * (size_t)sms * 16));
  PROBE_TRY_CUDA(cudaMalloc(&words, sizeof(unsigned) * nchain));
  PROBE_TRY_CUDA(cudaMalloc(&sink, sizeof(double)));
  int rc = kOk;
  std::vector<long long> h((size_t)sms * 16);
  // issue interval
  const int iters = 4096;
  const int wl[4] = {1, 4, 16, 4}, al[4] = {32, 32, 32, 4};
  for (int c = 0; c < 4 && rc == kOk; ++c) {
    k_probe_dfma_issue<<<sms, 32 * wl[c]>>>(iters, al[c], cyc, sink);
    k_probe_dfma_issue<<<sms, 32 * wl[c]>>>(iters, al[c], cyc, sink);
    rc = cuda_status(cudaDeviceSynchronize());
    if (rc != kOk) break;
    rc = cuda_status(cudaMemcpy(h.data(), cyc, sizeof(long long) * (size_t)sms * wl[c],
                                cudaMemcpyDeviceToHost));
    long long mx = 1;
    for (int i = 0; i < sms * wl[c]; ++i) mx = std::max(mx, h[i]);
    h_out[c] = (double)mx / ((double)iters * 8 * wl[c]);
  }
  // ping-pong: CTA 0 against CTAs a quarter, half, three quarters of the grid away and 1
  long long* out = cyc;
  const int rounds = 2000;
  const int bs_[4] = {1, sms / 4, sms / 2, (3 * sms) / 4};
  double lo = 1e30, hi = 0, acq = 0;
  for (int mode = 0; mode < 2 && rc == kOk; ++mode) {
    for (int k = 0; k < (mode == 0 ? 4 : 1) && rc == kOk; ++k) {
      unsigned* X = words;
      unsigned* Y = words + 4096;  // 16 KB apart
      int b = std::max(1, std::min(sms - 1, bs_[k])), r = rounds, m = mode;
      rc = cuda_status(cudaMemset(words, 0, sizeof(unsigned) * 8192));
      if (rc == kOk) rc = cuda_status(cudaMemset(out, 0, sizeof(long long) * 3));
      void* args[] = {&b, &r, &m, &X, &Y, &out};
      if (rc == kOk)
        rc = cuda_status(cudaLaunchCooperativeKernel((const void*)k_probe_pingpong, dim3(sms),
                                                     dim3(32), args, 0, 0));
      if (rc == kOk) rc = cuda_status(cudaDeviceSynchronize());
      long long o[3] = {0, 0, 0};
      if (rc == kOk) rc = cuda_status(cudaMemcpy(o, out, sizeof(o), cudaMemcpyDeviceToHost));
      if (rc != kOk) break;
      if (o[0] <= 0) {
        rc = kErrTimeout;
        break;
      }
      const double one_way = (double)o[0] / rounds / 2;
      if (mode == 0) {
        lo = std::min(lo, one_way);
        hi = std::max(hi, one_way);
      } else {
        acq = one_way;
      }
    }
  }
  h_out[4] = lo;
  h_out[5] = hi;
  h_out[6] = acq;
  // dependent L2-hit loads: p[i] = i + 32 (128-byte stride) over 4 MB
  if (rc == kOk) {
    std::vector<unsigned> ring(nchain);
    for (size_t i = 0; i < nchain; ++i) ring[i] = (unsigned)((i + 32) % nchain);
    rc = cuda_status(cudaMemcpy(words, ring.data(), sizeof(unsigned) * nchain,
                                cudaMemcpyHostToDevice));
    for (int rep = 0; rep < 2 && rc == kOk; ++rep) {
      k_probe_chain<<<1, 1>>>(words, 20000, cyc);
      rc = cuda_status(cudaDeviceSynchronize());
    }
    long long o = 0;
    if (rc == kOk) rc = cuda_status(cudaMemcpy(&o, cyc, sizeof(o), cudaMemcpyDeviceToHost));
    h_out[7] = (double)o / 20000;
  }
  cudaFree(cyc);
  cudaFree(words);
  cudaFree(sink);
  return rc;
}
