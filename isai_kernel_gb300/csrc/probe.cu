// Pipe-throughput probe used to set the compute roofline of the FP64
// kernels: DFMA, DMMA (mma.sync.m8n8k4.f64, the reference's tensor path) and
// FFMA rates of the current GPU.  Register-only kernels, one store per thread.
#include <algorithm>

#include "common.cuh"

namespace bilu {
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

}  // namespace
}  // namespace bilu

using namespace bilu;

// h_out[0..2] = DFMA, DMMA, FFMA throughput in TFLOP/s (best of two runs).
extern "C" int bilu_probe_rates(double* h_out) {
  if (!h_out) return BILU_ERR_ARG;
  int dev = 0, sms = 0;
  BILU_TRY_CUDA(cudaGetDevice(&dev));
  BILU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = sms * 8, block = 256;
  const double threads = (double)grid * block;
  double* buf = nullptr;
  BILU_TRY_CUDA(cudaMalloc(&buf, sizeof(double) * (size_t)grid * block));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best[3] = {0, 0, 0};
  int rc = BILU_OK;
  for (int rep = 0; rep < 2 && rc == BILU_OK; ++rep) {
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
