// Fused vector kernels for the Krylov solver (FP64).  On GB300 a dot or
// axpy over many basis vectors runs close to the DFMA limit (1.2 TFLOP/s,
// 1 DFMA per 8 B loaded) rather than HBM, so each kernel reads w once for
// all basis vectors and does no redundant FP64 work; reductions go through
// a fixed number of CTA partials summed in a fixed order (deterministic).
#include "blas1.cuh"

namespace bilu {

namespace {

template <int NV_CAP>
__device__ __forceinline__ void block_reduce_store(double* acc, int nout, double* out) {
  __shared__ double red[kRedThreads / 32][kPartStride];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV_CAP; ++i) {
    if (i < nout) {
      double v = acc[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][i] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < nout) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kRedThreads / 32; ++w) s += red[w][threadIdx.x];
    out[threadIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_multidot(long long n, const double* __restrict__ V,
                                                          long long ldv, int nv,
                                                          const double* __restrict__ w,
                                                          int with_ww,
                                                          double* __restrict__ partial,
                                                          const int* __restrict__ skip_flag) {
  if (skip_flag && *skip_flag == 0) return;
  double acc[kMaxVec + 1];
#pragma unroll
  for (int i = 0; i <= kMaxVec; ++i) acc[i] = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double we = w[e];
#pragma unroll
    for (int i = 0; i < kMaxVec; ++i)
      if (i < nv) acc[i] = fma(V[i * ldv + e], we, acc[i]);
    if (with_ww) acc[kMaxVec] = fma(we, we, acc[kMaxVec]);
  }
  if (with_ww) {
    // move the w.w term next to the nv dots
#pragma unroll
    for (int i = 0; i <= kMaxVec; ++i)
      if (i == nv) acc[i] = acc[kMaxVec];
  }
  block_reduce_store<kMaxVec + 1>(acc, nv + (with_ww ? 1 : 0),
                                  partial + (long long)blockIdx.x * kPartStride);
}

__global__ void __launch_bounds__(kRedThreads) k_multiaxpy_norm(
    long long n, const double* __restrict__ V, long long ldv, int nv,
    const double* __restrict__ coef, double sign, double* __restrict__ w,
    double* __restrict__ partial, const int* __restrict__ skip_flag) {
  if (skip_flag && *skip_flag == 0) return;
  __shared__ double c_s[kMaxVec];
  if (threadIdx.x < kMaxVec) c_s[threadIdx.x] = threadIdx.x < nv ? sign * coef[threadIdx.x] : 0.0;
  __syncthreads();
  double c[kMaxVec];
#pragma unroll
  for (int i = 0; i < kMaxVec; ++i) c[i] = c_s[i];
  double nrm = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double s = w[e];
#pragma unroll
    for (int i = 0; i < kMaxVec; ++i)
      if (i < nv) s = fma(c[i], V[i * ldv + e], s);
    w[e] = s;
    nrm = fma(s, s, nrm);
  }
  if (partial) {
    double a[1] = {nrm};
    block_reduce_store<1>(a, 1, partial + (long long)blockIdx.x * kPartStride);
  }
}

__global__ void k_reduce(const double* __restrict__ partial, int nout, double* __restrict__ out) {
  int i = threadIdx.x;
  if (i >= nout) return;
  double s = 0.0;
  for (int c = 0; c < kRedCTAs; ++c) s += partial[(long long)c * kPartStride + i];
  out[i] = s;
}

__global__ void k_scale_rsqrt(long long n, const double* __restrict__ x,
                              const double* __restrict__ nrm2, double* __restrict__ y) {
  double a = 1.0 / sqrt(*nrm2);
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    y[e] = x[e] * a;
}

__global__ void __launch_bounds__(kRedThreads) k_residual(long long n, const double* __restrict__ b,
                                                          const double* __restrict__ ax,
                                                          double* __restrict__ r,
                                                          double* __restrict__ partial) {
  double nrm = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double v = b[e] - ax[e];
    r[e] = v;
    nrm = fma(v, v, nrm);
  }
  double a[1] = {nrm};
  block_reduce_store<1>(a, 1, partial + (long long)blockIdx.x * kPartStride);
}

}  // namespace

int multidot(long long n, const double* V, long long ldv, int nv, const double* w, bool with_ww,
             double* partial, cudaStream_t st, const int* skip_flag) {
  if (nv < 0 || nv > kMaxVec) return BILU_ERR_ARG;
  k_multidot<<<kRedCTAs, kRedThreads, 0, st>>>(n, V, ldv, nv, w, with_ww ? 1 : 0, partial,
                                               skip_flag);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int multiaxpy_norm(long long n, const double* V, long long ldv, int nv, const double* coef,
                   double sign, double* w, double* partial, const int* skip_flag,
                   cudaStream_t st) {
  if (nv < 0 || nv > kMaxVec) return BILU_ERR_ARG;
  k_multiaxpy_norm<<<kRedCTAs, kRedThreads, 0, st>>>(n, V, ldv, nv, coef, sign, w, partial,
                                                     skip_flag);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int reduce_partials(const double* partial, int nout, double* out, cudaStream_t st) {
  if (nout < 1 || nout > kPartStride) return BILU_ERR_ARG;
  k_reduce<<<1, 64, 0, st>>>(partial, nout, out);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int scale_rsqrt(long long n, const double* x, const double* nrm2, double* y, cudaStream_t st) {
  k_scale_rsqrt<<<kRedCTAs, kRedThreads, 0, st>>>(n, x, nrm2, y);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int residual_norm(long long n, const double* b, const double* ax, double* r, double* partial,
                  cudaStream_t st) {
  k_residual<<<kRedCTAs, kRedThreads, 0, st>>>(n, b, ax, r, partial);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

}  // namespace bilu
