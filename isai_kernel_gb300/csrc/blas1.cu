// Fused vector kernels for the Krylov solver (FP64).  On GB300 a dot or
// axpy over many basis vectors runs close to the DFMA limit (1.2 TFLOP/s,
// 1 DFMA per 8 B loaded) rather than HBM, so each kernel reads w once for
// all basis vectors and does no redundant FP64 work; reductions go through
// a fixed number of CTA partials summed in a fixed order (deterministic).
#include "blas1.cuh"

namespace bilu {

namespace {

// Sum NOUT per-thread values over the CTA; thread i < NOUT writes sum i.
template <int NOUT>
__device__ __forceinline__ void block_reduce_store(const double (&acc)[NOUT > 0 ? NOUT : 1],
                                                   double* out) {
  __shared__ double red[kRedThreads / 32][kPartStride];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NOUT; ++i) {
    double v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < NOUT) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kRedThreads / 32; ++w) s += red[w][threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// h[i] = V_i . w for i < NV (and w.w at index NV when WW): w is read once,
// each basis vector once; one DFMA per loaded basis element.
template <int NV, bool WW>
__global__ void __launch_bounds__(kRedThreads) k_multidot(long long n, const double* __restrict__ V,
                                                          long long ldv,
                                                          const double* __restrict__ w,
                                                          double* __restrict__ partial,
                                                          const int* __restrict__ skip_flag) {
  if (skip_flag && *skip_flag == 0) return;
  constexpr int NOUT = NV + (WW ? 1 : 0);
  double acc[NOUT > 0 ? NOUT : 1];
#pragma unroll
  for (int i = 0; i < NOUT; ++i) acc[i] = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double we = w[e];
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] = fma(__ldcs(V + i * ldv + e), we, acc[i]);
    if (WW) acc[NOUT - 1] = fma(we, we, acc[NOUT - 1]);
  }
  block_reduce_store<NOUT>(acc, partial + (long long)blockIdx.x * kPartStride);
}

// w += sign * sum_i coef[i] V_i, with ||w_new||^2 partials.
template <int NV>
__global__ void __launch_bounds__(kRedThreads) k_multiaxpy_norm(
    long long n, const double* __restrict__ V, long long ldv, const double* __restrict__ coef,
    double sign, double* __restrict__ w, double* __restrict__ partial,
    const int* __restrict__ skip_flag) {
  if (skip_flag && *skip_flag == 0) return;
  double c[NV > 0 ? NV : 1];
#pragma unroll
  for (int i = 0; i < NV; ++i) c[i] = sign * __ldg(coef + i);
  double nrm = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double s = w[e];
#pragma unroll
    for (int i = 0; i < NV; ++i) s = fma(c[i], __ldcs(V + i * ldv + e), s);
    w[e] = s;
    nrm = fma(s, s, nrm);
  }
  if (partial) {
    double a[1] = {nrm};
    block_reduce_store<1>(a, partial + (long long)blockIdx.x * kPartStride);
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
                              const double* __restrict__ nrm2, double* __restrict__ y,
                              float* __restrict__ y32) {
  double a = 1.0 / sqrt(*nrm2);
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double v = x[e] * a;
    y[e] = v;
    if (y32) y32[e] = __double2float_rn(v);
  }
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
  block_reduce_store<1>(a, partial + (long long)blockIdx.x * kPartStride);
}

template <int NV>
void launch_multidot(long long n, const double* V, long long ldv, const double* w, bool ww,
                     double* partial, cudaStream_t st, const int* skip) {
  if (ww)
    k_multidot<NV, true><<<kRedCTAs, kRedThreads, 0, st>>>(n, V, ldv, w, partial, skip);
  else
    k_multidot<NV, false><<<kRedCTAs, kRedThreads, 0, st>>>(n, V, ldv, w, partial, skip);
}

template <int NV>
void launch_multiaxpy(long long n, const double* V, long long ldv, const double* coef,
                      double sign, double* w, double* partial, const int* skip, cudaStream_t st) {
  k_multiaxpy_norm<NV><<<kRedCTAs, kRedThreads, 0, st>>>(n, V, ldv, coef, sign, w, partial, skip);
}

#define BILU_NV_CASES(F, ...)                                                        \
  switch (nv) {                                                                      \
    case 0: F<0>(__VA_ARGS__); break;   case 1: F<1>(__VA_ARGS__); break;            \
    case 2: F<2>(__VA_ARGS__); break;   case 3: F<3>(__VA_ARGS__); break;            \
    case 4: F<4>(__VA_ARGS__); break;   case 5: F<5>(__VA_ARGS__); break;            \
    case 6: F<6>(__VA_ARGS__); break;   case 7: F<7>(__VA_ARGS__); break;            \
    case 8: F<8>(__VA_ARGS__); break;   case 9: F<9>(__VA_ARGS__); break;            \
    case 10: F<10>(__VA_ARGS__); break; case 11: F<11>(__VA_ARGS__); break;          \
    case 12: F<12>(__VA_ARGS__); break; case 13: F<13>(__VA_ARGS__); break;          \
    case 14: F<14>(__VA_ARGS__); break; case 15: F<15>(__VA_ARGS__); break;          \
    case 16: F<16>(__VA_ARGS__); break; case 17: F<17>(__VA_ARGS__); break;          \
    case 18: F<18>(__VA_ARGS__); break; case 19: F<19>(__VA_ARGS__); break;          \
    case 20: F<20>(__VA_ARGS__); break; case 21: F<21>(__VA_ARGS__); break;          \
    case 22: F<22>(__VA_ARGS__); break; case 23: F<23>(__VA_ARGS__); break;          \
    case 24: F<24>(__VA_ARGS__); break; case 25: F<25>(__VA_ARGS__); break;          \
    case 26: F<26>(__VA_ARGS__); break; case 27: F<27>(__VA_ARGS__); break;          \
    case 28: F<28>(__VA_ARGS__); break; case 29: F<29>(__VA_ARGS__); break;          \
    case 30: F<30>(__VA_ARGS__); break; case 31: F<31>(__VA_ARGS__); break;          \
    case 32: F<32>(__VA_ARGS__); break;                                              \
    default: return BILU_ERR_ARG;                                                    \
  }

// One modified Gram-Schmidt step fused with the next one's dot product:
// w -= h_prev * v_prev (h_prev read from device memory), then the partial of
// v_next . w (or w . w).  The basis vectors stream through with evict-first
// loads; w (one vector, 67 MB at 128^3) stays in the L2 (a sweep reads
// only the two basis vectors from DRAM), which leaves the two DFMAs per
// element as the bound.  Elements go in pairs through 16-byte accesses (the
// basis stride is a multiple of 32 elements and every vector starts on a
// 256-byte boundary) into two independent accumulators, so that a thread
// has two FMA chains in flight.  The CTA that finishes last sums the CTA
// partials in index order, so the result does not depend on which CTA
// that is.
__global__ void __launch_bounds__(kRedThreads, kSweepCTAs / 152) k_mgs_sweep(
    long long n, const double* __restrict__ vp, const double* __restrict__ hp,
    const double* __restrict__ vn, double* __restrict__ w, double* __restrict__ partial,
    unsigned* counter, double* out) {
  // launched as a programmatic dependent of the previous sweep: let the
  // next sweep's CTAs be scheduled during this one's reduction tail, and
  // wait here until the previous grid has finished and its writes (w, h,
  // the counter reset) are visible
  asm volatile("griddepcontrol.launch_dependents;");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const double h = vp ? -__ldcg(hp) : 0.0;
  double acc0 = 0.0, acc1 = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double2* w2 = reinterpret_cast<double2*>(w);
  const double2* vp2 = reinterpret_cast<const double2*>(vp);
  const double2* vn2 = reinterpret_cast<const double2*>(vn);
  for (long long e = tid; e < (n >> 1); e += stride) {
    double2 we = __ldcg(w2 + e);  // L2: w was written by the previous sweep
    if (vp) {
      const double2 p = __ldcs(vp2 + e);
      we.x = fma(h, p.x, we.x);
      we.y = fma(h, p.y, we.y);
      w2[e] = we;
    }
    const double2 o = vn ? __ldcs(vn2 + e) : we;
    acc0 = fma(o.x, we.x, acc0);
    acc1 = fma(o.y, we.y, acc1);
  }
  if ((n & 1) && tid == 0) {  // odd length: the last element
    double we = __ldcg(w + n - 1);
    if (vp) {
      we = fma(h, __ldcs(vp + n - 1), we);
      w[n - 1] = we;
    }
    const double o = vn ? __ldcs(vn + n - 1) : we;
    acc0 = fma(o, we, acc0);
  }
  double acc = acc0 + acc1;
  __shared__ double red[kRedThreads / 32];
  __shared__ bool last;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kRedThreads / 32; ++i) s += red[i];
    partial[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) s += __ldcg(partial + c);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < kRedThreads / 32; ++i) t += red[i];
    *out = t;
    *counter = 0u;
  }
}


// FP32 form of k_mgs_sweep for the inner solver: four elements per 16-byte
// access, FP32 products and sums per thread, FP64 from the warp sums on.
// w (33.5 MB at 128^3) and vn stay in the L2 (vn is read with ld.global.cg,
// so the next sweep finds it there as vp); vp streams with evict-first
// loads, the last use of that basis vector in this step.
__global__ void __launch_bounds__(kRedThreads, kSweepCTAs / 152) k_mgs_sweep_f32(
    long long n, const float* __restrict__ vp, const double* __restrict__ hp,
    const float* __restrict__ vn, float* __restrict__ w, double* __restrict__ partial,
    unsigned* counter, double* out) {
  asm volatile("griddepcontrol.launch_dependents;");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const float h = vp ? -(float)__ldcg(hp) : 0.0f;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float4* w4 = reinterpret_cast<float4*>(w);
  const float4* vp4 = reinterpret_cast<const float4*>(vp);
  const float4* vn4 = reinterpret_cast<const float4*>(vn);
  const long long n4 = n >> 2;
  for (long long e = tid; e < n4; e += stride) {
    float4 we = __ldcg(w4 + e);
    if (vp) {
      const float4 p = __ldcs(vp4 + e);
      we.x = fmaf(h, p.x, we.x);
      we.y = fmaf(h, p.y, we.y);
      we.z = fmaf(h, p.z, we.z);
      we.w = fmaf(h, p.w, we.w);
      w4[e] = we;
    }
    const float4 o = vn ? __ldcg(vn4 + e) : we;
    a0 = fmaf(o.x, we.x, a0);
    a1 = fmaf(o.y, we.y, a1);
    a2 = fmaf(o.z, we.z, a2);
    a3 = fmaf(o.w, we.w, a3);
  }
  if (tid < (n & 3)) {  // the last n % 4 elements
    const long long e = (n4 << 2) + tid;
    float we = __ldcg(w + e);
    if (vp) {
      we = fmaf(h, __ldcs(vp + e), we);
      w[e] = we;
    }
    const float o = vn ? __ldcg(vn + e) : we;
    a0 = fmaf(o, we, a0);
  }
  float accf = (a0 + a1) + (a2 + a3);
  __shared__ double red[kRedThreads / 32];
  __shared__ bool last;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) accf += __shfl_xor_sync(0xffffffffu, accf, o);
  if (lane == 0) red[warp] = (double)accf;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kRedThreads / 32; ++i) s += red[i];
    partial[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) s += __ldcg(partial + c);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < kRedThreads / 32; ++i) t += red[i];
    *out = t;
    *counter = 0u;
  }
}

__global__ void k_scale_rsqrt_f32(long long n, const float* __restrict__ x,
                                  const double* __restrict__ nrm2, float* __restrict__ y) {
  __shared__ float a_s;
  if (threadIdx.x == 0) {
    const double v = *nrm2;
    a_s = v > 0.0 ? (float)(1.0 / sqrt(v)) : 0.0f;
  }
  __syncthreads();
  const float a = a_s;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n4 = n >> 2;
  const float4* x4 = reinterpret_cast<const float4*>(x);
  float4* y4 = reinterpret_cast<float4*>(y);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
    float4 v = x4[e];
    v.x *= a;
    v.y *= a;
    v.z *= a;
    v.w *= a;
    y4[e] = v;
  }
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (n & 3)) y[(n4 << 2) + t] = x[(n4 << 2) + t] * a;
}

// One thread: Givens QR of the inner Hessenberg matrix and the triangular
// solve, as the host does for the outer one (the same rotation formulas).
__global__ void k_inner_lsq(int k, const double* __restrict__ Hraw, const double* __restrict__ ww,
                            double* __restrict__ y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double H[kMaxVec + 1][kMaxVec];
  double cs[kMaxVec], sn[kMaxVec], g[kMaxVec + 1];
  int steps = k;
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i <= j; ++i) H[i][j] = Hraw[i * k + j];
    const double hn = sqrt(ww[j]);
    H[j + 1][j] = hn;
    if (hn == 0.0) {
      steps = j + 1;
      break;
    }
  }
  g[0] = 1.0;
  for (int j = 0; j < steps; ++j) {
    for (int i = 0; i < j; ++i) {
      const double a = H[i][j], b = H[i + 1][j];
      H[i][j] = cs[i] * a + sn[i] * b;
      H[i + 1][j] = -sn[i] * a + cs[i] * b;
    }
    const double a = H[j][j], b = H[j + 1][j];
    const double den = sqrt(a * a + b * b);
    cs[j] = den != 0.0 ? a / den : 1.0;
    sn[j] = den != 0.0 ? b / den : 0.0;
    H[j][j] = cs[j] * a + sn[j] * b;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
  }
  for (int i = steps - 1; i >= 0; --i) {
    double v = g[i];
    for (int l = i + 1; l < steps; ++l) v -= H[i][l] * y[l];
    y[i] = H[i][i] != 0.0 ? v / H[i][i] : 0.0;
  }
  for (int i = steps; i < k; ++i) y[i] = 0.0;
}

template <int K>
__global__ void __launch_bounds__(kRedThreads) k_combine_f32(long long n,
                                                             const float* __restrict__ Q,
                                                             long long ldq,
                                                             const double* __restrict__ y,
                                                             double* __restrict__ z) {
  __shared__ float ys[K > 0 ? K : 1];
  if (threadIdx.x < K) ys[threadIdx.x] = (float)y[threadIdx.x];
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n4 = n >> 2;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const float4 q = __ldcs(reinterpret_cast<const float4*>(Q + i * ldq) + e);
      s.x = fmaf(ys[i], q.x, s.x);
      s.y = fmaf(ys[i], q.y, s.y);
      s.z = fmaf(ys[i], q.z, s.z);
      s.w = fmaf(ys[i], q.w, s.w);
    }
    double2* z2 = reinterpret_cast<double2*>(z + (e << 2));
    z2[0] = make_double2((double)s.x, (double)s.y);
    z2[1] = make_double2((double)s.z, (double)s.w);
  }
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (n & 3)) {
    const long long e = (n4 << 2) + t;
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < K; ++i) s = fmaf(ys[i], Q[i * ldq + e], s);
    z[e] = (double)s;
  }
}

template <int K>
void launch_combine(long long n, const float* Q, long long ldq, const double* y, double* z,
                    cudaStream_t st) {
  k_combine_f32<K><<<kRedCTAs, kRedThreads, 0, st>>>(n, Q, ldq, y, z);
}

}  // namespace

int multidot(long long n, const double* V, long long ldv, int nv, const double* w, bool with_ww,
             double* partial, cudaStream_t st, const int* skip_flag) {
  BILU_NV_CASES(launch_multidot, n, V, ldv, w, with_ww, partial, st, skip_flag);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int multiaxpy_norm(long long n, const double* V, long long ldv, int nv, const double* coef,
                   double sign, double* w, double* partial, const int* skip_flag,
                   cudaStream_t st) {
  BILU_NV_CASES(launch_multiaxpy, n, V, ldv, coef, sign, w, partial, skip_flag, st);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int reduce_partials(const double* partial, int nout, double* out, cudaStream_t st) {
  if (nout < 1 || nout > kPartStride) return BILU_ERR_ARG;
  k_reduce<<<1, 64, 0, st>>>(partial, nout, out);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int scale_rsqrt(long long n, const double* x, const double* nrm2, double* y, cudaStream_t st,
                float* y32) {
  k_scale_rsqrt<<<kRedCTAs, kRedThreads, 0, st>>>(n, x, nrm2, y, y32);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int mgs_sweep(long long n, const double* vp, const double* hp, const double* vn, double* w,
              double* partial, unsigned* counter, double* out, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kSweepCTAs);
  cfg.blockDim = dim3(kRedThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BILU_TRY_CUDA(cudaLaunchKernelEx(&cfg, k_mgs_sweep, n, vp, hp, vn, w, partial, counter, out));
  __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED);
  return BILU_OK;
}

int mgs_sweep_f32(long long n, const float* vp, const double* hp, const float* vn, float* w,
                  double* partial, unsigned* counter, double* out, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kSweepCTAs);
  cfg.blockDim = dim3(kRedThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BILU_TRY_CUDA(
      cudaLaunchKernelEx(&cfg, k_mgs_sweep_f32, n, vp, hp, vn, w, partial, counter, out));
  __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED);
  return BILU_OK;
}

int scale_rsqrt_f32(long long n, const float* x, const double* nrm2, float* y, cudaStream_t st) {
  k_scale_rsqrt_f32<<<kRedCTAs, kRedThreads, 0, st>>>(n, x, nrm2, y);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int inner_lsq(int k, const double* H, const double* ww, double* y, cudaStream_t st) {
  if (k < 1 || k > kMaxVec) return BILU_ERR_ARG;
  k_inner_lsq<<<1, 32, 0, st>>>(k, H, ww, y);
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int combine_f32(long long n, const float* Q, long long ldq, int k, const double* y, double* z,
                cudaStream_t st) {
  const int nv = k;
  BILU_NV_CASES(launch_combine, n, Q, ldq, y, z, st);
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
