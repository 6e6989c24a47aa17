// Fused vector kernels for the Krylov solver (FP64).  On GB300 a dot or
// axpy over many basis vectors runs close to the DFMA limit (1.2 TFLOP/s,
// 1 DFMA per 8 B loaded) rather than HBM, so each kernel reads w once for
// all basis vectors and does no redundant FP64 work; reductions go through
// a fixed number of CTA partials summed in a fixed order (deterministic).
#include "blas1.cuh"
#include "gridsync.cuh"

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

// Givens QR of the inner Hessenberg matrix and the triangular solve, with
// the host's rotation formulas for the outer one, on one warp: lane j owns
// column j; rotation q is formed from column q once rotations 0..q-1 have
// reached it and is then applied to the columns right of it by their lanes
// at once, so every element sees the same operations in the same order as
// a column-by-column loop (the same bits); the back substitution runs in
// lane 0.
__global__ void k_inner_lsq(int k, const double* __restrict__ Hraw, const double* __restrict__ ww,
                            double* __restrict__ y) {
  __shared__ double H[kMaxVec + 1][kMaxVec];
  __shared__ double g[kMaxVec + 1];
  const int j = threadIdx.x;
  if (blockIdx.x != 0 || j >= 32) return;
  // the steps end at the first zero subdiagonal entry
  const bool zero = j < k && ww[j] == 0.0;
  const unsigned zmask = __ballot_sync(0xffffffffu, zero);
  const int steps = zmask ? __ffs(zmask) : k;
  if (j < steps) {
    for (int i = 0; i <= j; ++i) H[i][j] = Hraw[i * k + j];
    H[j + 1][j] = sqrt(ww[j]);
  }
  if (j == 0) g[0] = 1.0;
  __syncwarp();
  for (int q = 0; q < steps; ++q) {
    const double a = H[q][q], b = H[q + 1][q];
    const double den = sqrt(a * a + b * b);
    const double cs = den != 0.0 ? a / den : 1.0;
    const double sn = den != 0.0 ? b / den : 0.0;
    __syncwarp();
    if (j == q) {
      H[q][q] = cs * a + sn * b;
      g[q + 1] = -sn * g[q];
      g[q] = cs * g[q];
    } else if (j > q && j < steps) {
      const double c0 = H[q][j], c1 = H[q + 1][j];
      H[q][j] = cs * c0 + sn * c1;
      H[q + 1][j] = -sn * c0 + cs * c1;
    }
    __syncwarp();
  }
  if (j == 0) {
    for (int i = steps - 1; i >= 0; --i) {
      double v = g[i];
      for (int l = i + 1; l < steps; ++l) v -= H[i][l] * y[l];
      y[i] = H[i][i] != 0.0 ? v / H[i][i] : 0.0;
    }
    for (int i = steps; i < k; ++i) y[i] = 0.0;
  }
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


// ---------------------------------------------------------------------------
// Whole modified Gram-Schmidt step in one cooperative launch: sweeps
// i = 0 .. j+1 over the same slice of w per CTA, sweep i applying
// h_{i-1} v_{i-1} and taking v_i . w (the last one w . w), then
// v_{j+1} = w / ||w|| (and its FP32 copy).  Between sweeps
// a counting grid barrier replaces the kernel boundary: each CTA writes its
// partial sum, meets the others at the barrier, and then every CTA adds all
// partials in index order (warp 0, fixed lane strides and shuffle tree), so
// every CTA holds the same h_i bit for bit and the result does not depend on
// timing.  The partials alternate between two halves of the buffer: a CTA
// writes sweep i+1's partial only after barrier i, and sweep i+2 (same half
// as i) only after barrier i+1, which every CTA reaches after it has read
// sweep i's partials.  A barrier that times out sets the error word and
// every CTA returns.  Memory traffic at 128^3 (ncu, one step of 17 sweeps):
// FP32 reads each basis vector once from DRAM (w and the previous basis
// vector are L2 hits); FP64 moves ~2.8 vectors a sweep (3.17 GB a step):
// w (67 MB) does not stay fully in the L2 beside the streamed basis
// vectors, even with evict-last hints on w; held there by an L2 persisting
// window it costs 3% less a sweep, which is then bound by the DFMA pipe's
// issue and the per-sweep synchronisation rather than by HBM.
template <class T>
struct MgsVec;
template <>
struct MgsVec<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static V ldcg(const V* p) { return __ldcg(p); }
  __device__ static V ldcs(const V* p) { return __ldcs(p); }
  // v_i streams through with evict-first loads: w (67 MB at 128^3) and a
  // kept v_i would not both fit in the L2
  __device__ static V ldnext(const V* p) { return __ldcs(p); }
  __device__ static void axpy(double h, const V& p, V& w) {
    w.x = fma(h, p.x, w.x);
    w.y = fma(h, p.y, w.y);
  }
  __device__ static void dot(const V& o, const V& w, double (&a)[4]) {
    a[0] = fma(o.x, w.x, a[0]);
    a[1] = fma(o.y, w.y, a[1]);
  }
  __device__ static void scale(V& v, double a) {
    v.x *= a;
    v.y *= a;
  }
};
template <>
struct MgsVec<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static V ldcg(const V* p) { return __ldcg(p); }
  __device__ static V ldcs(const V* p) { return __ldcs(p); }
  // v_i stays in the L2 for the next sweep, which reads it as v_{i-1}
  // (w and v_i take 67 MB at 128^3)
  __device__ static V ldnext(const V* p) { return __ldcg(p); }
  __device__ static void axpy(float h, const V& p, V& w) {
    w.x = fmaf(h, p.x, w.x);
    w.y = fmaf(h, p.y, w.y);
    w.z = fmaf(h, p.z, w.z);
    w.w = fmaf(h, p.w, w.w);
  }
  __device__ static void dot(const V& o, const V& w, float (&a)[4]) {
    a[0] = fmaf(o.x, w.x, a[0]);
    a[1] = fmaf(o.y, w.y, a[1]);
    a[2] = fmaf(o.z, w.z, a[2]);
    a[3] = fmaf(o.w, w.w, a[3]);
  }
  __device__ static void scale(V& v, float a) {
    v.x *= a;
    v.y *= a;
    v.z *= a;
    v.w *= a;
  }
};

// 512 threads, two CTAs per SM: half the partials and barrier arrivals of
// 256-thread CTAs at the same occupancy (measured 3-6% faster a sweep at
// 128^3, FP64 and FP32)
constexpr int kStepThreads = 512;
constexpr int kStepPerSM = 2;
// FP64 sweeps stage their loads through shared memory with cp.async,
// kStepStages element iterations ahead of the arithmetic (each thread reads
// back only its own slots): an FP64 sweep stalls on memory latency with the
// FP64 pipe ~70% busy, and the registers of a deeper unroll are not there at
// two CTAs of 512 threads per SM (41.2 -> 38.0 us a sweep at 128^3; the FP32
// sweep, bound by synchronisation and L2 traffic, is slower this way).
constexpr int kStepStages = 3;
constexpr size_t kStepStageBytes = (size_t)kStepStages * 3 * kStepThreads * 16;

__device__ __forceinline__ unsigned long long l2_policy_evict_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long l2_policy_evict_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// 16 bytes global -> shared, asynchronous, through the L2 only
__device__ __forceinline__ void cp_async16(void* smem, const void* g, unsigned long long pol) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(sa), "l"(g),
               "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T>
__global__ void __launch_bounds__(kStepThreads, kStepPerSM) k_mgs_step(
    long long n, const T* __restrict__ V, long long ldv, int j, T* __restrict__ w,
    double* __restrict__ hout, int hstride, double* __restrict__ wwout,
    double* __restrict__ partial, GridSync gs, T* __restrict__ vnext,
    float* __restrict__ vnext32) {
  using M = MgsVec<T>;
  using VT = typename M::V;
  constexpr int W = M::W;
  // sums run in the kernel's own precision: on GB300 every FP64 add (and
  // every FP32 <-> FP64 conversion) takes the FP64 pipe, which the FP64
  // kernel needs for its DFMAs and the FP32 kernel should not touch
  __shared__ T red_s[kStepThreads];
  __shared__ T h_s;
  unsigned passed = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int G = (int)gridDim.x;
  const long long stride = (long long)G * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nv = n / W;     // whole vectors
  const long long tail = nv * W;  // first element of the scalar tail
  VT* wv = reinterpret_cast<VT*>(w);
  // FP64 staging: w kept in the L2 as long as it fits, the basis vectors
  // streamed through
  unsigned long long pol_w = 0, pol_v = 0;
  if constexpr (sizeof(T) == 8) {
    pol_w = l2_policy_evict_last();
    pol_v = l2_policy_evict_first();
  }
  T h = T(0);
  for (int i = 0; i <= j + 1; ++i) {
    const T* vp = i > 0 ? V + (long long)(i - 1) * ldv : nullptr;
    const T* vn = i <= j ? V + (long long)i * ldv : nullptr;
    const T hn = -h;
    T a[4] = {T(0), T(0), T(0), T(0)};
    const VT* vpv = reinterpret_cast<const VT*>(vp);
    const VT* vnv = reinterpret_cast<const VT*>(vn);
    if constexpr (sizeof(T) == 8) {
      // iteration k of this thread: element tid + k * stride; slot k % S of
      // the thread's w, v_{i-1} and v_i stages, loaded S - 1 iterations ahead
      constexpr int S = kStepStages;
      extern __shared__ __align__(16) unsigned char step_stage[];
      VT* stage = reinterpret_cast<VT*>(step_stage);  // [S][3][kStepThreads]
      const long long K = tid < nv ? (nv - tid + stride - 1) / stride : 0;
      auto issue = [&](long long k) {
        const long long e = tid + k * stride;
        VT* sl = stage + (int)(k % S) * 3 * kStepThreads + threadIdx.x;
        cp_async16(sl, wv + e, pol_w);
        if (vpv) cp_async16(sl + kStepThreads, vpv + e, pol_v);
        if (vnv) cp_async16(sl + 2 * kStepThreads, vnv + e, pol_v);
      };
#pragma unroll
      for (int k = 0; k < S - 1; ++k) {
        if (k < K) issue(k);
        cp_async_commit();
      }
      for (long long k = 0; k < K; ++k) {
        if (k + S - 1 < K) issue(k + S - 1);
        cp_async_commit();
        cp_async_wait<S - 1>();  // iteration k's group has landed
        const VT* sl = stage + (int)(k % S) * 3 * kStepThreads + threadIdx.x;
        VT we = sl[0];
        if (vpv) {
          M::axpy(hn, sl[kStepThreads], we);
          wv[tid + k * stride] = we;
        }
        M::dot(vnv ? sl[2 * kStepThreads] : we, we, a);
      }
      cp_async_wait<0>();
      // the next sweep's first stages read v_i (as v_{i-1}) and v_{i+1}: start
      // those lines towards the L2 before the grid barrier (1-2% a sweep)
      for (long long k = 0; k < S - 1 && k < K; ++k) {
        const long long e = tid + k * stride;
        if (vnv) asm volatile("prefetch.global.L2 [%0];" ::"l"(vnv + e));
        if (i + 1 <= j)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(
              reinterpret_cast<const VT*>(V + (long long)(i + 1) * ldv) + e));
      }
    } else {
      // two elements' loads in flight per thread
#pragma unroll 2
      for (long long e = tid; e < nv; e += stride) {
        VT we = M::ldcg(wv + e);
        if (vp) {
          M::axpy(hn, M::ldcs(vpv + e), we);
          wv[e] = we;
        }
        M::dot(vn ? M::ldnext(vnv + e) : we, we, a);
      }
    }
    if (tid < n - tail) {  // the last n % W elements
      const long long e = tail + tid;
      T we = __ldcg(w + e);
      if (vp) {
        we = fma(hn, __ldcs(vp + e), we);
        w[e] = we;
      }
      const T o = vn ? __ldcg(vn + e) : we;
      a[0] = fma(o, we, a[0]);
    }
    // CTA partial, fixed order: the threads' sums through shared memory,
    // warp 0 adds eight per lane and then the lanes by a shuffle tree
    red_s[threadIdx.x] = (a[0] + a[1]) + (a[2] + a[3]);
    __syncthreads();
    T* part = reinterpret_cast<T*>(partial) + (long long)(i & 1) * kStepMaxCTAs;
    if (warp == 0) {
      T t = T(0);
#pragma unroll
      for (int q = 0; q < kStepThreads / 32; ++q) t += red_s[lane + 32 * q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) part[blockIdx.x] = t;  // lane 0 of warp 0 arrives at the barrier
    }
    if (!grid_sync_count(gs, passed)) return;
    // every CTA adds all partials in the same order
    if constexpr (sizeof(T) == 8) {
      // FP64: warp 0 alone (the adds take the FP64 pipe), lane l taking
      // partials l, l + 32, ... in ascending order, eight loads in flight,
      // then the shuffle tree
      if (warp == 0) {
        T t = T(0);
        for (int c0 = 0; c0 < G; c0 += 8 * 32) {
          T v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int c = c0 + lane + 32 * u;
            v[u] = c < G ? __ldcg(part + c) : T(0);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) t += v[u];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) h_s = t;
      }
    } else {
      // FP32: every thread loads its few partials at once (one L2 round
      // trip), the warps' trees, then warp 0 adds the eight warp sums
      T t = T(0);
      for (int c = threadIdx.x; c < G; c += kStepThreads) t += __ldcg(part + c);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      __syncthreads();  // red_s is free again (warp 0 read it before the barrier)
      if (lane == 0) red_s[warp] = t;
      __syncthreads();
      if (threadIdx.x == 0) {
        T u = T(0);
#pragma unroll
        for (int q = 0; q < kStepThreads / 32; ++q) u += red_s[q];
        h_s = u;
      }
    }
    __syncthreads();
    h = h_s;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (i <= j) hout[(long long)i * hstride] = (double)h;
      else *wwout = (double)h;
    }
  }
  // v_{j+1} = w / ||w|| over this CTA's slice (zeros when ||w|| = 0)
  if (vnext) {
    const T s = h > T(0) ? T(1) / sqrt(h) : T(0);
    VT* out = reinterpret_cast<VT*>(vnext);
    for (long long e = tid; e < nv; e += stride) {
      VT v = M::ldcg(wv + e);
      M::scale(v, s);
      out[e] = v;
      if (vnext32) {
        const T* vs = reinterpret_cast<const T*>(&v);
#pragma unroll
        for (int q = 0; q < W; ++q) vnext32[e * W + q] = (float)vs[q];
      }
    }
    if (tid < n - tail) {
      const long long e = tail + tid;
      const T v = __ldcg(w + e) * s;
      vnext[e] = v;
      if (vnext32) vnext32[e] = (float)v;
    }
  }
  grid_exit_count(gs);
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

template <class T>
int mgs_step_t(long long n, const T* V, long long ldv, int j, T* w, double* hout, int hstride,
               double* wwout, double* partial, unsigned* words, T* vnext, float* vnext32,
               cudaStream_t st) {
  static int grid = 0;
  const size_t smem = sizeof(T) == 8 ? kStepStageBytes : 0;
  if (!grid) {
    int per = 0, dev = 0, sms = 0;
    BILU_TRY_CUDA(cudaGetDevice(&dev));
    BILU_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (smem)
      BILU_TRY_CUDA(cudaFuncSetAttribute(k_mgs_step<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BILU_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mgs_step<T>,
                                                                kStepThreads, smem));
    grid = std::max(1, std::min(per, kStepPerSM)) * sms;
  }
  if (grid > kStepMaxCTAs) return BILU_ERR_UNSUPPORTED;
  GridSync gs;
  gs.count = words;
  gs.gen = words + 1;
  gs.err = reinterpret_cast<int*>(words + 2);
  gs.spin = kSpinLimit;
  void* args[] = {&n, &V, &ldv, &j, &w, &hout, &hstride, &wwout, &partial, &gs, &vnext, &vnext32};
  BILU_TRY_CUDA(cudaLaunchCooperativeKernel((const void*)k_mgs_step<T>, dim3(grid),
                                            dim3(kStepThreads), args, smem, st));
  BILU_LAUNCH_CHECK();
  return BILU_OK;
}

int mgs_step(long long n, const double* V, long long ldv, int j, double* w, double* hout,
             int hstride, double* wwout, double* partial, unsigned* words, double* vnext,
             float* vnext32, cudaStream_t st) {
  return mgs_step_t<double>(n, V, ldv, j, w, hout, hstride, wwout, partial, words, vnext,
                            vnext32, st);
}

int mgs_step_f32(long long n, const float* V, long long ldv, int j, float* w, double* hout,
                 int hstride, double* wwout, double* partial, unsigned* words, float* vnext,
                 cudaStream_t st) {
  return mgs_step_t<float>(n, V, ldv, j, w, hout, hstride, wwout, partial, words, vnext,
                           nullptr, st);
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

using namespace bilu;

// Test and measurement hook: one modified Gram-Schmidt step (mgs_step or
// its FP32 form) on caller vectors.
extern "C" size_t bilu_debug_mgs_step_ws_bytes(void) {
  return sizeof(double) * 2 * kStepMaxCTAs + 256 + sizeof(unsigned) * 4;
}

extern "C" int bilu_debug_mgs_step(long long n, int fp32, const void* d_V, long long ldv, int j,
                                   void* d_w, double* d_h, void* d_vnext, void* d_ws,
                                   size_t ws_bytes, bilu_stream_t stream) {
  if (n < 1 || j < 0 || j >= kMaxVec || ldv < n || !d_V || !d_w || !d_h || !d_ws ||
      ws_bytes < bilu_debug_mgs_step_ws_bytes())
    return BILU_ERR_ARG;
  // 16-byte vector accesses: every basis vector starts on a 16-byte boundary
  if ((ldv * (fp32 ? 4 : 8)) % 16 != 0 || ((uintptr_t)d_V | (uintptr_t)d_w) % 16 != 0 ||
      (d_vnext && (uintptr_t)d_vnext % 16 != 0))
    return BILU_ERR_ARG;
  cudaStream_t st = S(stream);
  double* partial = (double*)d_ws;
  unsigned* words = (unsigned*)((char*)d_ws + sizeof(double) * 2 * kStepMaxCTAs + 256);
  BILU_TRY_CUDA(cudaMemsetAsync(words, 0, sizeof(unsigned) * 4, st));
  int rc = fp32 ? mgs_step_f32(n, (const float*)d_V, ldv, j, (float*)d_w, d_h, 1, d_h + j + 1,
                               partial, words, (float*)d_vnext, st)
                : mgs_step(n, (const double*)d_V, ldv, j, (double*)d_w, d_h, 1, d_h + j + 1,
                           partial, words, (double*)d_vnext, nullptr, st);
  if (rc != BILU_OK) return rc;
  int err = 0;
  BILU_TRY_CUDA(cudaMemcpyAsync(&err, words + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  return err;
}
