// Vector kernels for the Krylov solver: fused multi-dot, multi-axpy with
// norm, deterministic reductions (fixed CTA count, fixed summation order).
#pragma once
#include "common.cuh"

namespace bilu {

constexpr int kRedCTAs = 152 * 4;  // partial-sum slots (fixed => deterministic)
constexpr int kRedThreads = 256;
constexpr int kMaxVec = 32;        // vectors per multi-dot / multi-axpy call
constexpr int kPartStride = kMaxVec + 2;
constexpr int kSweepCTAs = 152 * 6;  // CTAs of one MGS sweep (one partial each, one wave)

// partial[cta * kPartStride + i] = sum_e V[i][e] * w[e] (i < nv), and at
// index nv: sum_e w[e]^2 when with_ww.  Skipped (partials left as they
// are) when skip_flag is non-null and *skip_flag == 0.
int multidot(long long n, const double* V, long long ldv, int nv, const double* w, bool with_ww,
             double* partial, cudaStream_t st, const int* skip_flag = nullptr);
// w -= sum_i coef[i] V[i]  (or w += when sign > 0); partial[cta*kPartStride]
// = sum_e w_new[e]^2.  If skip_flag is non-null and *skip_flag == 0 the
// kernel returns without touching w.
int multiaxpy_norm(long long n, const double* V, long long ldv, int nv, const double* coef,
                   double sign, double* w, double* partial, const int* skip_flag,
                   cudaStream_t st);
// out[i] = sum_cta partial[cta*kPartStride + i], i < nout (one thread each).
int reduce_partials(const double* partial, int nout, double* out, cudaStream_t st);
// y = x * (1/sqrt(*nrm2)) with *nrm2 a device scalar; y32 (optional)
// receives the same vector rounded to FP32 (input of the FP32 apply).
int scale_rsqrt(long long n, const double* x, const double* nrm2, double* y, cudaStream_t st,
                float* y32 = nullptr);
// r = b - ax, partial norms of r
int residual_norm(long long n, const double* b, const double* ax, double* r, double* partial,
                  cudaStream_t st);

// One modified Gram-Schmidt sweep over w: if vp != null, w -= (*hp) * vp;
// then *out = vn . w (or w . w when vn == null), the CTA partials summed in a
// fixed order by the last CTA to finish (counter returns to 0 afterwards).
int mgs_sweep(long long n, const double* vp, const double* hp, const double* vn, double* w,
              double* partial, unsigned* counter, double* out, cudaStream_t st);

// ---- FP32 inner solver of the nested (GMRES-IR) mode ----
// The same fused sweep on FP32 vectors (vp, vn, w float; h read as double
// and rounded to FP32): FP32 products and per-thread FP32 sums, the warp
// sums widened to FP64 and the CTA partials added in a fixed order, so the
// dot products are reproducible run to run.  vn is read with an L2-keeping
// load (it is the next sweep's vp), vp with an evict-first load.
int mgs_sweep_f32(long long n, const float* vp, const double* hp, const float* vn, float* w,
                  double* partial, unsigned* counter, double* out, cudaStream_t st);
// y = x * (1/sqrt(*nrm2)) in FP32 (zeros when *nrm2 == 0).
int scale_rsqrt_f32(long long n, const float* x, const double* nrm2, float* y, cudaStream_t st);
// Least squares of the inner Arnoldi steps on the device (one thread): H
// holds (k+1) x k entries H[i*k + j] with the raw column entries h_ij
// (i <= j) and, in ww[j], ||w_j||^2 (the subdiagonal squared); Givens
// rotations in FP64 reduce H to triangular form against beta e_1 (beta = 1)
// and y[0..k) receives the solution (zeros beyond the first zero
// subdiagonal, where the steps found an invariant subspace).
int inner_lsq(int k, const double* H, const double* ww, double* y, cudaStream_t st);
// z = sum_{i<k} y_i Q_i: FP32 products and sums (i ascending), widened to
// FP64 (z is the outer flexible-GMRES direction).
int combine_f32(long long n, const float* Q, long long ldq, int k, const double* y, double* z,
                cudaStream_t st);

}  // namespace bilu
