// Vector kernels for the Krylov solver: fused multi-dot, multi-axpy with
// norm, deterministic reductions (fixed CTA count, fixed summation order).
#pragma once
#include "common.cuh"

namespace bilu {

constexpr int kRedCTAs = 152 * 4;  // partial-sum slots (fixed => deterministic)
constexpr int kRedThreads = 256;
constexpr int kMaxVec = 32;        // vectors per multi-dot / multi-axpy call
constexpr int kPartStride = kMaxVec + 2;

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

// ---- FP32 inner solver of the nested (GMRES-IR) mode ----
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

// Whole modified Gram-Schmidt step of Arnoldi step j in one cooperative
// launch: j+2 fused sweeps (sweep i applies w -= h_{i-1} v_{i-1} and takes
// h_i = v_i . w; the last one w . w) with a counting grid barrier between
// them: h_i into hout[i * hstride]
// (i <= j), ||w||^2 into *wwout, then vnext = w / ||w|| (and vnext32, its
// FP32 copy, when given; zeros when ||w|| = 0).  Sums are in the vectors'
// precision and in a fixed order (warp 0 of every CTA adds all CTA
// partials alike).  partial holds 2 * kStepMaxCTAs doubles; words are the barrier's count, exit count and
// error word (zero before the first launch; every launch leaves them zero
// unless a barrier timed out, which sets the error word to
// BILU_ERR_TIMEOUT).
constexpr int kStepMaxCTAs = 152 * 8;
int mgs_step(long long n, const double* V, long long ldv, int j, double* w, double* hout,
             int hstride, double* wwout, double* partial, unsigned* words, double* vnext,
             float* vnext32, cudaStream_t st);
// The FP32 form for the nested mode's inner solver: FP32 products and FP32
// sums throughout (the CTA partials and their sum too; the FP64 pipe is
// left alone), h and ||w||^2 written as FP64.
int mgs_step_f32(long long n, const float* V, long long ldv, int j, float* w, double* hout,
                 int hstride, double* wwout, double* partial, unsigned* words, float* vnext,
                 cudaStream_t st);

}  // namespace bilu
