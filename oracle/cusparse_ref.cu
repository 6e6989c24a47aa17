// cuSPARSE baseline harness -- TEST INFRASTRUCTURE ONLY.
//
// Runs the library calls the reference makes for BILU(0) and the block
// triangular solves with the reference's settings, so the GPU engine can be
// checked against cuSPARSE and timed beside it:
//   bsrilu02_inplace          bsrilu.h:20-66        (ROW direction, NO_LEVEL)
//   bsrsv2 L / U              BILU_cusparse.h:110-224 (L: unit lower, NO_LEVEL;
//                                                     U: non-unit upper, USE_LEVEL)
// Built on the GPU host by oracle/Makefile (`make cusparse`) into
// oracle/_ref/libcusparse_ref.so; never linked by the product library.
#include <cuda_runtime.h>
#include <cusparse.h>

#include <cstdio>

#define CK(x)                                    \
  do {                                           \
    cudaError_t e_ = (x);                        \
    if (e_ != cudaSuccess) return -100 - (int)e_; \
  } while (0)
#define CS(x)                                             \
  do {                                                    \
    cusparseStatus_t s_ = (x);                            \
    if (s_ != CUSPARSE_STATUS_SUCCESS) return -(int)s_;   \
  } while (0)

namespace {
float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}
}  // namespace

extern "C" {

// In-place BILU(0) of a device BSR matrix.  ms[0] analysis, ms[1] factor.
int cusp_bsrilu02(int nb, int nnzb, int bs, const int* d_row, const int* d_col, double* d_val,
                  int* zero_pivot, float* ms) {
  cusparseHandle_t h;
  CS(cusparseCreate(&h));
  cusparseMatDescr_t d;
  CS(cusparseCreateMatDescr(&d));
  CS(cusparseSetMatType(d, CUSPARSE_MATRIX_TYPE_GENERAL));
  CS(cusparseSetMatIndexBase(d, CUSPARSE_INDEX_BASE_ZERO));
  bsrilu02Info_t info;
  CS(cusparseCreateBsrilu02Info(&info));
  int bufsize = 0;
  CS(cusparseDbsrilu02_bufferSize(h, CUSPARSE_DIRECTION_ROW, nb, nnzb, d, d_val, d_row, d_col, bs,
                                  info, &bufsize));
  void* buf = nullptr;
  CK(cudaMalloc(&buf, bufsize));
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventRecord(e0);
  CS(cusparseDbsrilu02_analysis(h, CUSPARSE_DIRECTION_ROW, nb, nnzb, d, d_val, d_row, d_col, bs,
                                info, CUSPARSE_SOLVE_POLICY_NO_LEVEL, buf));
  cudaEventRecord(e1);
  CS(cusparseDbsrilu02(h, CUSPARSE_DIRECTION_ROW, nb, nnzb, d, d_val, d_row, d_col, bs, info,
                       CUSPARSE_SOLVE_POLICY_NO_LEVEL, buf));
  cudaEventRecord(e2);
  ms[0] = elapsed(e0, e1);
  ms[1] = elapsed(e1, e2);
  int zp = -1;
  cusparseStatus_t st = cusparseXbsrilu02_zeroPivot(h, info, &zp);
  *zero_pivot = st == CUSPARSE_STATUS_ZERO_PIVOT ? zp : -1;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaFree(buf);
  cusparseDestroyBsrilu02Info(info);
  cusparseDestroyMatDescr(d);
  cusparseDestroy(h);
  return 0;
}

// x = L^-1 b (lower != 0, unit) or U^-1 b on the packed factor, `reps`
// timed solves after one warm-up; ms[0] analysis, ms[1] mean solve.
int cusp_bsrsv2(int nb, int nnzb, int bs, const int* d_row, const int* d_col, const double* d_val,
                int lower, const double* d_b, double* d_x, int reps, float* ms) {
  cusparseHandle_t h;
  CS(cusparseCreate(&h));
  cusparseMatDescr_t d;
  CS(cusparseCreateMatDescr(&d));
  CS(cusparseSetMatIndexBase(d, CUSPARSE_INDEX_BASE_ZERO));
  CS(cusparseSetMatType(d, CUSPARSE_MATRIX_TYPE_GENERAL));
  CS(cusparseSetMatFillMode(d, lower ? CUSPARSE_FILL_MODE_LOWER : CUSPARSE_FILL_MODE_UPPER));
  CS(cusparseSetMatDiagType(d, lower ? CUSPARSE_DIAG_TYPE_UNIT : CUSPARSE_DIAG_TYPE_NON_UNIT));
  cusparseSolvePolicy_t pol = lower ? CUSPARSE_SOLVE_POLICY_NO_LEVEL : CUSPARSE_SOLVE_POLICY_USE_LEVEL;
  bsrsv2Info_t info;
  CS(cusparseCreateBsrsv2Info(&info));
  int bufsize = 0;
  CS(cusparseDbsrsv2_bufferSize(h, CUSPARSE_DIRECTION_ROW, CUSPARSE_OPERATION_NON_TRANSPOSE, nb,
                                nnzb, d, const_cast<double*>(d_val), d_row, d_col, bs, info,
                                &bufsize));
  void* buf = nullptr;
  CK(cudaMalloc(&buf, bufsize));
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  const double one = 1.0;
  cudaEventRecord(e0);
  CS(cusparseDbsrsv2_analysis(h, CUSPARSE_DIRECTION_ROW, CUSPARSE_OPERATION_NON_TRANSPOSE, nb,
                              nnzb, d, d_val, d_row, d_col, bs, info, pol, buf));
  cudaEventRecord(e1);
  CS(cusparseDbsrsv2_solve(h, CUSPARSE_DIRECTION_ROW, CUSPARSE_OPERATION_NON_TRANSPOSE, nb, nnzb,
                           &one, d, d_val, d_row, d_col, bs, info, d_b, d_x, pol, buf));
  cudaEventSynchronize(e1);
  cudaEvent_t s0, s1;
  cudaEventCreate(&s0);
  cudaEventCreate(&s1);
  cudaEventRecord(s0);
  for (int i = 0; i < reps; ++i)
    CS(cusparseDbsrsv2_solve(h, CUSPARSE_DIRECTION_ROW, CUSPARSE_OPERATION_NON_TRANSPOSE, nb, nnzb,
                             &one, d, d_val, d_row, d_col, bs, info, d_b, d_x, pol, buf));
  cudaEventRecord(s1);
  ms[0] = elapsed(e0, e1);
  ms[1] = reps > 0 ? elapsed(s0, s1) / reps : 0.f;
  (void)e2;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaEventDestroy(s0);
  cudaEventDestroy(s1);
  cudaFree(buf);
  cusparseDestroyBsrsv2Info(info);
  cusparseDestroyMatDescr(d);
  cusparseDestroy(h);
  return 0;
}

}  // extern "C"
