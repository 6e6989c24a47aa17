/*
 * C++ drop-in layer: the reference's own host entry points (names, argument
 * lists, pointer kinds and exit-on-error behaviour of gmfff/isai_kernel),
 * implemented over the C ABI of libbilu_isai.so (include/bilu_isai.h).  A
 * copy of the reference's main.cu pipeline that includes this header in
 * place of csr2bsr.h, isai_bsr.h, bcsc2bcsr.h, bsrilu.h, bsr2csr.h,
 * cape_sptrsv.h, bsr_tensor_SpMV.h, bcsc2bcsrAndSpMV.h, residual_check.h
 * and read_matrix.h builds against the library unchanged at these calls;
 * the reference's __global__ kernels that main.cu launches with <<<...>>>
 * become the host calls bilu_build_dinv, bilu_pairs_ptr / bilu_pairs_fill,
 * bilu_isai_compute, bilu_reorder_bcsc_to_bcsr and bilu_bcsr_spmv.
 *
 * Values are double (the reference's USE_DOUBLE build).  The block size of
 * csr_to_bsr5 and csr_cape_SpTRSV is the compile-time constant BS of the
 * reference's config.h, or BILU_COMPAT_BS when the includer defines it.
 * Host pointers and vectors stay host memory, device pointers stay device
 * memory, exactly as in the reference.  Errors print one line to stderr and
 * call std::exit(1), as the reference's CHECK macros do.
 */
#ifndef BILU_ISAI_COMPAT_HPP
#define BILU_ISAI_COMPAT_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

#include "bilu_isai.h"

#ifndef BILU_COMPAT_BS
#define BILU_COMPAT_BS BS
#endif

namespace bilu_compat {

[[noreturn]] inline void fail(const char* where, const char* what) {
  std::fprintf(stderr, "%s: %s\n", where, what);
  std::exit(1);
}

inline void check(int st, const char* where) {
  if (st != BILU_OK) {
    if (st == BILU_ERR_CUDA)
      std::fprintf(stderr, "%s: %s (cudaError_t %d)\n", where, bilu_status_string(st),
                   bilu_last_cuda_error());
    else
      std::fprintf(stderr, "%s: %s\n", where, bilu_status_string(st));
    std::exit(1);
  }
}

inline void cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) fail(where, cudaGetErrorString(e));
}

// Device buffer owned by a compat call (the reference allocates inside
// these functions as well).
template <class T>
struct Dev {
  T* p = nullptr;
  explicit Dev(size_t count, const char* where = "cudaMalloc") {
    cuda(cudaMalloc((void**)&p, sizeof(T) * (count ? count : 1)), where);
  }
  Dev(const T* host, size_t count, const char* where = "cudaMemcpy H2D") : Dev(count, where) {
    if (count) cuda(cudaMemcpy(p, host, sizeof(T) * count, cudaMemcpyHostToDevice), where);
  }
  ~Dev() { cudaFree(p); }
  Dev(const Dev&) = delete;
  Dev& operator=(const Dev&) = delete;
  void to_host(T* host, size_t count) const {
    if (count) cuda(cudaMemcpy(host, p, sizeof(T) * count, cudaMemcpyDeviceToHost), "D2H");
  }
};

inline void sync(const char* where) { cuda(cudaDeviceSynchronize(), where); }

}  // namespace bilu_compat

/* read_matrix.h:12 read_matrix_market_to_csr: general, symmetric and
 * skew-symmetric real / integer / pattern files, 0-based CSR on the host.
 * Prints the reader's error and returns false where the reference does. */
inline bool read_matrix_market_to_csr(const std::string& filename, int& nrows, int& ncols,
                                      std::vector<int>& rowPtr, std::vector<int>& colInd,
                                      std::vector<double>& vals) {
  long long nnz = 0, bad = -1;
  int st = bilu_mtx_read(filename.c_str(), &nrows, &ncols, &nnz, nullptr, nullptr, nullptr, &bad);
  if (st != BILU_OK) {
    std::cerr << "Cannot read " << filename << ": " << bilu_status_string(st) << "\n";
    return false;
  }
  rowPtr.assign((size_t)nrows + 1, 0);
  colInd.assign((size_t)nnz, 0);
  vals.assign((size_t)nnz, 0.0);
  st = bilu_mtx_read(filename.c_str(), &nrows, &ncols, &nnz, rowPtr.data(), colInd.data(),
                     vals.data(), &bad);
  if (st != BILU_OK) {
    std::cerr << "Cannot read " << filename << ": " << bilu_status_string(st) << "\n";
    return false;
  }
  return true;
}

/* csr2bsr.h:14 csr_to_bsr5: host CSR (n x n, n % BS == 0) to host BSR with
 * ascending block columns and summed duplicates; runs on the GPU. */
inline void csr_to_bsr5(int n, const std::vector<int>& csrRowPtr,
                        const std::vector<int>& csrColInd, const std::vector<double>& csrVal,
                        int& nb, std::vector<int>& bsrRowPtr, std::vector<int>& bsrColInd,
                        std::vector<double>& bsrVal) {
  using namespace bilu_compat;
  const int bs = BILU_COMPAT_BS;
  if (n % bs != 0) fail("csr_to_bsr5", "n is not a multiple of the block size");
  nb = n / bs;
  const size_t nnz = csrColInd.size();
  Dev<int> row(csrRowPtr.data(), (size_t)n + 1), col(csrColInd.data(), nnz);
  Dev<double> val(csrVal.data(), nnz);
  Dev<int> brow((size_t)nb + 1);
  Dev<char> ws(bilu_csr_to_bsr_ws_bytes(n, bs));
  int nnzb = 0;
  check(bilu_csr_to_bsr_rowptr(n, bs, row.p, col.p, brow.p, &nnzb, ws.p,
                               bilu_csr_to_bsr_ws_bytes(n, bs), nullptr),
        "csr_to_bsr5");
  Dev<int> bcol((size_t)nnzb);
  Dev<double> bval((size_t)nnzb * bs * bs);
  check(bilu_csr_to_bsr_fill(n, bs, row.p, col.p, val.p, brow.p, bcol.p, bval.p, nullptr),
        "csr_to_bsr5");
  bsrRowPtr.resize((size_t)nb + 1);
  bsrColInd.resize((size_t)nnzb);
  bsrVal.resize((size_t)nnzb * bs * bs);
  brow.to_host(bsrRowPtr.data(), (size_t)nb + 1);
  bcol.to_host(bsrColInd.data(), (size_t)nnzb);
  bval.to_host(bsrVal.data(), (size_t)nnzb * bs * bs);
}

/* isai_bsr.h:246 build_bcsc_pattern_from_bsr_scalarILU: BCSC pattern of
 * M_L (for_lower) or M_U from a host BSR pattern. */
inline void build_bcsc_pattern_from_bsr_scalarILU(int nb, const int* Abrow, const int* Abcol,
                                                  bool for_lower, std::vector<int>& Mbrow,
                                                  std::vector<int>& Mcol) {
  using namespace bilu_compat;
  const int nnzb = Abrow[nb];
  Dev<int> row(Abrow, (size_t)nb + 1), col(Abcol, (size_t)nnzb), ptr((size_t)nb + 1);
  const size_t wsb = bilu_isai_pattern_ws_bytes(nb, nnzb);
  Dev<char> ws(wsb);
  int mnnz = 0;
  check(bilu_isai_pattern_colptr(nb, row.p, col.p, for_lower, ptr.p, &mnnz, ws.p, wsb, nullptr),
        "build_bcsc_pattern_from_bsr_scalarILU");
  Dev<int> ind((size_t)mnnz);
  check(bilu_isai_pattern_fill(nb, row.p, col.p, for_lower, ptr.p, ind.p, ws.p, wsb, nullptr),
        "build_bcsc_pattern_from_bsr_scalarILU");
  Mbrow.resize((size_t)nb + 1);
  Mcol.resize((size_t)mnnz);
  ptr.to_host(Mbrow.data(), (size_t)nb + 1);
  ind.to_host(Mcol.data(), (size_t)mnnz);
}

/* bcsc2bcsr.h:11 build_triangular_bcsr_pattern_from_A: BCSR pattern of the
 * lower (c <= r) or upper (c >= r) part of a host BSR pattern. */
inline void build_triangular_bcsr_pattern_from_A(int nb, const int* A_bsrRow,
                                                 const int* A_bsrCol, bool lower,
                                                 std::vector<int>& T_bsrRow,
                                                 std::vector<int>& T_bsrCol) {
  using namespace bilu_compat;
  const int nnzb = A_bsrRow[nb];
  Dev<int> row(A_bsrRow, (size_t)nb + 1), col(A_bsrCol, (size_t)nnzb), trow((size_t)nb + 1);
  const size_t wsb = bilu_tri_pattern_ws_bytes(nb);
  Dev<char> ws(wsb);
  int tnnz = 0;
  check(bilu_tri_pattern_rowptr(nb, row.p, col.p, lower, trow.p, &tnnz, ws.p, wsb, nullptr),
        "build_triangular_bcsr_pattern_from_A");
  Dev<int> tcol((size_t)tnnz);
  check(bilu_tri_pattern_fill(nb, row.p, col.p, lower, trow.p, tcol.p, nullptr),
        "build_triangular_bcsr_pattern_from_A");
  T_bsrRow.resize((size_t)nb + 1);
  T_bsrCol.resize((size_t)tnnz);
  trow.to_host(T_bsrRow.data(), (size_t)nb + 1);
  tcol.to_host(T_bsrCol.data(), (size_t)tnnz);
}

/* bcsc2bcsr.h:32 build_map_bcsc2bcsr_host: position in the BCSR pattern of
 * every BCSC entry.  A BCSC entry missing from the BCSR pattern prints its
 * (row, col) and exits, as the reference does (bcsc2bcsr.h:53-56). */
inline void build_map_bcsc2bcsr_host(int nb, const std::vector<int>& bcscColPtr,
                                     const std::vector<int>& bcscRowInd,
                                     const std::vector<int>& bcsrRowPtr,
                                     const std::vector<int>& bcsrColInd,
                                     std::vector<int>& map_bcsc2bcsr) {
  using namespace bilu_compat;
  const size_t nnzb = bcscRowInd.size();
  Dev<int> cp(bcscColPtr.data(), (size_t)nb + 1), ci(bcscRowInd.data(), nnzb);
  Dev<int> rp(bcsrRowPtr.data(), (size_t)nb + 1), rc(bcsrColInd.data(), bcsrColInd.size());
  Dev<int> map(nnzb);
  Dev<char> ws(bilu_map_ws_bytes());
  int bad[2] = {-1, -1};
  const int st = bilu_map_bcsc2bcsr(nb, cp.p, ci.p, rp.p, rc.p, map.p, bad, ws.p,
                                    bilu_map_ws_bytes(), nullptr);
  if (st == BILU_ERR_PATTERN) {
    std::cerr << "map_bcsc2bcsr: entry (" << bad[0] << "," << bad[1] << ") not found in BCSR\n";
    std::exit(1);
  }
  check(st, "build_map_bcsc2bcsr_host");
  map_bcsc2bcsr.resize(nnzb);
  map.to_host(map_bcsc2bcsr.data(), nnzb);
}

/* bsrilu.h:20 bsrilu02_inplace: BILU(0) of a device BSR matrix in place
 * (the packed L\U layout of cuSPARSE bsrilu02, row direction).  A zero
 * pivot prints the block row and exits. */
inline void bsrilu02_inplace(int nb, int nnzb, int BS_, const int* d_bsrRow, const int* d_bsrCol,
                             double* d_bsrVal) {
  using namespace bilu_compat;
  const size_t wsb = bilu_bsrilu0_ws_bytes(nb, nnzb);
  Dev<char> ws(wsb);
  int zp = -1;
  const int st = bilu_bsrilu0(nb, nnzb, BS_, d_bsrRow, d_bsrCol, d_bsrVal, &zp, ws.p, wsb, nullptr);
  if (st == BILU_ERR_ZERO_PIVOT) {
    std::cerr << "bsrilu02: zero pivot at block row " << zp << "\n";
    std::exit(1);
  }
  check(st, "bsrilu02_inplace");
}

/* bcsc2bcsrAndSpMV.h:76 bcsc_to_bcsr: device BCSC (MB x NB blocks of R x C)
 * to device BCSR; columns come out ascending inside each row. */
inline void bcsc_to_bcsr(int MB, int NB, int R, int C, const int* d_MbrowU, const int* d_McolU,
                         const double* d_MvalU, int* d_row_ptr, int* d_col_ind, double* d_val) {
  using namespace bilu_compat;
  if (R != C) fail("bcsc_to_bcsr", "blocks must be square");
  int nnzb = 0;
  cuda(cudaMemcpy(&nnzb, d_MbrowU + NB, sizeof(int), cudaMemcpyDeviceToHost), "bcsc_to_bcsr");
  const size_t wsb = bilu_bcsc_to_bcsr_ws_bytes(MB, nnzb);
  Dev<char> ws(wsb);
  check(bilu_bcsc_to_bcsr(MB, NB, R, d_MbrowU, d_McolU, d_MvalU, d_row_ptr, d_col_ind, d_val,
                          ws.p, wsb, nullptr),
        "bcsc_to_bcsr");
  sync("bcsc_to_bcsr");
}

/* bsr2csr.h:19 bsr2csr_cusparse: host BSR to CSR in host arrays that the
 * function allocates with malloc (the caller frees them, as with the
 * reference); *nnzbsr2csr = nnzb * blockDim^2.  Returns 0. */
inline int bsr2csr_cusparse(const int* bsrRowPtr_A, const int* bsrColInd_A,
                            const double* bsrVal_A, const int mb, const int nnzb,
                            const int blockDim, int** bsr2csrRowPtrA_tmp,
                            int** bsr2csrColIndA_tmp, double** bsr2csrVal_tmp, int* nnzbsr2csr) {
  using namespace bilu_compat;
  const size_t bs2 = (size_t)blockDim * blockDim, m = (size_t)mb * blockDim;
  const size_t nnz = (size_t)nnzb * bs2;
  Dev<int> row(bsrRowPtr_A, (size_t)mb + 1), col(bsrColInd_A, (size_t)nnzb);
  Dev<double> val(bsrVal_A, nnz);
  Dev<int> crow(m + 1), ccol(nnz);
  Dev<double> cval(nnz);
  check(bilu_bsr_to_csr(mb, blockDim, row.p, col.p, val.p, crow.p, ccol.p, cval.p, nullptr),
        "bsr2csr_cusparse");
  *bsr2csrRowPtrA_tmp = (int*)std::malloc(sizeof(int) * (m + 1));
  *bsr2csrColIndA_tmp = (int*)std::malloc(sizeof(int) * (nnz ? nnz : 1));
  *bsr2csrVal_tmp = (double*)std::malloc(sizeof(double) * (nnz ? nnz : 1));
  if (!*bsr2csrRowPtrA_tmp || !*bsr2csrColIndA_tmp || !*bsr2csrVal_tmp)
    fail("bsr2csr_cusparse", "out of host memory");
  crow.to_host(*bsr2csrRowPtrA_tmp, m + 1);
  ccol.to_host(*bsr2csrColIndA_tmp, nnz);
  cval.to_host(*bsr2csrVal_tmp, nnz);
  *nnzbsr2csr = (int)nnz;
  return 0;
}

/* cape_sptrsv.h:105 csr_cape_SpTRSV: solves L U x = b with the packed
 * scalar ILU factor in host CSR (unit lower L = the strictly lower entries,
 * U = the upper entries with the diagonal), x written into b as the
 * reference's comment on b states.  (The reference's own body clears its
 * device copy of b before the solves and never copies a result back,
 * cape_sptrsv.h:152-153; a caller of this layer gets the solution.)  The
 * CSR matrix is viewed as BSR with blocks of BS: explicit zeros inside a
 * block change nothing in either substitution, so the block solves give
 * the scalar result; m must be a multiple of BS and every diagonal entry
 * stored. */
inline void csr_cape_SpTRSV(int m, int* csrRowPtrA, int* csrColIdxA, double* csrValA, int nnz,
                            double* b) {
  using namespace bilu_compat;
  const int bs = BILU_COMPAT_BS;
  if (m % bs != 0) fail("csr_cape_SpTRSV", "m is not a multiple of the block size");
  const int nb = m / bs;
  Dev<int> row(csrRowPtrA, (size_t)m + 1), col(csrColIdxA, (size_t)nnz);
  Dev<double> val(csrValA, (size_t)nnz);
  Dev<int> brow((size_t)nb + 1);
  const size_t cwb = bilu_csr_to_bsr_ws_bytes(m, bs);
  Dev<char> cws(cwb);
  int nnzb = 0;
  check(bilu_csr_to_bsr_rowptr(m, bs, row.p, col.p, brow.p, &nnzb, cws.p, cwb, nullptr),
        "csr_cape_SpTRSV");
  Dev<int> bcol((size_t)nnzb);
  Dev<double> bval((size_t)nnzb * bs * bs);
  check(bilu_csr_to_bsr_fill(m, bs, row.p, col.p, val.p, brow.p, bcol.p, bval.p, nullptr),
        "csr_cape_SpTRSV");
  Dev<double> x(b, (size_t)m), z((size_t)m), y((size_t)m);
  const size_t wsb = bilu_sptrsv_ws_bytes(nb, nnzb);
  Dev<char> ws(wsb);
  check(bilu_sptrsv(nb, nnzb, bs, brow.p, bcol.p, bval.p, 1, x.p, z.p, ws.p, wsb, nullptr),
        "csr_cape_SpTRSV");
  check(bilu_sptrsv(nb, nnzb, bs, brow.p, bcol.p, bval.p, 0, z.p, y.p, ws.p, wsb, nullptr),
        "csr_cape_SpTRSV");
  y.to_host(b, (size_t)m);
}

/* bsr_tensor_SpMV.h:402 bsr_SpMV_tensorcore: res_Y = A Val_B with A a host
 * BSR matrix of mb x mb blocks of bdim x bdim (block products on the FP64
 * pipe: on GB300 DFMA is faster than DMMA for these blocks).  Val_C is
 * unused, as in the reference, which only writes its device copy. */
inline void bsr_SpMV_tensorcore(const int* bsrRowPtr_A, const int* bsrColIdx_A,
                                const double* bsrVal_A, const int mb, const int nnzb,
                                const int bdim, const double* Val_B, double* Val_C,
                                double* res_Y) {
  using namespace bilu_compat;
  (void)Val_C;
  const size_t n = (size_t)mb * bdim;
  Dev<int> row(bsrRowPtr_A, (size_t)mb + 1), col(bsrColIdx_A, (size_t)nnzb);
  Dev<double> val(bsrVal_A, (size_t)nnzb * bdim * bdim), x(Val_B, n), y(n);
  check(bilu_bcsr_spmv(mb, bdim, row.p, col.p, val.p, x.p, y.p, nullptr), "bsr_SpMV_tensorcore");
  y.to_host(res_Y, n);
}

/* residual_check.h:17 compute_rel_errors_csr: prints
 * ||x - x_true|| / ||x_true|| (when x_true is given) and ||b - A x|| / ||b||
 * for a host CSR matrix, host b / x_true and a device x, in the reference's
 * output format.  The norms are computed on the GPU (bilu_rel_errors on the
 * BSR view with blocks of BS). */
template <typename T>
inline void compute_rel_errors_csr(int n, const int* csrRowPtrA, const int* csrColIdxA,
                                   const T* csrValA, const T* b_host, const T* x_true,
                                   const T* d_x, const char* tag = "ISAI") {
  static_assert(sizeof(T) == sizeof(double), "the library's residual check is FP64");
  using namespace bilu_compat;
  const int bs = BILU_COMPAT_BS;
  if (n % bs != 0) fail("compute_rel_errors_csr", "n is not a multiple of the block size");
  const int nb = n / bs;
  const size_t nnz = (size_t)csrRowPtrA[n];
  Dev<int> row(csrRowPtrA, (size_t)n + 1), col(csrColIdxA, nnz);
  Dev<double> val((const double*)csrValA, nnz), b((const double*)b_host, (size_t)n);
  Dev<int> brow((size_t)nb + 1);
  const size_t cwb = bilu_csr_to_bsr_ws_bytes(n, bs);
  Dev<char> cws(cwb);
  int nnzb = 0;
  check(bilu_csr_to_bsr_rowptr(n, bs, row.p, col.p, brow.p, &nnzb, cws.p, cwb, nullptr),
        "compute_rel_errors_csr");
  Dev<int> bcol((size_t)nnzb);
  Dev<double> bval((size_t)nnzb * bs * bs);
  check(bilu_csr_to_bsr_fill(n, bs, row.p, col.p, val.p, brow.p, bcol.p, bval.p, nullptr),
        "compute_rel_errors_csr");
  Dev<double> xt((size_t)(x_true ? n : 1));
  if (x_true)
    cuda(cudaMemcpy(xt.p, x_true, sizeof(double) * n, cudaMemcpyHostToDevice),
         "compute_rel_errors_csr");
  const size_t wsb = bilu_rel_errors_ws_bytes(nb, bs);
  Dev<char> ws(wsb);
  double out[2] = {0.0, 0.0};
  check(bilu_rel_errors(nb, bs, brow.p, bcol.p, bval.p, b.p, x_true ? xt.p : nullptr,
                        (const double*)d_x, out, ws.p, wsb, nullptr),
        "compute_rel_errors_csr");
  if (x_true) std::cout << "[" << tag << "] rel_error_x = " << out[0] << "\n";
  double nbn = 0.0;
  for (int i = 0; i < n; ++i) nbn += (double)b_host[i] * (double)b_host[i];
  nbn = std::sqrt(nbn);
  std::cout << "[" << tag << "] rel_residual = " << out[1] << "  (||r||2=" << out[1] * nbn
            << ", ||b||2=" << nbn << ")\n";
}

#endif /* BILU_ISAI_COMPAT_HPP */
