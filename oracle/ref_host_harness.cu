// Reference host-code harness: TEST INFRASTRUCTURE ONLY.
//
// Compiled (by oracle/Makefile, target `ref`) against the reference headers
// where they lie, once per block size, into oracle/_ref/libref_bs<N>.so.  It
// exposes the reference's own host functions through extern "C" wrappers with
// plain pointers so tests/golden/make_golden.py can run them on seeded inputs
// and record golden vectors that pin the CPU oracle.  Only host code of the
// reference runs here; no CUDA call is made.
#include "common.h"
#include "csr2bsr.h"
#include "read_matrix.h"
#include "isai_bsr.h"
#include "bcsc2bcsr.h"
#include "bcsc2bcsrAndSpMV.h"
#include "spmv_debug.h"

#include <cstring>
#include <string>
#include <vector>

namespace {
template <class T>
void put(const std::vector<T>& v, T* dst) {
  if (!v.empty()) std::memcpy(dst, v.data(), sizeof(T) * v.size());
}
}  // namespace

extern "C" {

int ref_block_size(void) { return BS; }

// csr2bsr.h:14 csr_to_bsr5.  Returns nnzb; outputs are written when the
// capacity (in blocks) is large enough.
int ref_csr_to_bsr(int n, const int* row, const int* col, const double* val,
                   int nnz, int* bsrRow, int* bsrCol, double* bsrVal,
                   int cap_blocks) {
  std::vector<int> r(row, row + n + 1), c(col, col + nnz);
  std::vector<double> v(val, val + nnz);
  int nb = 0;
  std::vector<int> br, bc;
  std::vector<double> bv;
  csr_to_bsr5(n, r, c, v, nb, br, bc, bv);
  int nnzb = (int)bc.size();
  if (nnzb <= cap_blocks) {
    put(br, bsrRow);
    put(bc, bsrCol);
    put(bv, bsrVal);
  }
  return nnzb;
}

// isai_bsr.h:246 build_bcsc_pattern_from_bsr_scalarILU
int ref_isai_pattern(int nb, const int* Arow, const int* Acol, int lower,
                     int* Mptr, int* Mind, int cap) {
  std::vector<int> mp, mi;
  build_bcsc_pattern_from_bsr_scalarILU(nb, Arow, Acol, lower != 0, mp, mi);
  int nnz = (int)mi.size();
  if (nnz <= cap) {
    put(mp, Mptr);
    put(mi, Mind);
  }
  return nnz;
}

// bcsc2bcsr.h:11 build_triangular_bcsr_pattern_from_A
int ref_tri_pattern(int nb, const int* Arow, const int* Acol, int lower,
                    int* Trow, int* Tcol, int cap) {
  std::vector<int> tr, tc;
  build_triangular_bcsr_pattern_from_A(nb, Arow, Acol, lower != 0, tr, tc);
  int nnz = (int)tc.size();
  if (nnz <= cap) {
    put(tr, Trow);
    put(tc, Tcol);
  }
  return nnz;
}

// bcsc2bcsr.h:32 build_map_bcsc2bcsr_host (exits the process on mismatch,
// so callers only pass consistent patterns)
int ref_map_bcsc2bcsr(int nb, const int* cscPtr, const int* cscInd,
                      const int* csrRow, const int* csrCol, int* map) {
  std::vector<int> cp(cscPtr, cscPtr + nb + 1);
  std::vector<int> ci(cscInd, cscInd + cscPtr[nb]);
  std::vector<int> rp(csrRow, csrRow + nb + 1);
  std::vector<int> rc(csrCol, csrCol + csrRow[nb]);
  std::vector<int> m;
  build_map_bcsc2bcsr_host(nb, cp, ci, rp, rc, m);
  put(m, map);
  return (int)m.size();
}

// bcsc2bcsrAndSpMV.h:119 cpu_bcsr_spmv
int ref_cpu_bcsr_spmv(int mb, const int* row, const int* col, const double* val,
                      const double* x, double* y) {
  cpu_bcsr_spmv(mb, BS, BS, row, col, val, x, y);
  return 0;
}

// spmv_debug.h:44 spmvdbg::bcsc_matvec_bsr5_cpu
int ref_bcsc_matvec(int nb, const int* Mptr, const int* Mind, const double* Mval,
                    const double* x, double* y) {
  std::vector<int> mp(Mptr, Mptr + nb + 1), mi(Mind, Mind + Mptr[nb]);
  std::vector<double> mv(Mval, Mval + (size_t)Mptr[nb] * BS2), xv(x, x + (size_t)nb * BS), yv;
  spmvdbg::bcsc_matvec_bsr5_cpu(nb, mp, mi, mv, xv, yv);
  put(yv, y);
  return 0;
}

// read_matrix.h:12 read_matrix_market_to_csr.  Returns nnz (or -1).
int ref_read_mtx(const char* path, int* nrows, int* ncols, int* row, int* col,
                 double* val, int cap) {
  int m = 0, n = 0;
  std::vector<int> rp, ci;
  std::vector<double> v;
  if (!read_matrix_market_to_csr(std::string(path), m, n, rp, ci, v)) return -1;
  *nrows = m;
  *ncols = n;
  int nnz = (int)ci.size();
  if (nnz <= cap) {
    put(rp, row);
    put(ci, col);
    put(v, val);
  }
  return nnz;
}

}  // extern "C"
