// The reference's main.cu pipeline (main.cu:449-866), call for call, on
// libbilu_isai.so through the C++ drop-in layer (include/bilu_isai_compat.hpp)
// and, where main.cu launches the reference's kernels with <<<...>>>, the C
// ABI calls that replace them.  A compiled, non-Python caller of the
// library for the parity tests (tests/test_gpu_compat.py builds and runs it).
//
//   compat_pipeline matrix.mtx outdir
//
// Writes to outdir (raw little-endian arrays): lu.f64 (BILU(0) values),
// MrowL/McolL/MvalL and MrowU/McolU/MvalU (BCSR ISAI factors, int32 /
// f64), mbcscL/mindL (BCSC pattern of M_L), x.f64 (M_U M_L b with
// b = A * 0.7), spmv.f64 (bsr_SpMV_tensorcore of A on x_true), csr_row /
// csr_col / csr_val (bsr2csr_cusparse of the factor), cape.f64
// (csr_cape_SpTRSV of that CSR factor on b), bcsr_from_bcsc.f64 (bcsc_to_bcsr
// of M_L's BCSC values); stdout carries the residual check lines of
// compute_rel_errors_csr.
#include <cstdio>
#include <string>
#include <vector>

#ifndef COMPAT_BS
#define COMPAT_BS 4
#endif
constexpr int BS = COMPAT_BS;  // the reference's config.h constant for this build
#include "bilu_isai_compat.hpp"

namespace {

template <class T>
void dump(const std::string& dir, const char* name, const T* p, size_t n) {
  std::string path = dir + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) bilu_compat::fail("dump", path.c_str());
  if (n && std::fwrite(p, sizeof(T), n, f) != n) bilu_compat::fail("dump", path.c_str());
  std::fclose(f);
}

template <class T>
void dump_dev(const std::string& dir, const char* name, const T* d, size_t n) {
  std::vector<T> h(n);
  if (n) bilu_compat::cuda(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost), name);
  dump(dir, name, h.data(), n);
}

}  // namespace

int main(int argc, char** argv) {
  using bilu_compat::check;
  using bilu_compat::cuda;
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s matrix.mtx outdir\n", argv[0]);
    return 2;
  }
  const std::string filename = argv[1], out = argv[2];
  constexpr int BS2 = BS * BS;

  // 1. read mtx -> CSR (main.cu:479-497)
  int nrows = 0, ncols = 0;
  std::vector<int> csrRow, csrCol;
  std::vector<double> csrVal;
  if (!read_matrix_market_to_csr(filename, nrows, ncols, csrRow, csrCol, csrVal)) return 1;
  if (nrows != ncols) return 1;

  // 2. CSR -> BSR (main.cu:502-507)
  int nb = 0;
  std::vector<int> bsrRow, bsrCol;
  std::vector<double> bsrVal;
  csr_to_bsr5(nrows, csrRow, csrCol, csrVal, nb, bsrRow, bsrCol, bsrVal);
  const int nnzb = (int)bsrCol.size();

  // 3. ISAI BCSC patterns (main.cu:515-523)
  std::vector<int> MbrowL, McolL, MbrowU, McolU;
  build_bcsc_pattern_from_bsr_scalarILU(nb, bsrRow.data(), bsrCol.data(), true, MbrowL, McolL);
  build_bcsc_pattern_from_bsr_scalarILU(nb, bsrRow.data(), bsrCol.data(), false, MbrowU, McolU);
  const int nnzbL = MbrowL.back(), nnzbU = MbrowU.back();

  // 4. triangular BCSR patterns, the nnzb guard and the maps (main.cu:531-556)
  std::vector<int> MbcsrRowL, MbcsrColL, mapL, MbcsrRowU, MbcsrColU, mapU;
  build_triangular_bcsr_pattern_from_A(nb, bsrRow.data(), bsrCol.data(), true, MbcsrRowL,
                                       MbcsrColL);
  build_triangular_bcsr_pattern_from_A(nb, bsrRow.data(), bsrCol.data(), false, MbcsrRowU,
                                       MbcsrColU);
  if ((int)MbcsrColL.size() != nnzbL || (int)MbcsrColU.size() != nnzbU) {
    std::fprintf(stderr, "L/U pattern mismatch\n");
    return 1;
  }
  build_map_bcsc2bcsr_host(nb, MbrowL, McolL, MbcsrRowL, MbcsrColL, mapL);
  build_map_bcsc2bcsr_host(nb, MbrowU, McolU, MbcsrRowU, MbcsrColU, mapU);

  // 5. A to the GPU, BILU(0) in place (main.cu:560-590)
  bilu_compat::Dev<int> d_Abrow(bsrRow.data(), bsrRow.size()), d_Abcol(bsrCol.data(), bsrCol.size());
  bilu_compat::Dev<double> d_Abval(bsrVal.data(), bsrVal.size());
  bsrilu02_inplace(nb, nnzb, BS, d_Abrow.p, d_Abcol.p, d_Abval.p);
  dump_dev(out, "lu.f64", d_Abval.p, bsrVal.size());

  // 6. ISAI patterns, maps and BCSR patterns on the GPU (main.cu:600-660)
  bilu_compat::Dev<int> d_MbrowL(MbrowL.data(), MbrowL.size()), d_McolL(McolL.data(), McolL.size());
  bilu_compat::Dev<int> d_MbrowU(MbrowU.data(), MbrowU.size()), d_McolU(McolU.data(), McolU.size());
  bilu_compat::Dev<int> d_mapL(mapL.data(), mapL.size()), d_mapU(mapU.data(), mapU.size());
  bilu_compat::Dev<int> d_RowL(MbcsrRowL.data(), MbcsrRowL.size()),
      d_ColL(MbcsrColL.data(), MbcsrColL.size());
  bilu_compat::Dev<int> d_RowU(MbcsrRowU.data(), MbcsrRowU.size()),
      d_ColU(MbcsrColU.data(), MbcsrColU.size());
  bilu_compat::Dev<double> d_MvalL((size_t)nnzbL * BS2), d_MvalU((size_t)nnzbU * BS2);
  bilu_compat::Dev<double> d_ValL((size_t)nnzbL * BS2), d_ValU((size_t)nnzbU * BS2);

  // 7. Dinv, pair lists, ISAI-L / ISAI-U (main.cu:664-777): the kernel
  //    launches become the C ABI calls that replace them
  for (int lower = 1; lower >= 0; --lower) {
    const int* d_Mptr = lower ? d_MbrowL.p : d_MbrowU.p;
    const int* d_Mind = lower ? d_McolL.p : d_McolU.p;
    const int mnnz = lower ? nnzbL : nnzbU;
    bilu_compat::Dev<double> d_Dinv((size_t)nb * BS2);
    check(bilu_build_dinv(nb, BS, d_Abrow.p, d_Abcol.p, d_Abval.p, lower, d_Dinv.p, nullptr),
          "build_Dinv");
    bilu_compat::Dev<int> d_PairPtr((size_t)mnnz + 1);
    const size_t pwb = bilu_pairs_ws_bytes(mnnz);
    bilu_compat::Dev<char> pws(pwb);
    int total = 0, nmax = 0;
    check(bilu_pairs_ptr(nb, d_Abrow.p, d_Abcol.p, d_Mptr, d_Mind, lower, d_PairPtr.p, &total,
                         &nmax, pws.p, pwb, nullptr),
          "count_pairs");
    bilu_compat::Dev<int> d_PL((size_t)total), d_PS((size_t)total);
    check(bilu_pairs_fill(nb, d_Abrow.p, d_Abcol.p, d_Mptr, d_Mind, lower, d_PairPtr.p, d_PL.p,
                          d_PS.p, nullptr),
          "fill_pairs");
    check(bilu_isai_compute(nb, BS, d_Abval.p, d_Mptr, d_Mind, lower, d_PairPtr.p, d_PL.p,
                            d_PS.p, d_Dinv.p, lower ? d_MvalL.p : d_MvalU.p, nullptr),
          "isai");
  }

  // 8. BCSC values -> BCSR values (main.cu:782-788)
  check(bilu_reorder_bcsc_to_bcsr(nnzbL, BS, d_mapL.p, d_MvalL.p, d_ValL.p, nullptr), "reorder L");
  check(bilu_reorder_bcsc_to_bcsr(nnzbU, BS, d_mapU.p, d_MvalU.p, d_ValU.p, nullptr), "reorder U");
  bilu_compat::sync("reorder");
  dump(out, "MrowL.i32", MbcsrRowL.data(), MbcsrRowL.size());
  dump(out, "McolL.i32", MbcsrColL.data(), MbcsrColL.size());
  dump_dev(out, "MvalL.f64", d_ValL.p, (size_t)nnzbL * BS2);
  dump(out, "MrowU.i32", MbcsrRowU.data(), MbcsrRowU.size());
  dump(out, "McolU.i32", MbcsrColU.data(), MbcsrColU.size());
  dump_dev(out, "MvalU.f64", d_ValU.p, (size_t)nnzbU * BS2);
  dump(out, "mbcscL.i32", MbrowL.data(), MbrowL.size());
  dump(out, "mindL.i32", McolL.data(), McolL.size());

  // 9. apply x = M_U (M_L b) with b = A x_true, x_true = 0.7 (main.cu:795-846)
  const int n = nrows;
  std::vector<double> x_true(n, 0.7), b(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int p = csrRow[i]; p < csrRow[i + 1]; ++p) b[i] += csrVal[p] * x_true[csrCol[p]];
  dump(out, "b.f64", b.data(), b.size());
  bilu_compat::Dev<double> d_b(b.data(), b.size()), d_y((size_t)n), d_x((size_t)n);
  check(bilu_bcsr_spmv(nb, BS, d_RowL.p, d_ColL.p, d_ValL.p, d_b.p, d_y.p, nullptr), "M_L b");
  check(bilu_bcsr_spmv(nb, BS, d_RowU.p, d_ColU.p, d_ValU.p, d_y.p, d_x.p, nullptr), "M_U y");
  bilu_compat::sync("apply");
  dump_dev(out, "x.f64", d_x.p, (size_t)n);

  // 10. residual check (main.cu:857-866)
  compute_rel_errors_csr<double>(nb * BS, csrRow.data(), csrCol.data(), csrVal.data(), b.data(),
                                 x_true.data(), d_x.p, "M_U M_L apply");

  // 11. the other entry points of the reference's host API on the same data
  std::vector<double> spmv(n);
  bsr_SpMV_tensorcore(bsrRow.data(), bsrCol.data(), bsrVal.data(), nb, nnzb, BS, x_true.data(),
                      nullptr, spmv.data());
  dump(out, "spmv.f64", spmv.data(), spmv.size());
  std::vector<double> lu(bsrVal.size());
  cuda(cudaMemcpy(lu.data(), d_Abval.p, sizeof(double) * lu.size(), cudaMemcpyDeviceToHost), "lu");
  int *crow = nullptr, *ccol = nullptr, cnnz = 0;
  double* cval = nullptr;
  bsr2csr_cusparse(bsrRow.data(), bsrCol.data(), lu.data(), nb, nnzb, BS, &crow, &ccol, &cval,
                   &cnnz);
  dump(out, "csr_row.i32", crow, (size_t)n + 1);
  dump(out, "csr_col.i32", ccol, (size_t)cnnz);
  dump(out, "csr_val.f64", cval, (size_t)cnnz);
  std::vector<double> cape(b);
  csr_cape_SpTRSV(n, crow, ccol, cval, cnnz, cape.data());
  dump(out, "cape.f64", cape.data(), cape.size());
  std::free(crow);
  std::free(ccol);
  std::free(cval);
  bilu_compat::Dev<int> d_r2((size_t)nb + 1), d_c2((size_t)nnzbL);
  bilu_compat::Dev<double> d_v2((size_t)nnzbL * BS2);
  bcsc_to_bcsr(nb, nb, BS, BS, d_MbrowL.p, d_McolL.p, d_MvalL.p, d_r2.p, d_c2.p, d_v2.p);
  dump_dev(out, "bcsr_from_bcsc.f64", d_v2.p, (size_t)nnzbL * BS2);
  std::printf("compat pipeline ok: n %d nb %d nnzb %d nnzbL %d nnzbU %d\n", n, nb, nnzb, nnzbL,
              nnzbU);
  return 0;
}
