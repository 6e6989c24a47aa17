/*
 * CPU oracle for the block-ILU(0) + ISAI preconditioner path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (gmfff/isai_kernel), used by tests/, by the smoke check and by the
 * CPU-baseline leg of bench.py as the checker.  Nothing in the product
 * library (isai_kernel_gb300/) links, loads or calls it.
 *
 * Conventions (same as the reference):
 *   BSR: 0-based int32 rowPtr[nb+1], colInd[nnzb] ascending within a row,
 *        values val[nnzb*bs*bs] row-major inside each block.
 *   BCSC (ISAI patterns): colPtr[nb+1] ("Mbrow"), rowInd ("Mcol") ascending.
 *   Packed BILU(0): strictly-lower blocks hold L, strictly-upper blocks hold U,
 *        the diagonal block holds unit-lower L_kk (strict lower part) and
 *        U_kk (upper part incl. diagonal).
 * Every function returns 0 on success and a negative code on error.
 */
#ifndef BILU_ORACLE_H
#define BILU_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define ORC_OK 0
#define ORC_ERR_ARG (-1)
#define ORC_ERR_PATTERN (-2)
#define ORC_ERR_ZERO_PIVOT (-3)
#define ORC_ERR_NOT_CONVERGED (-6)

int orc_num_threads(void);
void orc_set_num_threads(int n);

/* csr2bsr.h:14-76 */
int orc_csr_to_bsr_count(int n, int bs, const int* csrRow, const int* csrCol,
                         int* bsrRow /* nb+1 */);
int orc_csr_to_bsr_fill(int n, int bs, const int* csrRow, const int* csrCol,
                        const double* csrVal, const int* bsrRow, int* bsrCol,
                        double* bsrVal);

/* isai_bsr.h:246-284 */
int orc_isai_pattern_count(int nb, const int* Arow, const int* Acol, int lower,
                           int* Mptr /* nb+1 */);
int orc_isai_pattern_fill(int nb, const int* Arow, const int* Acol, int lower,
                          const int* Mptr, int* Mind);

/* Symbolic product C = pattern(X A), rows sorted and distinct (ISAI(k));
 * Ccol == NULL counts only. */
int orc_pattern_product(int nb, const int* Xrow, const int* Xcol, const int* Arow,
                        const int* Acol, int* Crow, int* Ccol);

/* bcsc2bcsr.h:11-30 */
int orc_tri_pattern_count(int nb, const int* Arow, const int* Acol, int lower,
                          int* Trow /* nb+1 */);
int orc_tri_pattern_fill(int nb, const int* Arow, const int* Acol, int lower,
                         const int* Trow, int* Tcol);
/* bcsc2bcsr.h:32-60 */
int orc_map_bcsc2bcsr(int nb, const int* cscPtr, const int* cscInd,
                      const int* csrRow, const int* csrCol, int* map,
                      int* bad_row, int* bad_col);
/* bcsc2bcsr.h:63-80 */
int orc_reorder_bcsc_to_bcsr(int nnzb, int bs, const int* map,
                             const double* src, double* dst);
/* bcsc2bcsrAndSpMV.h:76-117 (deterministic: ascending columns per row) */
int orc_bcsc_to_bcsr(int mb, int nbcol, int bs, const int* cscPtr,
                     const int* cscInd, const double* cscVal, int* rowPtr,
                     int* colInd, double* val);
/* bsr2csr.h:19-137 (ROW direction) */
int orc_bsr_to_csr(int mb, int bs, const int* Arow, const int* Acol,
                   const double* Aval, int* csrRow, int* csrCol,
                   double* csrVal);

/* bsrilu.h:20-66 (cuSPARSE bsrilu02, scalar-ILU(0)-on-block-pattern semantics) */
int orc_bsrilu0(int nb, int bs, const int* Arow, const int* Acol, double* Aval,
                int* zero_pivot);
/* scalar ILU(0) on CSR (IKJ), used to pin the block form */
int orc_csr_ilu0(int n, const int* row, const int* col, double* val,
                 int* zero_pivot);

/* isai_bsr.h:91-158 (+ lookup :33-57, Gauss-Jordan :61-88) */
int orc_dinv(int nb, int bs, const int* Arow, const int* Acol,
             const double* Aval, int lower, double* Dinv);

/* isai_bsr.h:1378-1476 + thrust::exclusive_scan main.cu:684 */
int orc_count_pairs_lower(int nb, const int* Arow, const int* Acol,
                          const int* Mptr, const int* Mind, int* counts);
int orc_fill_pairs_lower(int nb, const int* Arow, const int* Acol,
                         const int* Mptr, const int* Mind, const int* PairPtr,
                         int* PairPLocal, int* PairSrc);

/* isai_bsr.h:288-399 */
int orc_isai_lower(int nb, int bs, const double* Aval, const int* Mptr,
                   const int* Mind, const int* PairPtr, const int* PairPLocal,
                   const int* PairSrc, const double* DinvL, double* Mval);
/* isai_bsr.h:161-242 */
int orc_isai_upper(int nb, int bs, const int* Arow, const int* Acol,
                   const double* Aval, const int* Mptr, const int* Mind,
                   const double* DinvU, double* Mval);

/* bcsc2bcsrAndSpMV.h:119-138 (cpu_bcsr_spmv) */
int orc_bcsr_spmv(int mb, int bs, const int* row, const int* col,
                  const double* val, const double* x, double* y);
/* same, with values stored in FP32 and FP32 accumulation */
int orc_bcsr_spmv_f32(int mb, int bs, const int* row, const int* col,
                      const float* val, const float* x, float* y);

/* cape_sptrsv.h:8-53 / :55-103, restated blockwise on the packed BILU(0) */
int orc_sptrsv_lower(int nb, int bs, const int* row, const int* col,
                     const double* val, const double* b, double* x);
int orc_sptrsv_upper(int nb, int bs, const int* row, const int* col,
                     const double* val, const double* b, double* x);

/* residual_check.h:16-71 */
int orc_rel_errors_csr(int n, const int* row, const int* col, const double* val,
                       const double* b, const double* x_true, const double* x,
                       double* rel_err, double* rel_res);

/* Right-preconditioned restarted (F)GMRES(m), modified Gram-Schmidt,
 * Givens rotations, x0 = 0.  The reference has no Krylov solver; this is the
 * oracle that defines iteration counts.  precond: 0 none, 1 ISAI FP64
 * (z = M_U (M_L v)), 2 ISAI with FP32-stored factors and FP32 accumulation,
 * 3 exact BILU(0) (z = U^-1 L^-1 v by the two block triangular solves; the
 * packed factor is passed as Lrow/Lcol/Lval, U is unused), 4 as 2 plus an
 * FP32-stored A in the Arnoldi product (z rounded to FP32, FP32
 * accumulation); the true residual at every restart uses the FP64 A.
 * hist (optional, length maxit+1) receives the residual estimate per
 * iteration. */
int orc_gmres(int nb, int bs, const int* Arow, const int* Acol,
              const double* Aval, const int* Lrow, const int* Lcol,
              const double* Lval, const int* Urow, const int* Ucol,
              const double* Uval, int precond, const double* b, double* x,
              int restart, double tol, int maxit, int* iters, double* relres,
              double* hist);
/* The same with precond 5, the nested (GMRES-IR) mode: each z_j of the FP64
 * outer FGMRES is inner_k steps of FP32 right-preconditioned GMRES on
 * A z = v_j from z = 0 (FP32-stored A, FP32-stored ISAI, FP32 modified
 * Gram-Schmidt, Hessenberg least squares in double); the outer residuals,
 * orthogonalisation and true residual at every restart stay FP64.
 * inner_total (optional) receives the number of inner steps taken. */
int orc_gmres_ex(int nb, int bs, const int* Arow, const int* Acol,
                 const double* Aval, const int* Lrow, const int* Lcol,
                 const double* Lval, const int* Urow, const int* Ucol,
                 const double* Uval, int precond, int inner_k, const double* b,
                 double* x, int restart, double tol, int maxit, int* iters,
                 long long* inner_total, double* relres, double* hist);

#ifdef __cplusplus
}
#endif
#endif
