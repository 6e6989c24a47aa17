/*
 * bilu_isai.h -- C ABI of the GB300 block-ILU(0) + ISAI preconditioner engine
 * (libbilu_isai.so, sm_103a).
 *
 * Drop-in boundary for the host/kernel entry points of gmfff/isai_kernel.
 * Each declaration names the reference function (file:line) it replaces.
 * The reference is header-only CUDA C++ with compile-time BS and exit(1) on
 * error; this ABI takes the block size at run time, returns a status code and
 * never exits.
 *
 * Conventions
 *   - Pointers are DEVICE pointers unless the name starts with h_.
 *   - The caller owns every buffer.  Entry points that need scratch take
 *     (d_ws, ws_bytes); the matching *_ws_bytes() query gives the size.
 *   - BSR/BCSR: int32 rowPtr[nb+1], colInd[nnzb] strictly ascending per row,
 *     values nnzb*bs*bs row-major inside a block.  BCSC (ISAI patterns):
 *     colPtr[nb+1] ("Mbrow"), rowInd ("Mcol") ascending.
 *   - Packed BILU(0) as cuSPARSE bsrilu02: strictly lower blocks = L,
 *     diagonal block = unit-lower L_kk (strict lower part) and U_kk,
 *     strictly upper blocks = U.
 *   - Supported block sizes: 4, 5, 8.  Preconditioner choice: BILU_FP64
 *     (plain ISAI), BILU_FP32 (FP32-stored ISAI factors, FP32
 *     accumulation), BILU_ILU (exact BILU(0): two block triangular solves
 *     per apply, FP64), BILU_FP32_INNER (FP32 ISAI and an FP32-stored A in
 *     the Arnoldi products; orthogonalisation, true residuals and restarts
 *     stay FP64) or BILU_ILU_FP32 (exact BILU(0) applied in FP32 on an
 *     FP32 copy of the factor; FP64 operator product and Krylov vectors).
 *   - stream may be NULL (legacy default stream).  Calls are asynchronous
 *     unless documented to return a host value (h_ outputs synchronise).
 */
#ifndef BILU_ISAI_H
#define BILU_ISAI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* bilu_stream_t; /* == cudaStream_t */

enum bilu_status {
  BILU_OK = 0,
  BILU_ERR_ARG = -1,           /* bad size, block size, pointer or flag */
  BILU_ERR_PATTERN = -2,       /* missing diagonal block, unsorted row, ... */
  BILU_ERR_ZERO_PIVOT = -3,    /* singular pivot; index via h_info */
  BILU_ERR_TIMEOUT = -4,       /* a sync-free wait gave up (bounded spin) */
  BILU_ERR_CUDA = -5,          /* CUDA runtime error (launch, copy) */
  BILU_ERR_NOT_CONVERGED = -6, /* Krylov solver hit maxit */
  BILU_ERR_WORKSPACE = -7,     /* workspace too small */
  BILU_ERR_UNSUPPORTED = -8,   /* block size / precision / file kind not built */
  BILU_ERR_IO = -9             /* file missing, unreadable, malformed or corrupt */
};

enum bilu_precision {
  BILU_FP64 = 0,
  BILU_FP32 = 1,
  BILU_ILU = 2,
  BILU_FP32_INNER = 3,
  BILU_ILU_FP32 = 4,
  BILU_NESTED = 5
};

const char* bilu_status_string(int status);
int bilu_version(void);
/* last CUDA error seen by the library on this thread (cudaError_t value) */
int bilu_last_cuda_error(void);
/* number of kernels this library has launched since it was loaded */
unsigned long long bilu_kernel_launches(void);

/* ------------------------------------------------------------------ */
/* Format conversions and patterns                                     */
/* ------------------------------------------------------------------ */

/* Replaces csr_to_bsr5 (csr2bsr.h:14).  Two phases: rowcounts writes
 * d_bsrRowPtr[nb+1] and *h_nnzb; fill writes colInd/val.  Duplicate scalar
 * entries are summed, block columns come out ascending. */
size_t bilu_csr_to_bsr_ws_bytes(int n, int bs);
int bilu_csr_to_bsr_rowptr(int n, int bs, const int* d_csrRowPtr, const int* d_csrColInd,
                           int* d_bsrRowPtr, int* h_nnzb, void* d_ws, size_t ws_bytes,
                           bilu_stream_t stream);
int bilu_csr_to_bsr_fill(int n, int bs, const int* d_csrRowPtr, const int* d_csrColInd,
                         const double* d_csrVal, const int* d_bsrRowPtr, int* d_bsrColInd,
                         double* d_bsrVal, bilu_stream_t stream);

/* Replaces bsr2csr_cusparse (bsr2csr.h:19), row direction, on the device:
 * csr arrays have mb*bs+1, nnzb*bs*bs, nnzb*bs*bs entries. */
int bilu_bsr_to_csr(int mb, int bs, const int* d_bsrRowPtr, const int* d_bsrColInd,
                    const double* d_bsrVal, int* d_csrRowPtr, int* d_csrColInd,
                    double* d_csrVal, bilu_stream_t stream);

/* Replaces build_bcsc_pattern_from_bsr_scalarILU (isai_bsr.h:246): ISAI
 * pattern of M_L (lower=1) or M_U (lower=0) in BCSC.  Two phases. */
size_t bilu_isai_pattern_ws_bytes(int nb, int nnzb); /* nnzb of A */
int bilu_isai_pattern_colptr(int nb, const int* d_Arow, const int* d_Acol, int lower,
                             int* d_Mptr, int* h_nnz, void* d_ws, size_t ws_bytes,
                             bilu_stream_t stream);
int bilu_isai_pattern_fill(int nb, const int* d_Arow, const int* d_Acol, int lower,
                           const int* d_Mptr, int* d_Mind, void* d_ws, size_t ws_bytes,
                           bilu_stream_t stream);

/* Symbolic block-pattern product C = pattern(X A) (no counterpart in the
 * reference; ISAI(k) uses the lower / upper triangle of pattern(A^k) as the
 * M_L / M_U pattern, and the pattern functions of this section accept it in
 * place of A's).  Two phases like the others: row pointer (h_nnz = nnz(C)),
 * then columns (sorted, distinct).  A row that gathers more than 1024
 * candidate columns returns BILU_ERR_UNSUPPORTED with its index in
 * *h_bad_row. */
size_t bilu_pattern_product_ws_bytes(int nb);
int bilu_pattern_product_rowptr(int nb, const int* d_Xrow, const int* d_Xcol, const int* d_Arow,
                                const int* d_Acol, int* d_Crow, int* h_nnz, int* h_bad_row,
                                void* d_ws, size_t ws_bytes, bilu_stream_t stream);
int bilu_pattern_product_fill(int nb, const int* d_Xrow, const int* d_Xcol, const int* d_Arow,
                              const int* d_Acol, const int* d_Crow, int* d_Ccol, void* d_ws,
                              size_t ws_bytes, bilu_stream_t stream);

/* Replaces build_triangular_bcsr_pattern_from_A (bcsc2bcsr.h:11). */
size_t bilu_tri_pattern_ws_bytes(int nb);
int bilu_tri_pattern_rowptr(int nb, const int* d_Arow, const int* d_Acol, int lower,
                            int* d_Trow, int* h_nnz, void* d_ws, size_t ws_bytes,
                            bilu_stream_t stream);
int bilu_tri_pattern_fill(int nb, const int* d_Arow, const int* d_Acol, int lower,
                          const int* d_Trow, int* d_Tcol, bilu_stream_t stream);

/* Replaces build_map_bcsc2bcsr_host (bcsc2bcsr.h:32).  Returns
 * BILU_ERR_PATTERN (and the first missing (row, col) in h_bad[2]) where the
 * reference exits. */
int bilu_map_bcsc2bcsr(int nb, const int* d_cscPtr, const int* d_cscInd, const int* d_csrRow,
                       const int* d_csrCol, int* d_map, int* h_bad, void* d_ws,
                       size_t ws_bytes, bilu_stream_t stream);
size_t bilu_map_ws_bytes(void);

/* Replaces reorder_bcsc_val_to_bcsr_bs5 (bcsc2bcsr.h:63). */
int bilu_reorder_bcsc_to_bcsr(int nnzb, int bs, const int* d_map, const double* d_src,
                              double* d_dst, bilu_stream_t stream);

/* Replaces bcsc_to_bcsr (bcsc2bcsrAndSpMV.h:76); deterministic: columns
 * ascending inside each row, row_ptr[mb] written. */
size_t bilu_bcsc_to_bcsr_ws_bytes(int mb, int nnzb);
int bilu_bcsc_to_bcsr(int mb, int nbcol, int bs, const int* d_cscPtr, const int* d_cscInd,
                      const double* d_cscVal, int* d_rowPtr, int* d_colInd, double* d_val,
                      void* d_ws, size_t ws_bytes, bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Factorisation                                                       */
/* ------------------------------------------------------------------ */

/* Replaces bsrilu02_inplace (bsrilu.h:20; cuSPARSE bsrilu02, row direction,
 * no level information): BILU(0) in place.  A level analysis of the lower
 * DAG picks the schedule: levels of at least 4096 block rows on average and
 * no row with more than 32 dependencies -> one cooperative launch with a
 * bounded grid barrier per level (a bs-lane group per row); otherwise
 * sync-free (warp per row, atomic tickets in level order, bounded waits on
 * ready flags).
 * h_info[0] receives the first block row with a zero pivot (or -1);
 * BILU_ERR_ZERO_PIVOT then. */
size_t bilu_bsrilu0_ws_bytes(int nb, int nnzb);
int bilu_bsrilu0(int nb, int nnzb, int bs, const int* d_row, const int* d_col, double* d_val,
                 int* h_info, void* d_ws, size_t ws_bytes, bilu_stream_t stream);
/* Same with the schedule chosen by the caller: -1 as recommended by the
 * analysis, 0 level schedule, 1 sync-free (both give identical factors). */
int bilu_bsrilu0_ex(int nb, int nnzb, int bs, const int* d_row, const int* d_col, double* d_val,
                    int schedule, int* h_info, void* d_ws, size_t ws_bytes, bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* ISAI setup                                                          */
/* ------------------------------------------------------------------ */

/* Replaces build_DinvL_from_BSR5_kernel_fix (isai_bsr.h:91, lower=1) and
 * build_DinvU_from_BSR5_kernel_fix (isai_bsr.h:126, lower=0). */
int bilu_build_dinv(int nb, int bs, const int* d_Arow, const int* d_Acol, const double* d_Aval,
                    int lower, double* d_Dinv, bilu_stream_t stream);

/* Replaces count_pairs_lower_kernel_v2 (isai_bsr.h:1378) + the exclusive
 * scan (main.cu:684) + fill_pairs_lower_kernel_v2 (isai_bsr.h:1427).
 * lower=0 builds the analogous list for M_U (p > idx, descending p), which
 * the reference resolves by binary search inside its ISAI-U kernel.
 * pairs_ptr writes d_PairPtr[Mnnz+1] and *h_total; fill writes the lists.
 * h_nmax (optional) receives the longest ISAI column. */
size_t bilu_pairs_ws_bytes(int mnnz);
int bilu_pairs_ptr(int nb, const int* d_Arow, const int* d_Acol, const int* d_Mptr,
                   const int* d_Mind, int lower, int* d_PairPtr, int* h_total, int* h_nmax,
                   void* d_ws, size_t ws_bytes, bilu_stream_t stream);
int bilu_pairs_fill(int nb, const int* d_Arow, const int* d_Acol, const int* d_Mptr,
                    const int* d_Mind, int lower, const int* d_PairPtr, int* d_PairPLocal,
                    int* d_PairSrc, bilu_stream_t stream);

/* Replaces the ISAI-L kernels (isai_bsr.h:288,733,869,976,1287,1332,1355,
 * cacheY_isai.h:159) for lower=1 and isai_upper_bsr5_warpcol_with_Dinv_kernel
 * (isai_bsr.h:161) for lower=0: M values in BCSC order (nnzbM*bs*bs). */
int bilu_isai_compute(int nb, int bs, const double* d_Aval, const int* d_Mptr, const int* d_Mind,
                      int lower, const int* d_PairPtr, const int* d_PairPLocal,
                      const int* d_PairSrc, const double* d_Dinv, double* d_Mval,
                      bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Apply: SpMV / SpMM / ISAI apply                                     */
/* ------------------------------------------------------------------ */

/* Replaces bcsr_spmv (bcsc2bcsrAndSpMV.h:49) and bsr_SpMV_tensorcore
 * (bsr_tensor_SpMV.h:402): y = M x.  FP64 values and vectors.  Rows of more
 * than 64 blocks are summed by a whole CTA instead of one lane group; the
 * first call with a given d_row array (and mb, bs) finds out whether there
 * are such rows with a synchronising reduction over d_row, later calls
 * reuse the answer (a stale answer after reusing d_row for another pattern
 * only costs speed).  The same holds for bilu_bcsr_spmv_f32 and
 * bilu_isai_apply. */
int bilu_bcsr_spmv(int mb, int bs, const int* d_row, const int* d_col, const double* d_val,
                   const double* d_x, double* d_y, bilu_stream_t stream);
/* The SpMV layout word of a pattern, as cached by the entry points above:
 * bit 0 (1) when rows of more than 64 blocks are present (the kernel in
 * which the CTA shares such rows); bit 1 (2) when rows hold more than 5
 * blocks on average (FP32-stored values: one block row per lane group
 * instead of two).  Synchronises the stream on the first query of a
 * pattern. */
int bilu_spmv_layout(int mb, int bs, const int* d_row, bilu_stream_t stream, int* h_layout);
/* FP32-stored values, FP32 accumulation; x and y each FP64 or FP32
 * (x_fp32 / y_fp32 flags). */
int bilu_bcsr_spmv_f32(int mb, int bs, const int* d_row, const int* d_col, const float* d_val,
                       const void* d_x, int x_fp32, void* d_y, int y_fp32, bilu_stream_t stream);
/* Multi-RHS: Y[n, k] = M X[n, k] (row-major, ld = k), k <= 64, FP64. */
int bilu_bcsr_spmm(int mb, int bs, int k, const int* d_row, const int* d_col,
                   const double* d_val, const double* d_X, double* d_Y, bilu_stream_t stream);
/* Multi-RHS with FP32-stored values (FP32 accumulation), FP64 X/Y. */
int bilu_bcsr_spmm_f32(int mb, int bs, int k, const int* d_row, const int* d_col,
                       const float* d_val, const double* d_X, double* d_Y,
                       bilu_stream_t stream);
/* Convert FP64 values to FP32 storage (round to nearest). */
int bilu_convert_f64_to_f32(size_t count, const double* d_src, float* d_dst,
                            bilu_stream_t stream);

/* Preconditioner apply of main.cu:817-846: y = M_L b, x = M_U y.
 * prec BILU_FP64: d_Lval/d_Uval are double*, d_tmp holds n doubles.
 * prec BILU_FP32: float* values, d_tmp holds n floats; b and x FP64. */
int bilu_isai_apply(int nb, int bs, int prec, const int* d_Lrow, const int* d_Lcol,
                    const void* d_Lval, const int* d_Urow, const int* d_Ucol,
                    const void* d_Uval, const double* d_b, void* d_tmp, double* d_x,
                    bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Sync-free block triangular solves                                   */
/* ------------------------------------------------------------------ */

/* Replaces spTrSolveL / spTrSolveU (cape_sptrsv.h:8,55) and
 * csr_cape_SpTRSV (cape_sptrsv.h:105), blockwise on the packed BILU(0):
 * lower: unit-lower L x = b; upper: U x = b.  One-shot form: level analysis
 * then the schedule it recommends (see the analysis / solve split below).
 * d_x must not be d_b (BILU_ERR_ARG): the level-order solve marks every x
 * entry pending before it starts. */
size_t bilu_sptrsv_ws_bytes(int nb, int nnzb);
int bilu_sptrsv(int nb, int nnzb, int bs, const int* d_row, const int* d_col, const double* d_val,
                int lower, const double* d_b, double* d_x, void* d_ws, size_t ws_bytes,
                bilu_stream_t stream);
/* Analysis / solve split (as cuSPARSE bsrsv2 analysis + solve,
 * BILU_cusparse.h:203-220): the analysis (diagonal positions, dependency
 * levels and the rows in level order; bilu_sptrsv_analysis_bytes(nb) bytes
 * in d_info, scratch bilu_sptrsv_analysis_ws_bytes) is computed once per
 * pattern and triangle, together with a schedule recommendation: the level
 * order when no row has more than 8 dependencies, the sync-free schedule
 * otherwise (the record's fourth word holds BILU(0)'s recommendation).
 * bilu_sptrsv_solve runs the recommended schedule; bilu_sptrsv_solve_level
 * forces the level-order kernel (one cooperative launch; rows taken in level
 * order by lane groups, each waiting only for the x entries it reads, which
 * start as a signalling-NaN pattern; rows with more than 32 dependencies
 * instead take a warp each and a bounded grid barrier per level);
 * bilu_sptrsv_solve_syncfree forces the sync-free kernel of the reference's
 * design (block rows taken by atomic tickets in level order, per-row ready
 * flags polled by the dependent rows, every wait bounded:
 * BILU_ERR_TIMEOUT).  All give identical x. */
size_t bilu_sptrsv_analysis_bytes(int nb);
size_t bilu_sptrsv_analysis_ws_bytes(int nb, int nnzb);
size_t bilu_sptrsv_solve_ws_bytes(int nb);
int bilu_sptrsv_analysis(int nb, int nnzb, int bs, const int* d_row, const int* d_col, int lower,
                         void* d_info, void* d_ws, size_t ws_bytes, bilu_stream_t stream);
int bilu_sptrsv_solve(int nb, int bs, const int* d_row, const int* d_col, const double* d_val,
                      int lower, int unit, const void* d_info, const double* d_b, double* d_x,
                      void* d_ws, size_t ws_bytes, bilu_stream_t stream);
int bilu_sptrsv_solve_level(int nb, int bs, const int* d_row, const int* d_col,
                            const double* d_val, int lower, int unit, const void* d_info,
                            const double* d_b, double* d_x, void* d_ws, size_t ws_bytes,
                            bilu_stream_t stream);
int bilu_sptrsv_solve_syncfree(int nb, int bs, const int* d_row, const int* d_col,
                               const double* d_val, int lower, int unit, const void* d_info,
                               const double* d_b, double* d_x, void* d_ws, size_t ws_bytes,
                               bilu_stream_t stream);
/* General form: lower/upper triangle of a packed factor, unit or non-unit
 * diagonal (bilu_sptrsv uses lower+unit and upper+non-unit). */
int bilu_sptrsv_ex(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                   const double* d_val, int lower, int unit, const double* d_b, double* d_x,
                   void* d_ws, size_t ws_bytes, bilu_stream_t stream);
/* Transposed solves over the BCSC view of the same packed factor (adjoint):
 * lower: L^T x = b (upper-triangular, unit diagonal); upper: U^T x = b.
 * The workspace holds the transposed factor. */
size_t bilu_sptrsv_transpose_ws_bytes(int nb, int nnzb, int bs);
int bilu_sptrsv_transpose(int nb, int bs, const int* d_row, const int* d_col,
                          const double* d_val, int lower, const double* d_b, double* d_x,
                          void* d_ws, size_t ws_bytes, bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Adjoint helpers                                                     */
/* ------------------------------------------------------------------ */

/* BCSC view of a BCSR matrix as a BCSR matrix of the transpose: pattern
 * transposed (columns ascending) and every block transposed. */
size_t bilu_bsr_transpose_ws_bytes(int mb, int nnzb);
int bilu_bsr_transpose(int mb, int bs, const int* d_row, const int* d_col, const double* d_val,
                       int* d_trow, int* d_tcol, double* d_tval, void* d_ws, size_t ws_bytes,
                       bilu_stream_t stream);
/* y = M^T x for a BCSR matrix (transposed SpMV, deterministic). */
size_t bilu_spmv_transpose_ws_bytes(int mb, int nnzb);
int bilu_bcsr_spmv_transpose(int mb, int bs, const int* d_row, const int* d_col,
                             const double* d_val, const double* d_x, double* d_y,
                             void* d_ws, size_t ws_bytes, bilu_stream_t stream);
/* Masked outer product: G[p] (+)= scale * u[row(p)] v[col(p)]^T for every
 * stored block p (gradient of block values).  accumulate: add into G. */
int bilu_masked_outer(int mb, int bs, const int* d_row, const int* d_col, const double* d_u,
                      const double* d_v, double scale, int accumulate, double* d_G,
                      bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Verification                                                        */
/* ------------------------------------------------------------------ */

/* Replaces compute_rel_errors_csr (residual_check.h:17) on the device for a
 * BSR matrix: h_out[0] = ||x - x_true|| / ||x_true|| (x_true may be NULL),
 * h_out[1] = ||b - A x|| / ||b||. */
size_t bilu_rel_errors_ws_bytes(int nb, int bs);
int bilu_rel_errors(int nb, int bs, const int* d_row, const int* d_col, const double* d_val,
                    const double* d_b, const double* d_x_true, const double* d_x,
                    double* h_out, void* d_ws, size_t ws_bytes, bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Engine handle: setup + preconditioned (F)GMRES                      */
/* ------------------------------------------------------------------ */

typedef struct bilu_ctx bilu_ctx;

/* Creates a handle bound to the current device and `stream`.  The handle
 * owns the device memory of everything it builds. */
int bilu_ctx_create(bilu_ctx** ctx, bilu_stream_t stream);
int bilu_ctx_destroy(bilu_ctx* ctx);

/* Copies the BSR matrix (device pointers; the values are not modified) and
 * runs the whole setup on the GPU: BILU(0), ISAI patterns, pair lists, Dinv,
 * ISAI-L/U, BCSC->BCSR reorder, FP32 copies when prec_mask has
 * 1 << BILU_FP32, level analyses of both triangles when it has
 * 1 << BILU_ILU, FP32 copies of the ISAI factors and of A when it has
 * 1 << BILU_FP32_INNER, an FP32 copy of the factor and of its reciprocal
 * pivots when it has 1 << BILU_ILU_FP32 (built when no row of either
 * triangle has more than 32 dependencies), FP32 copies of the ISAI factors
 * and of A when it has 1 << BILU_NESTED.  A prec_mask of exact-ILU bits
 * alone builds BILU(0) and the level analyses only (no ISAI; solves in the
 * other modes then return BILU_ERR_ARG).
 * h_times (optional, 4 doubles, milliseconds): factor (BILU(0)'s level
 * analysis, its match lists and the factorisation, with the copies of A), patterns (ISAI
 * patterns and pair lists), isai (Dinv, column solves, reorders), total.
 * The structure steps run first, then the value steps. */
int bilu_ctx_setup(bilu_ctx* ctx, int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                   const double* d_val, int prec_mask, double* h_times);

/* ISAI level for the next bilu_ctx_setup: k = 1 (default) uses the
 * pattern of A as the reference does; k = 2, 3 use the pattern of A^k
 * (ISAI(k): denser approximate inverses, fewer iterations, a costlier
 * apply). */
int bilu_ctx_set_isai_level(bilu_ctx* ctx, int k);
/* Schedule of the next setup's BILU(0) and of the exact-ILU solves: -1 (the
 * default) as the level analyses recommend, 0 level schedule, 1 sync-free. */
int bilu_ctx_set_schedule(bilu_ctx* ctx, int schedule);

/* Right-preconditioned restarted (F)GMRES(restart) with modified
 * Gram-Schmidt and Givens rotations, x0 = 0: prec BILU_FP64 applies the FP64 ISAI, BILU_FP32 the
 * FP32-stored ISAI (flexible GMRES, FP64 residuals/orthogonalisation,
 * FP64 true residual at every restart = iterative refinement), BILU_ILU the
 * exact BILU(0) by level-scheduled triangular solves, BILU_FP32_INNER the
 * FP32 ISAI with the FP32-stored A in the Arnoldi products (the true FP64
 * residual at every restart corrects the inner precision, as in GMRES with
 * iterative refinement), BILU_NESTED the nested GMRES-IR form: every
 * preconditioned vector z_j of the FP64 flexible outer GMRES is a fixed
 * number of steps (bilu_ctx_set_inner, default 8) of right-preconditioned
 * GMRES in FP32 on A z = v_j with the FP32-stored A and ISAI, FP32
 * Gram-Schmidt and the Hessenberg least squares on the device; the outer
 * residuals, orthogonalisation and true residual at every restart stay
 * FP64.  h_iters then counts outer steps (bilu_ctx_inner_steps gives the
 * inner ones); prec -1 runs without preconditioner.  A choice the setup did not build returns BILU_ERR_ARG.  h_iters, h_relres: iteration count and final true
 * relative residual.  h_hist (optional, maxit+1 doubles) receives the
 * residual estimate after every iteration. */
int bilu_ctx_solve(bilu_ctx* ctx, int prec, const double* d_b, double* d_x, int restart,
                   double tol, int maxit, int* h_iters, double* h_relres, double* h_hist);

/* Counters of the last solve: h_out[0] = Arnoldi steps, h_out[1] = restart
 * cycles. */
int bilu_ctx_stats(bilu_ctx* ctx, long long* h_out);
/* Inner FP32 GMRES steps per outer step of the nested mode (1..32; default
 * 8), for the next solve; no counterpart in the reference. */
int bilu_ctx_set_inner(bilu_ctx* ctx, int k);
/* Inner steps the last BILU_NESTED solve took in total. */
int bilu_ctx_inner_steps(bilu_ctx* ctx, long long* h_steps);

/* Preconditioner switch by measurement (SpTRSV apply vs SpMV apply):
 * runs up to `cycles` restart cycles (fewer when it reaches tol) from x0 = 0
 * with each choice whose bit
 * (1 << BILU_FP64 / BILU_FP32 / BILU_ILU / BILU_FP32_INNER / BILU_ILU_FP32)
 * is in `mask` and that the setup built, and returns in *h_choice the one
 * with the largest residual reduction per second over its last cycle
 * (restarted GMRES gains most in its first cycle); h_rate (optional, 4
 * doubles, 5 when mask has 1 << BILU_ILU_FP32) receives the scores in
 * decimal digits per second, indexed by choice. */
int bilu_ctx_select(bilu_ctx* ctx, const double* d_b, int restart, int cycles, double tol,
                    int mask, int* h_choice, double* h_rate);

/* Host-buffer convenience (the end-to-end call): copies A and b from host
 * memory, runs the setup `prec` needs (any bilu_precision) and the solve,
 * copies x back.  The values and b copy on a second stream while the
 * setup's structure phase (level analysis, BILU(0)'s match lists, ISAI
 * patterns, pair lists) runs on `stream`; with pinned host buffers the two
 * overlap.  The uploaded values become the handle's copy of A (no second
 * device copy).  Device buffers of
 * this call and of every handle come from a memory pool private to the
 * library that keeps freed memory reserved, so repeated calls do not map
 * their buffers again. */
int bilu_solve_host(int nb, int nnzb, int bs, const int* h_row, const int* h_col,
                    const double* h_val, const double* h_b, double* h_x, int prec, int restart,
                    double tol, int maxit, int* h_iters, double* h_relres, double* h_times,
                    bilu_stream_t stream);

/* Accessors for the arrays a handle built (device pointers, owned by the
 * handle): which = 0 A factored values (double), 1 M_L BCSR rowptr,
 * 2 M_L colind, 3 M_L values (double), 4 M_U rowptr, 5 M_U colind,
 * 6 M_U values (double), 7 M_L values (float), 8 M_U values (float).
 * h_count receives the number of elements. */
int bilu_ctx_get(bilu_ctx* ctx, int which, const void** d_ptr, long long* h_count);

/* ------------------------------------------------------------------ */
/* Host-side ingest                                                    */
/* ------------------------------------------------------------------ */

/* Replaces read_matrix_market_to_csr (read_matrix.h:12): a Matrix Market
 * coordinate file to 0-based CSR with rows sorted by column (ties keep file
 * order, duplicates are kept, as the reference keeps them).  Real and
 * integer values; "pattern" entries read as 1.0; "symmetric" / "hermitian"
 * files are expanded to both triangles and "skew-symmetric" ones with the
 * mirrored value negated (the reference ignores the symmetry qualifier).
 * Two calls: with h_row/h_col/h_val NULL it returns the sizes (h_nnz = the
 * expanded entry count); then with arrays of nrows+1 / h_nnz / h_nnz
 * elements (*h_nnz = their capacity) it fills them.  BILU_ERR_IO for a
 * missing file, a missing banner or size line, or a bad entry (its 0-based
 * index in *h_bad_entry); BILU_ERR_UNSUPPORTED for array or complex files. */
int bilu_mtx_read(const char* path, int* h_nrows, int* h_ncols, long long* h_nnz, int* h_row,
                  int* h_col, double* h_val, long long* h_bad_entry);
/* Binary BSR file (no counterpart in the reference): a 40-byte header
 * (magic "BILUBSR1", block size, nb, nnzb, a 64-bit FNV-1a checksum of the
 * payload), then rowptr[nb+1], colind[nnzb] (int32) and the values
 * (nnzb*bs*bs doubles, row-major blocks), little-endian.  bilu_bsr_load
 * with NULL arrays reads the header only; with arrays it checks the sizes
 * against *h_nb, *h_nnzb and *h_bs, the checksum (BILU_ERR_IO on mismatch) and
 * the structure (BILU_ERR_PATTERN). */
int bilu_bsr_save(const char* path, int nb, int nnzb, int bs, const int* h_row, const int* h_col,
                  const double* h_val);
int bilu_bsr_load(const char* path, int* h_nb, int* h_nnzb, int* h_bs, int* h_row, int* h_col,
                  double* h_val);

/* ------------------------------------------------------------------ */
/* Batched multi-RHS solves (no counterpart in the reference)          */
/* ------------------------------------------------------------------ */

typedef struct bilu_batch bilu_batch;

int bilu_batch_create(bilu_batch** batch, bilu_stream_t stream);
int bilu_batch_destroy(bilu_batch* batch);
/* S systems given as one block-diagonal BSR matrix with global column
 * indices: system s owns block rows [h_sys_ptr[s], h_sys_ptr[s+1]) and every
 * block of those rows must lie in the same range (BILU_ERR_PATTERN
 * otherwise).  Runs the whole setup once on the union (FP32 ISAI included);
 * the device arrays must stay valid until the batch is destroyed. */
int bilu_batch_setup(bilu_batch* batch, int S, const int* h_sys_ptr, int nnzb, int bs,
                     const int* d_row, const int* d_col, const double* d_val, double* h_times);
/* k (<= 32) right-hand sides per system, B and X row-major [nb*bs, k]:
 * every (system, right-hand side) pair runs FGMRES(restart) with the FP32
 * ISAI apply (BSR x dense SpMM, one launch over the batch), FP64 operator,
 * modified Gram-Schmidt segmented by system and device-side Givens
 * rotations; each Arnoldi step is a replayed CUDA graph.  Systems are
 * processed in contiguous waves whose Krylov storage fits mem_budget bytes
 * (<= 0: 64 GiB).  h_iters / h_relres [S*k] (system-major) receive the
 * per-pair iteration counts and final true relative residuals; h_stats (4):
 * waves, graph launches, pair-steps, solve milliseconds. */
int bilu_batch_solve(bilu_batch* batch, int k, const double* d_B, double* d_X, int restart,
                     double tol, int maxit, long long mem_budget, int* h_iters,
                     double* h_relres, double* h_stats);
/* Autotuner result: h_cfg = {rows per warp of the operator SpMM, of the
 * apply SpMM, tile rows (fixed: tiles partition the dot products)};
 * h_ms[6] = timed candidates (1, 2, 4 rows per warp) for the operator and
 * the apply. */
int bilu_batch_tuning(bilu_batch* batch, int* h_cfg, double* h_ms);
/* How bilu_batch_solve runs an Arnoldi step: 1 (default) as one
 * cooperative launch over every (system, tile) of the wave -- the FP32
 * apply, the operator SpMM, the Gram-Schmidt sweeps with their per-system
 * sums, the normalisation and the Givens step, with bounded grid barriers
 * between them; 0 as a replayed CUDA graph of one launch per phase.  Both
 * give the same bits. */
int bilu_batch_set_schedule(bilu_batch* batch, int persistent);

/* ------------------------------------------------------------------ */
/* Allocation-free solve                                               */
/* ------------------------------------------------------------------ */

/* No counterpart in the reference.  The sync-free block triangular solve of
 * bilu_sptrsv for callers that cannot allocate device memory (hosts whose
 * device memory belongs to a fixed arena or budget, plugins limited to the
 * buffers they are handed): it takes only inputs and the output and keeps
 * its scratch in one fixed, file-scope device array of about 6 MiB that
 * every device holds from the moment the library is loaded until the
 * process exits.  It never calls cudaMalloc, cudaFree or any allocating
 * routine.  Like bilu_sptrsv it waits on the stream before it returns (the
 * pattern check and the error word are read back to the host).
 *   - nb may not exceed bilu_sptrsv_noalloc_max_rows() (262144 block rows);
 *     larger systems return BILU_ERR_WORKSPACE without touching the GPU.
 *   - d_b and d_x may not be the same buffer (BILU_ERR_ARG); a block row
 *     without a stored diagonal block returns BILU_ERR_PATTERN.
 *   - The first call on a device looks up the array's device address with
 *     cudaGetSymbolAddress (no allocation) and caches it.
 *   - The call synchronises its stream, so it cannot be recorded into a
 *     CUDA graph.
 *   - All calls share the one array and every call re-initialises the parts
 *     that must start at zero.  Calls whose executions overlap on the GPU
 *     (different streams, or different host threads) race on it: serialise
 *     them. */
int bilu_sptrsv_noalloc_max_rows(void);
int bilu_sptrsv_noalloc(int nb, int bs, const int* d_row, const int* d_col, const double* d_val,
                        int lower, const double* d_b, double* d_x, bilu_stream_t stream);

/* ------------------------------------------------------------------ */
/* Testing hook (no counterpart in the reference)                      */
/* ------------------------------------------------------------------ */

/* bilu_sptrsv with block row withhold_row never publishing its ready flag and
 * a spin budget of spin_limit polls (<= the built-in limit): the rows that
 * depend on it give up and the call returns BILU_ERR_TIMEOUT instead of
 * hanging.  Exercises the failure path of the sync-free kernels. */
int bilu_debug_sptrsv_withhold(int nb, int bs, const int* d_row, const int* d_col,
                               const double* d_val, int lower, const double* d_b, double* d_x,
                               int withhold_row, long long spin_limit, void* d_ws,
                               size_t ws_bytes, bilu_stream_t stream);
/* The same for the level-order (flow) solve: block row withhold_row never
 * stores its x entries, the rows reading them give up after spin_limit
 * polls, BILU_ERR_TIMEOUT.  Workspace bilu_sptrsv_ws_bytes(nb, nnzb);
 * patterns with rows of more than 32 dependencies: BILU_ERR_UNSUPPORTED. */
int bilu_debug_sptrsv_withhold_flow(int nb, int nnzb, int bs, const int* d_row, const int* d_col,
                                    const double* d_val, int lower, const double* d_b,
                                    double* d_x, int withhold_row, long long spin_limit,
                                    void* d_ws, size_t ws_bytes, bilu_stream_t stream);
/* Sets the SpMV layout word (0 to 3, see bilu_spmv_layout) the entry
 * points use for the pattern (d_row, mb, bs), replacing the one they found.
 * Every layout gives the product to within rounding for any pattern; this
 * exercises the kernels the check would not pick for a given pattern. */
int bilu_debug_spmv_layout_set(int mb, int bs, const int* d_row, int layout);
/* One modified Gram-Schmidt step of the Krylov solvers' orthogonalisation
 * kernel (one cooperative launch): w is orthogonalised against the j+1
 * basis vectors V[0..j] (stride ldv elements, FP64, or FP32 when fp32 != 0)
 * by fused sweeps; d_h[0..j] receives h_i = v_i . w, d_h[j+1] = ||w||^2,
 * and d_vnext (optional) w / ||w||.  Vectors start on 16-byte boundaries;
 * workspace bilu_debug_mgs_step_ws_bytes().  Synchronises the stream;
 * returns BILU_ERR_TIMEOUT if a grid barrier gave up. */
size_t bilu_debug_mgs_step_ws_bytes(void);
int bilu_debug_mgs_step(long long n, int fp32, const void* d_V, long long ldv, int j, void* d_w,
                        double* d_h, void* d_vnext, void* d_ws, size_t ws_bytes,
                        bilu_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* BILU_ISAI_H */
