/*
 * CPU oracle for the block-ILU(0) + ISAI preconditioner path.
 *
 * TEST INFRASTRUCTURE ONLY (checker, never the thing measured or shipped).
 * A plain-C restatement of the reference (gmfff/isai_kernel); each function
 * cites the reference file:line whose behaviour it restates.  Compiled with
 * -ffp-contract=off so results are identical on x86-64 and aarch64 hosts.
 * Loops with independent iterations use OpenMP; every reduction is summed in
 * fixed chunks so results do not depend on the thread count.
 */
#include "bilu_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXBS 8
#define CHUNK 8192

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* ------------------------------------------------------------------------ */
/* csr2bsr.h:14-76: per block row, blocks keyed by block column in a sorted
 * map; duplicates accumulate (first contribution assigns, later ones add). */
static int block_row_cols(int br, int bs, const int* csrRow, const int* csrCol,
                          int** buf, int* cap) {
  int r0 = br * bs, r1 = r0 + bs;
  int len = csrRow[r1] - csrRow[r0];
  if (len > *cap) {
    free(*buf);
    *cap = len > 64 ? len : 64;
    *buf = (int*)malloc(sizeof(int) * (size_t)(*cap));
  }
  int m = 0;
  for (int p = csrRow[r0]; p < csrRow[r1]; ++p) (*buf)[m++] = csrCol[p] / bs;
  qsort(*buf, (size_t)m, sizeof(int), cmp_int);
  int u = 0;
  for (int i = 0; i < m; ++i)
    if (u == 0 || (*buf)[u - 1] != (*buf)[i]) (*buf)[u++] = (*buf)[i];
  return u;
}

int orc_csr_to_bsr_count(int n, int bs, const int* csrRow, const int* csrCol,
                         int* bsrRow) {
  if (bs < 1 || bs > MAXBS || n < 0 || n % bs) return ORC_ERR_ARG;
  int nb = n / bs;
  int* buf = NULL;
  int cap = 0;
  bsrRow[0] = 0;
  for (int br = 0; br < nb; ++br)
    bsrRow[br + 1] = bsrRow[br] + block_row_cols(br, bs, csrRow, csrCol, &buf, &cap);
  free(buf);
  return ORC_OK;
}

int orc_csr_to_bsr_fill(int n, int bs, const int* csrRow, const int* csrCol,
                        const double* csrVal, const int* bsrRow, int* bsrCol,
                        double* bsrVal) {
  if (bs < 1 || bs > MAXBS || n < 0 || n % bs) return ORC_ERR_ARG;
  int nb = n / bs, bs2 = bs * bs;
  int* buf = NULL;
  int cap = 0;
  for (int br = 0; br < nb; ++br) {
    int u = block_row_cols(br, bs, csrRow, csrCol, &buf, &cap);
    int base = bsrRow[br];
    if (bsrRow[br + 1] - base != u) { free(buf); return ORC_ERR_PATTERN; }
    memcpy(bsrCol + base, buf, sizeof(int) * (size_t)u);
    char* created = (char*)calloc((size_t)(u > 0 ? u : 1), 1);
    for (int lr = 0; lr < bs; ++lr) {
      int row = br * bs + lr;
      for (int p = csrRow[row]; p < csrRow[row + 1]; ++p) {
        int gc = csrCol[p], bc = gc / bs, lc = gc % bs;
        int* hit = (int*)bsearch(&bc, bsrCol + base, (size_t)u, sizeof(int), cmp_int);
        int k = (int)(hit - (bsrCol + base));
        double* blk = bsrVal + (size_t)(base + k) * bs2;
        if (!created[k]) {
          for (int e = 0; e < bs2; ++e) blk[e] = 0.0;
          blk[lr * bs + lc] = csrVal[p];
          created[k] = 1;
        } else {
          blk[lr * bs + lc] += csrVal[p];
        }
      }
    }
    free(created);
  }
  free(buf);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* isai_bsr.h:246-284: column j of M_L = {j} U {r >= j : A(r,j) != 0};
 * column j of M_U = {j} U {r <= j : A(r,j) != 0}; sorted, unique. */
int orc_isai_pattern_count(int nb, const int* Arow, const int* Acol, int lower,
                           int* Mptr) {
  int* cnt = (int*)calloc((size_t)nb + 1, sizeof(int));
  for (int br = 0; br < nb; ++br)
    for (int p = Arow[br]; p < Arow[br + 1]; ++p) {
      int bc = Acol[p];
      if (bc < 0 || bc >= nb) { free(cnt); return ORC_ERR_PATTERN; }
      if (bc == br) continue; /* diagonal counted once below */
      if (lower ? (bc > br) : (bc < br)) continue;
      cnt[bc]++;
    }
  Mptr[0] = 0;
  for (int j = 0; j < nb; ++j) Mptr[j + 1] = Mptr[j] + cnt[j] + 1;
  free(cnt);
  return ORC_OK;
}

int orc_isai_pattern_fill(int nb, const int* Arow, const int* Acol, int lower,
                          const int* Mptr, int* Mind) {
  int* pos = (int*)malloc(sizeof(int) * (size_t)(nb > 0 ? nb : 1));
  for (int j = 0; j < nb; ++j) pos[j] = Mptr[j];
  /* Rows are visited in ascending order and the diagonal is appended when
   * row j is reached: a lower column only receives rows >= j and an upper
   * column only rows <= j, so both come out ascending without a sort. */
  for (int br = 0; br < nb; ++br) {
    for (int p = Arow[br]; p < Arow[br + 1]; ++p) {
      int bc = Acol[p];
      if (bc == br) continue;
      if (lower ? (bc > br) : (bc < br)) continue;
      Mind[pos[bc]++] = br;
    }
    Mind[pos[br]++] = br;
  }
  for (int j = 0; j < nb; ++j)
    if (pos[j] != Mptr[j + 1]) { free(pos); return ORC_ERR_PATTERN; }
  free(pos);
  return ORC_OK;
}

/* Symbolic product C = pattern(X A) (ISAI(k) patterns; no counterpart in
 * the reference): row i of C is the sorted union of the rows of A named by
 * row i of X.  Ccol == NULL: counts only (Crow[nb] = nnz). */
int orc_pattern_product(int nb, const int* Xrow, const int* Xcol, const int* Arow,
                        const int* Acol, int* Crow, int* Ccol) {
  int cap = 64;
  int* buf = (int*)malloc(sizeof(int) * (size_t)cap);
  Crow[0] = 0;
  for (int i = 0; i < nb; ++i) {
    int m = 0;
    for (int p = Xrow[i]; p < Xrow[i + 1]; ++p) {
      int c = Xcol[p];
      for (int q = Arow[c]; q < Arow[c + 1]; ++q) {
        if (m == cap) {
          cap *= 2;
          buf = (int*)realloc(buf, sizeof(int) * (size_t)cap);
        }
        buf[m++] = Acol[q];
      }
    }
    qsort(buf, (size_t)m, sizeof(int), cmp_int);
    int u = 0;
    for (int t = 0; t < m; ++t)
      if (t == 0 || buf[t] != buf[t - 1]) {
        if (Ccol) Ccol[Crow[i] + u] = buf[t];
        ++u;
      }
    Crow[i + 1] = Crow[i] + u;
  }
  free(buf);
  return ORC_OK;
}

/* bcsc2bcsr.h:11-30 */
int orc_tri_pattern_count(int nb, const int* Arow, const int* Acol, int lower,
                          int* Trow) {
  Trow[0] = 0;
  for (int r = 0; r < nb; ++r) {
    int c = 0;
    for (int p = Arow[r]; p < Arow[r + 1]; ++p)
      if (lower ? (Acol[p] <= r) : (Acol[p] >= r)) ++c;
    Trow[r + 1] = Trow[r] + c;
  }
  return ORC_OK;
}

int orc_tri_pattern_fill(int nb, const int* Arow, const int* Acol, int lower,
                         const int* Trow, int* Tcol) {
  for (int r = 0; r < nb; ++r) {
    int o = Trow[r];
    for (int p = Arow[r]; p < Arow[r + 1]; ++p)
      if (lower ? (Acol[p] <= r) : (Acol[p] >= r)) Tcol[o++] = Acol[p];
  }
  return ORC_OK;
}

/* bcsc2bcsr.h:32-60: linear search of each BCSC entry in its BCSR row */
int orc_map_bcsc2bcsr(int nb, const int* cscPtr, const int* cscInd,
                      const int* csrRow, const int* csrCol, int* map,
                      int* bad_row, int* bad_col) {
  for (int c = 0; c < nb; ++c)
    for (int k = cscPtr[c]; k < cscPtr[c + 1]; ++k) {
      int r = cscInd[k], found = -1;
      for (int p = csrRow[r]; p < csrRow[r + 1]; ++p)
        if (csrCol[p] == c) { found = p; break; }
      if (found < 0) {
        if (bad_row) *bad_row = r;
        if (bad_col) *bad_col = c;
        return ORC_ERR_PATTERN;
      }
      map[k] = found;
    }
  return ORC_OK;
}

/* bcsc2bcsr.h:63-80 */
int orc_reorder_bcsc_to_bcsr(int nnzb, int bs, const int* map,
                             const double* src, double* dst) {
  int bs2 = bs * bs;
  for (int k = 0; k < nnzb; ++k)
    memcpy(dst + (size_t)map[k] * bs2, src + (size_t)k * bs2, sizeof(double) * bs2);
  return ORC_OK;
}

/* bcsc2bcsrAndSpMV.h:76-117, restated deterministically: rows keep the
 * column-ascending order in which the BCSC columns are visited. */
int orc_bcsc_to_bcsr(int mb, int nbcol, int bs, const int* cscPtr,
                     const int* cscInd, const double* cscVal, int* rowPtr,
                     int* colInd, double* val) {
  int bs2 = bs * bs;
  int nnzb = cscPtr[nbcol];
  for (int i = 0; i <= mb; ++i) rowPtr[i] = 0;
  for (int k = 0; k < nnzb; ++k) {
    if (cscInd[k] < 0 || cscInd[k] >= mb) return ORC_ERR_PATTERN;
    rowPtr[cscInd[k] + 1]++;
  }
  for (int i = 0; i < mb; ++i) rowPtr[i + 1] += rowPtr[i];
  int* next = (int*)malloc(sizeof(int) * (size_t)(mb > 0 ? mb : 1));
  for (int i = 0; i < mb; ++i) next[i] = rowPtr[i];
  for (int c = 0; c < nbcol; ++c)
    for (int k = cscPtr[c]; k < cscPtr[c + 1]; ++k) {
      int d = next[cscInd[k]]++;
      colInd[d] = c;
      if (cscVal && val)
        memcpy(val + (size_t)d * bs2, cscVal + (size_t)k * bs2, sizeof(double) * bs2);
    }
  free(next);
  return ORC_OK;
}

/* bsr2csr.h:19-137 (cusparseDbsr2csr, CUSPARSE_DIRECTION_ROW): scalar row
 * br*bs+r lists, block by block, the bs entries of row r of each block. */
int orc_bsr_to_csr(int mb, int bs, const int* Arow, const int* Acol,
                   const double* Aval, int* csrRow, int* csrCol,
                   double* csrVal) {
  int bs2 = bs * bs;
  csrRow[0] = 0;
  for (int br = 0; br < mb; ++br) {
    int len = (Arow[br + 1] - Arow[br]) * bs;
    for (int r = 0; r < bs; ++r) {
      int row = br * bs + r;
      int o = csrRow[row];
      csrRow[row + 1] = o + len;
      for (int p = Arow[br]; p < Arow[br + 1]; ++p)
        for (int c = 0; c < bs; ++c) {
          csrCol[o] = Acol[p] * bs + c;
          csrVal[o] = Aval[(size_t)p * bs2 + r * bs + c];
          ++o;
        }
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* binary search of block column bc in block row br (isai_bsr.h:33-57) */
static int find_block(const int* row, const int* col, int br, int bc) {
  int s = row[br], e = row[br + 1] - 1;
  while (s <= e) {
    int m = (s + e) >> 1;
    int c = col[m];
    if (c == bc) return m;
    if (c < bc) s = m + 1; else e = m - 1;
  }
  return -1;
}

/* bsrilu.h:20-66.  cuSPARSE bsrilu02 computes, in place, the incomplete LU
 * factorisation whose scalar form is ILU(0) on the block-dense pattern:
 * a_ik /= a_kk for k < i, then a_ij -= a_ik*a_kj for j > k in the pattern
 * (IKJ order).  Restated blockwise, keeping the scalar operation order. */
int orc_bsrilu0(int nb, int bs, const int* Arow, const int* Acol, double* Aval,
                int* zero_pivot) {
  int bs2 = bs * bs;
  int first_zero = -1;
  int* diag = (int*)malloc(sizeof(int) * (size_t)(nb > 0 ? nb : 1));
  for (int i = 0; i < nb; ++i) {
    diag[i] = find_block(Arow, Acol, i, i);
    if (diag[i] < 0) {
      if (zero_pivot) *zero_pivot = i;
      free(diag);
      return ORC_ERR_PATTERN;
    }
  }
  for (int I = 0; I < nb; ++I) {
    int rs = Arow[I], re = Arow[I + 1];
    for (int pk = rs; pk < re && Acol[pk] < I; ++pk) {
      int K = Acol[pk];
      double* L = Aval + (size_t)pk * bs2;
      const double* Ukk = Aval + (size_t)diag[K] * bs2;
      for (int k = 0; k < bs; ++k) {
        for (int r = 0; r < bs; ++r) {
          L[r * bs + k] = L[r * bs + k] / Ukk[k * bs + k];
          double l = L[r * bs + k];
          for (int c = k + 1; c < bs; ++c) L[r * bs + c] -= l * Ukk[k * bs + c];
        }
        /* rows of U_KJ for every J > K present in both row I and row K */
        int qk = diag[K] + 1, qe = Arow[K + 1];
        for (int pj = pk + 1; pj < re; ++pj) {
          int J = Acol[pj];
          while (qk < qe && Acol[qk] < J) ++qk;
          if (qk >= qe) break;
          if (Acol[qk] != J) continue;
          double* Aij = Aval + (size_t)pj * bs2;
          const double* Ukj = Aval + (size_t)qk * bs2;
          for (int r = 0; r < bs; ++r) {
            double l = L[r * bs + k];
            for (int c = 0; c < bs; ++c) Aij[r * bs + c] -= l * Ukj[k * bs + c];
          }
        }
      }
    }
    /* diagonal block and the U blocks to its right, scalar row by row */
    double* D = Aval + (size_t)diag[I] * bs2;
    for (int r = 0; r < bs; ++r) {
      for (int k = 0; k < r; ++k) {
        D[r * bs + k] = D[r * bs + k] / D[k * bs + k];
        double l = D[r * bs + k];
        for (int c = k + 1; c < bs; ++c) D[r * bs + c] -= l * D[k * bs + c];
        for (int pj = diag[I] + 1; pj < re; ++pj) {
          double* U = Aval + (size_t)pj * bs2;
          for (int c = 0; c < bs; ++c) U[r * bs + c] -= l * U[k * bs + c];
        }
      }
      if (D[r * bs + r] == 0.0 && first_zero < 0) first_zero = I;
    }
  }
  free(diag);
  if (zero_pivot) *zero_pivot = first_zero;
  return first_zero >= 0 ? ORC_ERR_ZERO_PIVOT : ORC_OK;
}

/* scalar ILU(0), IKJ variant, on a CSR matrix with sorted columns */
int orc_csr_ilu0(int n, const int* row, const int* col, double* val,
                 int* zero_pivot) {
  int first_zero = -1;
  int* dpos = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    dpos[i] = -1;
    for (int p = row[i]; p < row[i + 1]; ++p)
      if (col[p] == i) dpos[i] = p;
    if (dpos[i] < 0) { free(dpos); if (zero_pivot) *zero_pivot = i; return ORC_ERR_PATTERN; }
  }
  for (int i = 0; i < n; ++i) {
    for (int pk = row[i]; pk < row[i + 1] && col[pk] < i; ++pk) {
      int k = col[pk];
      val[pk] = val[pk] / val[dpos[k]];
      double l = val[pk];
      int q = dpos[k] + 1;
      for (int pj = pk + 1; pj < row[i + 1]; ++pj) {
        int j = col[pj];
        while (q < row[k + 1] && col[q] < j) ++q;
        if (q >= row[k + 1]) break;
        if (col[q] == j) val[pj] -= l * val[q];
      }
    }
    if (val[dpos[i]] == 0.0 && first_zero < 0) first_zero = i;
  }
  free(dpos);
  if (zero_pivot) *zero_pivot = first_zero;
  return first_zero >= 0 ? ORC_ERR_ZERO_PIVOT : ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* isai_bsr.h:61-88: Gauss-Jordan without pivoting, eps 1e-14 */
static int invert_dense(int bs, const double* A, double* Ainv) {
  double M[MAXBS * MAXBS], I[MAXBS * MAXBS];
  int bs2 = bs * bs;
  for (int i = 0; i < bs2; ++i) { M[i] = A[i]; I[i] = 0.0; }
  for (int d = 0; d < bs; ++d) I[d * bs + d] = 1.0;
  for (int k = 0; k < bs; ++k) {
    double piv = M[k * bs + k];
    if (fabs(piv) < 1e-14) return 0;
    double invp = 1.0 / piv;
    for (int j = 0; j < bs; ++j) { M[k * bs + j] *= invp; I[k * bs + j] *= invp; }
    for (int i = 0; i < bs; ++i) {
      if (i == k) continue;
      double f = M[i * bs + k];
      for (int j = 0; j < bs; ++j) {
        M[i * bs + j] -= f * M[k * bs + j];
        I[i * bs + j] -= f * I[k * bs + j];
      }
    }
  }
  for (int i = 0; i < bs2; ++i) Ainv[i] = I[i];
  return 1;
}

/* isai_bsr.h:91-158: inverse of the unit-lower (lower=1) or upper (lower=0)
 * part of each diagonal block; a missing block reads as zero; a failed
 * inversion retries once with 1e-12 added to the diagonal. */
int orc_dinv(int nb, int bs, const int* Arow, const int* Acol,
             const double* Aval, int lower, double* Dinv) {
  int bs2 = bs * bs;
  int status = ORC_OK;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nb; ++k) {
    double B[MAXBS * MAXBS];
    int pos = find_block(Arow, Acol, k, k);
    for (int e = 0; e < bs2; ++e) B[e] = pos >= 0 ? Aval[(size_t)pos * bs2 + e] : 0.0;
    for (int i = 0; i < bs; ++i) {
      for (int j = 0; j < bs; ++j)
        if (lower ? (j > i) : (j < i)) B[i * bs + j] = 0.0;
      if (lower) B[i * bs + i] = 1.0;
    }
    if (!invert_dense(bs, B, Dinv + (size_t)k * bs2)) {
      for (int d = 0; d < bs; ++d) B[d * bs + d] += 1e-12;
      if (!invert_dense(bs, B, Dinv + (size_t)k * bs2)) {
#pragma omp critical
        status = ORC_ERR_ZERO_PIVOT;
      }
    }
  }
  return status;
}

/* ------------------------------------------------------------------------ */
/* isai_bsr.h:1378-1424: sorted merge of A row t with S_j, counting matches
 * whose local position is < idx. */
int orc_count_pairs_lower(int nb, const int* Arow, const int* Acol,
                          const int* Mptr, const int* Mind, int* counts) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < nb; ++j) {
    int start = Mptr[j], end = Mptr[j + 1];
    for (int idx = 0; idx < end - start; ++idx) {
      int t = Mind[start + idx];
      int iA = Arow[t], a1 = Arow[t + 1], iS = start, cnt = 0;
      while (iA < a1 && iS < end) {
        int cA = Acol[iA], cS = Mind[iS];
        if (cA == cS) { if (iS - start < idx) ++cnt; ++iA; ++iS; }
        else if (cA < cS) ++iA;
        else ++iS;
      }
      counts[start + idx] = cnt;
    }
  }
  return ORC_OK;
}

/* isai_bsr.h:1427-1476 */
int orc_fill_pairs_lower(int nb, const int* Arow, const int* Acol,
                         const int* Mptr, const int* Mind, const int* PairPtr,
                         int* PairPLocal, int* PairSrc) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < nb; ++j) {
    int start = Mptr[j], end = Mptr[j + 1];
    for (int idx = 0; idx < end - start; ++idx) {
      int t = Mind[start + idx];
      int iA = Arow[t], a1 = Arow[t + 1], iS = start;
      int out = PairPtr[start + idx];
      while (iA < a1 && iS < end) {
        int cA = Acol[iA], cS = Mind[iS];
        if (cA == cS) {
          int pl = iS - start;
          if (pl < idx) { PairPLocal[out] = pl; PairSrc[out] = iA; ++out; }
          ++iA; ++iS;
        } else if (cA < cS) ++iA;
        else ++iS;
      }
    }
  }
  return ORC_OK;
}

/* C = A*B summed over k for each element (the scalar kernels' order) */
static void blk_mul(int bs, const double* A, const double* B, double* C) {
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < bs; ++c) {
      double s = 0.0;
      for (int k = 0; k < bs; ++k) s += A[r * bs + k] * B[k * bs + c];
      C[r * bs + c] = s;
    }
}

/* isai_bsr.h:288-399: column j of M_L by forward substitution over S_j:
 * rhs = delta_{t,j} I; rhs -= A(t,p) Y_p for each pair; Y = DinvL[t] rhs. */
int orc_isai_lower(int nb, int bs, const double* Aval, const int* Mptr,
                   const int* Mind, const int* PairPtr, const int* PairPLocal,
                   const int* PairSrc, const double* DinvL, double* Mval) {
  int bs2 = bs * bs;
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < nb; ++j) {
    double rhs[MAXBS * MAXBS], prod[MAXBS * MAXBS];
    int start = Mptr[j], N = Mptr[j + 1] - start;
    for (int idx = 0; idx < N; ++idx) {
      int t = Mind[start + idx];
      for (int e = 0; e < bs2; ++e)
        rhs[e] = (t == j && e / bs == e % bs) ? 1.0 : 0.0;
      for (int q = PairPtr[start + idx]; q < PairPtr[start + idx + 1]; ++q) {
        blk_mul(bs, Aval + (size_t)PairSrc[q] * bs2,
                Mval + (size_t)(start + PairPLocal[q]) * bs2, prod);
        for (int e = 0; e < bs2; ++e) rhs[e] -= prod[e];
      }
      blk_mul(bs, DinvL + (size_t)t * bs2, rhs, Mval + (size_t)(start + idx) * bs2);
    }
  }
  return ORC_OK;
}

/* isai_bsr.h:161-242: column j of M_U by backward substitution over S_j;
 * U(t, S_j[p]) for p > idx is looked up in A row t (missing -> zero). */
int orc_isai_upper(int nb, int bs, const int* Arow, const int* Acol,
                   const double* Aval, const int* Mptr, const int* Mind,
                   const double* DinvU, double* Mval) {
  int bs2 = bs * bs;
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < nb; ++j) {
    double rhs[MAXBS * MAXBS], prod[MAXBS * MAXBS];
    int start = Mptr[j], N = Mptr[j + 1] - start;
    for (int idx = N - 1; idx >= 0; --idx) {
      int t = Mind[start + idx];
      for (int e = 0; e < bs2; ++e)
        rhs[e] = (t == j && e / bs == e % bs) ? 1.0 : 0.0;
      for (int p = N - 1; p > idx; --p) {
        int pos = find_block(Arow, Acol, t, Mind[start + p]);
        if (pos < 0) continue; /* a zero block changes nothing */
        blk_mul(bs, Aval + (size_t)pos * bs2, Mval + (size_t)(start + p) * bs2, prod);
        for (int e = 0; e < bs2; ++e) rhs[e] -= prod[e];
      }
      blk_mul(bs, DinvU + (size_t)t * bs2, rhs, Mval + (size_t)(start + idx) * bs2);
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* bcsc2bcsrAndSpMV.h:119-138 */
int orc_bcsr_spmv(int mb, int bs, const int* row, const int* col,
                  const double* val, const double* x, double* y) {
  int bs2 = bs * bs;
#pragma omp parallel for schedule(static, 1024)
  for (int br = 0; br < mb; ++br)
    for (int r = 0; r < bs; ++r) {
      double sum = 0.0;
      for (int idx = row[br]; idx < row[br + 1]; ++idx) {
        const double* blk = val + (size_t)idx * bs2;
        int bc = col[idx];
        for (int c = 0; c < bs; ++c) sum += blk[r * bs + c] * x[(size_t)bc * bs + c];
      }
      y[(size_t)br * bs + r] = sum;
    }
  return ORC_OK;
}

int orc_bcsr_spmv_f32(int mb, int bs, const int* row, const int* col,
                      const float* val, const float* x, float* y) {
  int bs2 = bs * bs;
#pragma omp parallel for schedule(static, 1024)
  for (int br = 0; br < mb; ++br)
    for (int r = 0; r < bs; ++r) {
      float sum = 0.0f;
      for (int idx = row[br]; idx < row[br + 1]; ++idx) {
        const float* blk = val + (size_t)idx * bs2;
        int bc = col[idx];
        for (int c = 0; c < bs; ++c) sum += blk[r * bs + c] * x[(size_t)bc * bs + c];
      }
      y[(size_t)br * bs + r] = sum;
    }
  return ORC_OK;
}

/* cape_sptrsv.h:8-53 semantics (unit lower, no divide), blockwise on the
 * packed BILU(0): strictly-lower blocks + strict lower part of the diagonal
 * block. */
int orc_sptrsv_lower(int nb, int bs, const int* row, const int* col,
                     const double* val, const double* b, double* x) {
  int bs2 = bs * bs;
  for (int I = 0; I < nb; ++I) {
    int d = -1;
    for (int r = 0; r < bs; ++r) {
      double s = b[(size_t)I * bs + r];
      for (int p = row[I]; p < row[I + 1]; ++p) {
        int K = col[p];
        if (K > I) break;
        if (K == I) { d = p; break; }
        const double* L = val + (size_t)p * bs2;
        for (int c = 0; c < bs; ++c) s -= L[r * bs + c] * x[(size_t)K * bs + c];
      }
      if (d < 0) return ORC_ERR_PATTERN;
      const double* D = val + (size_t)d * bs2;
      for (int c = 0; c < r; ++c) s -= D[r * bs + c] * x[(size_t)I * bs + c];
      x[(size_t)I * bs + r] = s;
    }
  }
  return ORC_OK;
}

/* cape_sptrsv.h:55-103 semantics (upper, divide by the diagonal) */
int orc_sptrsv_upper(int nb, int bs, const int* row, const int* col,
                     const double* val, const double* b, double* x) {
  int bs2 = bs * bs;
  for (int I = nb - 1; I >= 0; --I) {
    int d = find_block(row, col, I, I);
    if (d < 0) return ORC_ERR_PATTERN;
    const double* D = val + (size_t)d * bs2;
    for (int r = bs - 1; r >= 0; --r) {
      double s = b[(size_t)I * bs + r];
      for (int p = row[I + 1] - 1; p > d; --p) {
        const double* U = val + (size_t)p * bs2;
        int J = col[p];
        for (int c = 0; c < bs; ++c) s -= U[r * bs + c] * x[(size_t)J * bs + c];
      }
      for (int c = bs - 1; c > r; --c) s -= D[r * bs + c] * x[(size_t)I * bs + c];
      x[(size_t)I * bs + r] = s / D[r * bs + r];
    }
  }
  return ORC_OK;
}

/* residual_check.h:16-71 */
int orc_rel_errors_csr(int n, const int* row, const int* col, const double* val,
                       const double* b, const double* x_true, const double* x,
                       double* rel_err, double* rel_res) {
  if (x_true && rel_err) {
    double nd = 0.0, nt = 0.0;
    for (int i = 0; i < n; ++i) {
      double d = x[i] - x_true[i];
      nd += d * d;
      nt += x_true[i] * x_true[i];
    }
    nd = sqrt(nd);
    nt = sqrt(nt);
    *rel_err = nt > 0.0 ? nd / nt : 0.0;
  }
  double nr = 0.0, nbn = 0.0;
  for (int i = 0; i < n; ++i) {
    double ax = 0.0;
    for (int p = row[i]; p < row[i + 1]; ++p) ax += val[p] * x[col[p]];
    double r = b[i] - ax;
    nr += r * r;
    nbn += b[i] * b[i];
  }
  nr = sqrt(nr);
  nbn = sqrt(nbn);
  if (rel_res) *rel_res = nbn > 0.0 ? nr / nbn : INFINITY;
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Krylov helpers: chunked, thread-count-independent reductions */
static double dot_chunked(size_t n, const double* a, const double* b) {
  size_t nch = (n + CHUNK - 1) / CHUNK;
  double* part = (double*)malloc(sizeof(double) * (nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nch; ++c) {
    size_t lo = (size_t)c * CHUNK, hi = lo + CHUNK < n ? lo + CHUNK : n;
    double s = 0.0;
    for (size_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0.0;
  for (size_t c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}

typedef struct {
  int nb, bs;
  const int *Lrow, *Lcol, *Urow, *Ucol;
  const double *Lval, *Uval;
  float *Lval32, *Uval32, *v32, *y32, *z32;
  double* y;
} isai_apply_t;

static void isai_apply(const isai_apply_t* P, int precond, const double* v,
                       double* z, size_t n) {
  if (precond == 0) {
    memcpy(z, v, sizeof(double) * n);
  } else if (precond == 3) {
    /* exact BILU(0): L (Lrow/Lcol/Lval = packed factor) unit-lower solve,
     * then the upper solve on the same packed factor */
    orc_sptrsv_lower(P->nb, P->bs, P->Lrow, P->Lcol, P->Lval, v, P->y);
    orc_sptrsv_upper(P->nb, P->bs, P->Lrow, P->Lcol, P->Lval, P->y, z);
  } else if (precond == 1) {
    orc_bcsr_spmv(P->nb, P->bs, P->Lrow, P->Lcol, P->Lval, v, P->y);
    orc_bcsr_spmv(P->nb, P->bs, P->Urow, P->Ucol, P->Uval, P->y, z);
  } else {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) P->v32[i] = (float)v[i];
    orc_bcsr_spmv_f32(P->nb, P->bs, P->Lrow, P->Lcol, P->Lval32, P->v32, P->y32);
    orc_bcsr_spmv_f32(P->nb, P->bs, P->Urow, P->Ucol, P->Uval32, P->y32, P->z32);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) z[i] = (double)P->z32[i];
  }
}

/* One modified Gram-Schmidt sweep over w, chunk by chunk: w -= hp * vp
 * (when vp is given), then the chunked dot product vn . w (w . w when vn is
 * NULL).  Inside a chunk every element of w is updated before it enters the
 * dot product, so the result equals the separate update pass followed by
 * dot_chunked, bit for bit, with one pass over the vectors instead of two. */
static double sweep_chunked(size_t n, const double* vp, double hp, const double* vn,
                            double* w) {
  size_t nch = (n + CHUNK - 1) / CHUNK;
  double* part = (double*)malloc(sizeof(double) * (nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nch; ++c) {
    size_t lo = (size_t)c * CHUNK, hi = lo + CHUNK < n ? lo + CHUNK : n;
    if (vp)
      for (size_t i = lo; i < hi; ++i) w[i] -= hp * vp[i];
    const double* o = vn ? vn : w;
    double s = 0.0;
    for (size_t i = lo; i < hi; ++i) s += o[i] * w[i];
    part[c] = s;
  }
  double s = 0.0;
  for (size_t c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}

/* The same in FP32: float products and float sums inside each chunk, the
 * chunk sums added in double in chunk order (thread-count independent). */
static double sweep_chunked_f32(size_t n, const float* vp, float hp, const float* vn,
                                float* w) {
  size_t nch = (n + CHUNK - 1) / CHUNK;
  double* part = (double*)malloc(sizeof(double) * (nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nch; ++c) {
    size_t lo = (size_t)c * CHUNK, hi = lo + CHUNK < n ? lo + CHUNK : n;
    if (vp)
      for (size_t i = lo; i < hi; ++i) w[i] -= hp * vp[i];
    const float* o = vn ? vn : w;
    float s = 0.0f;
    for (size_t i = lo; i < hi; ++i) s += o[i] * w[i];
    part[c] = (double)s;
  }
  double s = 0.0;
  for (size_t c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}

/* Inner solve of the nested (GMRES-IR) mode: k steps of right-preconditioned
 * GMRES in FP32 on A s = v, from s = 0, with the FP32-stored A and the
 * FP32-stored ISAI (M = M_U M_L), modified Gram-Schmidt in FP32 (fused
 * sweeps, sweep_chunked_f32), the Hessenberg least-squares problem in
 * double.  v has unit norm (the outer basis vector), so the start vector is
 * v rounded to FP32 with beta = 1: FGMRES accepts any scaling of its
 * preconditioned vectors.  The preconditioned vectors q_i = M u_i are kept,
 * and z = sum_i y_i q_i (FP32 accumulation, i ascending) widened to FP64.
 * A zero subdiagonal entry (an invariant subspace) ends the steps early.
 * Returns the number of steps taken. */
typedef struct {
  int nb, bs, k;
  const int *Arow, *Acol, *Lrow, *Lcol, *Urow, *Ucol;
  const float *A32, *L32, *U32;
  float *Ub, *Qb, *w, *t;    /* (k+1) n, k n, n, n */
  double *H, *cs, *sn, *g, *y;  /* (k+1) k, k, k, k+1, k */
} inner_t;

static int inner_gmres_f32(const inner_t* I, const double* v, double* z) {
  const size_t n = (size_t)I->nb * I->bs;
  const int k = I->k;
  float* u0 = I->Ub;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < (long)n; ++e) u0[e] = (float)v[e];
  for (int i = 0; i <= k; ++i) I->g[i] = 0.0;
  I->g[0] = 1.0;
  int steps = 0;
  for (int j = 0; j < k; ++j) {
    float* uj = I->Ub + n * (size_t)j;
    float* qj = I->Qb + n * (size_t)j;
    orc_bcsr_spmv_f32(I->nb, I->bs, I->Lrow, I->Lcol, I->L32, uj, I->t);
    orc_bcsr_spmv_f32(I->nb, I->bs, I->Urow, I->Ucol, I->U32, I->t, qj);
    orc_bcsr_spmv_f32(I->nb, I->bs, I->Arow, I->Acol, I->A32, qj, I->w);
    /* fused sweeps: sweep i applies h_{i-1} u_{i-1} and takes u_i . w */
    for (int i = 0; i <= j; ++i) {
      const float* up = i > 0 ? I->Ub + n * (size_t)(i - 1) : NULL;
      const float hp = i > 0 ? (float)I->H[(i - 1) * k + j] : 0.0f;
      I->H[i * k + j] = sweep_chunked_f32(n, up, hp, I->Ub + n * (size_t)i, I->w);
    }
    double hn = sqrt(sweep_chunked_f32(n, I->Ub + n * (size_t)j, (float)I->H[j * k + j], NULL,
                                       I->w));
    I->H[(j + 1) * k + j] = hn;
    if (hn != 0.0) {
      float inv = (float)(1.0 / hn);
      float* un = I->Ub + n * (size_t)(j + 1);
#pragma omp parallel for schedule(static)
      for (long e = 0; e < (long)n; ++e) un[e] = I->w[e] * inv;
    }
    for (int i = 0; i < j; ++i) {
      double a = I->H[i * k + j], c = I->H[(i + 1) * k + j];
      I->H[i * k + j] = I->cs[i] * a + I->sn[i] * c;
      I->H[(i + 1) * k + j] = -I->sn[i] * a + I->cs[i] * c;
    }
    double a = I->H[j * k + j], c = I->H[(j + 1) * k + j];
    double den = sqrt(a * a + c * c);
    I->cs[j] = den != 0.0 ? a / den : 1.0;
    I->sn[j] = den != 0.0 ? c / den : 0.0;
    I->H[j * k + j] = I->cs[j] * a + I->sn[j] * c;
    I->H[(j + 1) * k + j] = 0.0;
    I->g[j + 1] = -I->sn[j] * I->g[j];
    I->g[j] = I->cs[j] * I->g[j];
    steps = j + 1;
    if (hn == 0.0) break;
  }
  for (int i = steps - 1; i >= 0; --i) {
    double s = I->g[i];
    for (int l = i + 1; l < steps; ++l) s -= I->H[i * k + l] * I->y[l];
    I->y[i] = I->H[i * k + i] != 0.0 ? s / I->H[i * k + i] : 0.0;
  }
#pragma omp parallel for schedule(static)
  for (long e = 0; e < (long)n; ++e) {
    float s = 0.0f;
    for (int i = 0; i < steps; ++i) s += (float)I->y[i] * I->Qb[n * (size_t)i + e];
    z[e] = (double)s;
  }
  return steps;
}

/* Restarted right-preconditioned (F)GMRES(m):
 *   r0 = b - A x0 (x0 = 0), beta = ||r0||; V_0 = r0 * (1/beta); g = beta e_1
 *   for j: z_j = M v_j; w = A z_j;
 *          modified Gram-Schmidt: for i = 0..j: h_i = v_i . w, w -= h_i v_i;
 *          h(j+1,j) = ||w||; v_{j+1} = w * (1/h(j+1,j)); Givens rotations;
 *          stop the cycle when |g_{j+1}| <= tol*||b|| or the budget is used
 *   x += Z y (upper-triangular solve of H y = g); true residual at restart.
 * The iteration count is the number of inner (Arnoldi) steps. */
int orc_gmres(int nb, int bs, const int* Arow, const int* Acol,
              const double* Aval, const int* Lrow, const int* Lcol,
              const double* Lval, const int* Urow, const int* Ucol,
              const double* Uval, int precond, const double* b, double* x,
              int restart, double tol, int maxit, int* iters, double* relres,
              double* hist) {
  return orc_gmres_ex(nb, bs, Arow, Acol, Aval, Lrow, Lcol, Lval, Urow, Ucol, Uval, precond, 0,
                      b, x, restart, tol, maxit, iters, NULL, relres, hist);
}

int orc_gmres_ex(int nb, int bs, const int* Arow, const int* Acol,
                 const double* Aval, const int* Lrow, const int* Lcol,
                 const double* Lval, const int* Urow, const int* Ucol,
                 const double* Uval, int precond, int inner_k, const double* b,
                 double* x, int restart, double tol, int maxit, int* iters,
                 long long* inner_total, double* relres, double* hist) {
  size_t n = (size_t)nb * bs;
  int m = restart;
  if (m < 1 || nb < 1) return ORC_ERR_ARG;
  if (precond == 5 && inner_k < 1) return ORC_ERR_ARG;
  long long inner_sum = 0;
  double* V = (double*)malloc(sizeof(double) * n * (size_t)(m + 1));
  double* Z = (double*)malloc(sizeof(double) * n * (size_t)m);
  double* w = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double*)calloc((size_t)m, sizeof(double)), *sn = (double*)calloc((size_t)m, sizeof(double));
  double *g = (double*)calloc((size_t)m + 1, sizeof(double)), *yv = (double*)calloc((size_t)m, sizeof(double));
  double* hcol = (double*)calloc((size_t)m + 1, sizeof(double));
  isai_apply_t P = {nb, bs, Lrow, Lcol, Urow, Ucol, Lval, Uval, NULL, NULL, NULL, NULL, NULL, NULL};
  float* A32 = NULL;
  if (precond >= 1) P.y = (double*)malloc(sizeof(double) * n);
  if (precond == 4 || precond == 5) {
    size_t na = (size_t)Arow[nb] * bs * bs;
    A32 = (float*)malloc(sizeof(float) * na);
    for (size_t i = 0; i < na; ++i) A32[i] = (float)Aval[i];
  }
  if (precond == 2 || precond == 4 || precond == 5) {
    int nL = Lrow[nb], nU = Urow[nb];
    size_t bs2 = (size_t)bs * bs;
    P.Lval32 = (float*)malloc(sizeof(float) * nL * bs2);
    P.Uval32 = (float*)malloc(sizeof(float) * nU * bs2);
    for (size_t i = 0; i < (size_t)nL * bs2; ++i) P.Lval32[i] = (float)Lval[i];
    for (size_t i = 0; i < (size_t)nU * bs2; ++i) P.Uval32[i] = (float)Uval[i];
    P.v32 = (float*)malloc(sizeof(float) * n);
    P.y32 = (float*)malloc(sizeof(float) * n);
    P.z32 = (float*)malloc(sizeof(float) * n);
  }
  inner_t I;
  memset(&I, 0, sizeof(I));
  if (precond == 5) {
    int k = inner_k;
    I.nb = nb;
    I.bs = bs;
    I.k = k;
    I.Arow = Arow; I.Acol = Acol; I.Lrow = Lrow; I.Lcol = Lcol; I.Urow = Urow; I.Ucol = Ucol;
    I.A32 = A32; I.L32 = P.Lval32; I.U32 = P.Uval32;
    I.Ub = (float*)malloc(sizeof(float) * n * (size_t)(k + 1));
    I.Qb = (float*)malloc(sizeof(float) * n * (size_t)k);
    I.w = (float*)malloc(sizeof(float) * n);
    I.t = (float*)malloc(sizeof(float) * n);
    I.H = (double*)calloc((size_t)(k + 1) * k, sizeof(double));
    I.cs = (double*)calloc((size_t)k, sizeof(double));
    I.sn = (double*)calloc((size_t)k, sizeof(double));
    I.g = (double*)calloc((size_t)k + 1, sizeof(double));
    I.y = (double*)calloc((size_t)k, sizeof(double));
  }
  for (size_t i = 0; i < n; ++i) x[i] = 0.0;
  double bnorm = sqrt(dot_chunked(n, b, b));
  if (bnorm == 0.0) bnorm = 1.0;
  memcpy(r, b, sizeof(double) * n);
  double beta = sqrt(dot_chunked(n, r, r));
  int total = 0, status = ORC_ERR_NOT_CONVERGED;
  double res = beta / bnorm;
  if (hist) hist[0] = res;
  if (res <= tol) status = ORC_OK;
  while (status != ORC_OK && total < maxit) {
    double binv = 1.0 / beta;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) V[i] = r[i] * binv;
    for (int i = 0; i <= m; ++i) g[i] = 0.0;
    g[0] = beta;
    int jlast = -1;
    for (int j = 0; j < m && total < maxit; ++j) {
      double* vj = V + n * (size_t)j;
      double* zj = Z + n * (size_t)j;
      if (precond == 5)
        inner_sum += inner_gmres_f32(&I, vj, zj);
      else
        isai_apply(&P, precond == 4 ? 2 : precond, vj, zj, n);
      if (precond == 4) {
        /* FP32-stored A in the Arnoldi product: z rounded to FP32, FP32
         * accumulation, result widened to FP64 */
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) P.v32[i] = (float)zj[i];
        orc_bcsr_spmv_f32(nb, bs, Arow, Acol, A32, P.v32, P.y32);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) w[i] = (double)P.y32[i];
      } else {
        orc_bcsr_spmv(nb, bs, Arow, Acol, Aval, zj, w);
      }
      /* modified Gram-Schmidt */
      /* fused sweeps: sweep i applies h_{i-1} v_{i-1} and takes v_i . w */
      for (int i = 0; i <= j; ++i)
        H[i * m + j] = sweep_chunked(n, i > 0 ? V + n * (size_t)(i - 1) : NULL,
                                     i > 0 ? H[(i - 1) * m + j] : 0.0, V + n * (size_t)i, w);
      double hn = sqrt(sweep_chunked(n, V + n * (size_t)j, H[j * m + j], NULL, w));
      H[(j + 1) * m + j] = hn;
      double* vn = V + n * (size_t)(j + 1);
      if (hn != 0.0) {
        double inv = 1.0 / hn;
#pragma omp parallel for schedule(static)
        for (long e = 0; e < (long)n; ++e) vn[e] = w[e] * inv;
      }
      for (int i = 0; i < j; ++i) {
        double a = H[i * m + j], c = H[(i + 1) * m + j];
        H[i * m + j] = cs[i] * a + sn[i] * c;
        H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
      }
      double a = H[j * m + j], c = H[(j + 1) * m + j];
      double den = sqrt(a * a + c * c);
      cs[j] = den != 0.0 ? a / den : 1.0;
      sn[j] = den != 0.0 ? c / den : 0.0;
      H[j * m + j] = cs[j] * a + sn[j] * c;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++total;
      jlast = j;
      res = fabs(g[j + 1]) / bnorm;
      if (hist) hist[total] = res;
      if (res <= tol || hn == 0.0) break;
    }
    for (int i = jlast; i >= 0; --i) {
      double s = g[i];
      for (int k = i + 1; k <= jlast; ++k) s -= H[i * m + k] * yv[k];
      yv[i] = s / H[i * m + i];
    }
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)n; ++e) {
      double s = x[e];
      for (int i = 0; i <= jlast; ++i) s += yv[i] * Z[n * (size_t)i + e];
      x[e] = s;
    }
    orc_bcsr_spmv(nb, bs, Arow, Acol, Aval, x, w);
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)n; ++e) r[e] = b[e] - w[e];
    beta = sqrt(dot_chunked(n, r, r));
    res = beta / bnorm;
    if (res <= tol) status = ORC_OK;
    if (beta == 0.0) break;
  }
  if (iters) *iters = total;
  if (inner_total) *inner_total = inner_sum;
  if (relres) *relres = res;
  free(V); free(Z); free(w); free(r); free(H); free(cs); free(sn); free(g); free(yv); free(hcol);
  free(P.y); free(P.Lval32); free(P.Uval32); free(P.v32); free(P.y32); free(P.z32);
  free(A32);
  free(I.Ub); free(I.Qb); free(I.w); free(I.t); free(I.H); free(I.cs); free(I.sn); free(I.g);
  free(I.y);
  return status;
}
