// Engine handle: whole-pipeline setup on the GPU and the preconditioned
// (F)GMRES solver.  This is the composition main.cu:449-866 performs by hand
// (patterns, bsrilu02, Dinv, pairs, ISAI-L/U, reorder, one apply), extended
// with the Krylov solver the reference does not have.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "blas1.cuh"
#include "common.cuh"
#include "scan.cuh"

namespace bilu {

thread_local int g_last_cuda_error = 0;
unsigned long long g_launches = 0;

// implemented in the other translation units
size_t isai_pattern_ws(int nb, long long nnzb);
int isai_pattern_colptr_impl(int nb, const int* row, const int* col, int lower, int* Mptr,
                             int* h_nnz, Carver& ws, cudaStream_t st);
int isai_pattern_fill_impl(int nb, const int* row, const int* col, int lower, const int* Mptr,
                           int* Mind, int mnnz, Carver& ws, cudaStream_t st);
int tri_pattern_rowptr_impl(int nb, const int* row, const int* col, int lower, int* Trow,
                            int* h_nnz, Carver& ws, cudaStream_t st);
int tri_pattern_fill_impl(int nb, const int* row, const int* col, int lower, const int* Trow,
                          int* Tcol, cudaStream_t st);
int map_impl(int nb, const int* cptr, const int* cind, const int* rrow, const int* rcol, int* map,
             int* h_bad, Carver& ws, cudaStream_t st);
int reorder_impl(long long nnzb, int bs, const int* map, const double* src, double* dst,
                 cudaStream_t st, float* dst32);
size_t syncfree_ws(int nb);
int diag_positions(int nb, const int* row, const int* col, int* diag, int* h_bad, Carver& ws,
                   cudaStream_t st);
size_t level_sched_ws(int nb, long long nnzb);
size_t bilu0_ws(int nb, long long nnzb);
size_t levels_ws(int nb, long long ndeps);
size_t pattern_product_ws(int n);
int pattern_product_rowptr(int n, const int* Xrow, const int* Xcol, const int* Arow,
                           const int* Acol, int* Crow, int* h_nnz, int* h_bad, Carver& ws,
                           cudaStream_t st);
int pattern_product_fill(int n, const int* Xrow, const int* Xcol, const int* Arow,
                         const int* Acol, const int* Crow, int* Ccol, Carver& ws,
                         cudaStream_t st);
int level_analysis(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                   int lower, int* order, int* lvl, int* nlev_d, int* h_nlev, Carver& ws,
                   cudaStream_t st, int* h_sched, int* h_maxdeg);
int sptrsv_syncfree_async(int nb, int bs, const int* row, const int* col, const int* diag,
                          const int* order, const double* val, int lower, int unit,
                          const double* b, double* x, int* flags, int* ticket, int* err,
                          cudaStream_t st, const double* rdiag);
int sptrsv_flow_f32_async(int nb, int bs, const int* row, const int* col, const int* diag,
                          const int* order, const int* lvl, const int* nlev_d, const float* val,
                          int lower, int unit, const float* b32, float* x32, double* y64,
                          unsigned* words, cudaStream_t st, const float* rdiag32, int maxdeg);
int sptrsv_levels_async(int nb, int bs, const int* row, const int* col, const int* diag,
                        const int* order, const int* lvl, const int* nlev_d, const double* val,
                        int lower, int unit, const double* b, double* x, unsigned* words,
                        cudaStream_t st, const double* rdiag, int maxdeg);
int bilu0_impl(int nb, long long nnzb, int bs, const int* row, const int* col, const int* diag,
               double* val, int* h_zp, Carver& ws, cudaStream_t st, int schedule,
               double* rdiag, LevelOut* keep);
int bilu0_analyze(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                  LevelOut& keep, Carver& ws, cudaStream_t st);
int bilu0_factor(int nb, long long nnzb, int bs, const int* row, const int* col,
                 const int* diag, double* val, int* h_zp, Carver& ws, cudaStream_t st,
                 int schedule, double* rdiag, const LevelOut& keep);
int bilu0_match_count(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                      int* mptr, long long cap, long long* h_total, Carver& ws, cudaStream_t st);
int bilu0_match_fill(int nb, long long nnzb, const int* row, const int* col, const int* diag,
                     const int* mptr, int2* mpair, cudaStream_t st);
int dinv_impl(int nb, int bs, const int* row, const int* col, const double* val, int lower,
              double* Dinv, int* d_fail, cudaStream_t st);
size_t pairs_ws(long long mnnz);
int pairs_ptr_impl(int nb, const int* Arow, const int* Acol, const int* Mptr, const int* Mind,
                   int lower, int* PairPtr, int mnnz, int* h_total, int* h_nmax, Carver& ws,
                   cudaStream_t st);
int pairs_fill_impl(int nb, const int* Arow, const int* Acol, const int* Mptr, const int* Mind,
                    int lower, const int* PairPtr, int mnnz, int* PL, int* PS, cudaStream_t st);
int isai_impl(int nb, int bs, const double* Aval, const int* Mptr, const int* Mind, int lower,
              const int* pp, const int* pl, const int* ps, const double* Dinv, double* Mval,
              cudaStream_t st);
int spmv_any(int mb, int bs, int prec, const int* row, const int* col, const void* val,
             const void* x, int x32, void* y, int y32, cudaStream_t st, int layout);
int spmv_layout_of(int mb, int bs, const int* row, void* d_words, cudaStream_t st,
                   int* h_layout);
int isai_apply_impl(int nb, int bs, int prec, const int* Lrow, const int* Lcol, const void* Lval,
                    const int* Urow, const int* Ucol, const void* Uval, const double* b,
                    void* tmp, double* x, cudaStream_t st, int longL, int longU);
int isai_apply_f32_staged(int nb, int bs, const int* Lrow, const int* Lcol, const float* Lval,
                          const int* Urow, const int* Ucol, const float* Uval, const float* b32,
                          float* tmp, double* x, cudaStream_t st, float* x32, int longL,
                          int longU);

namespace {

}  // namespace

}  // namespace bilu

using namespace bilu;

namespace bilu {
namespace {

// The library's device buffers come from a private stream-ordered memory
// pool per device whose release threshold keeps freed memory reserved:
// the host-buffer entry point creates and destroys a handle (several GB of
// factor, ISAI and Krylov storage at 128^3) per call, and mapping that
// memory anew each time is a visible part of the call.  Other users of the
// default pool in the process are not affected.
cudaMemPool_t lib_pool(int dev) {
  static std::mutex mu;
  static std::vector<cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)pools.size() <= dev) pools.resize(dev + 1, nullptr);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return nullptr;
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = p;
  }
  return pools[dev];
}

// Every buffer from here is freed with cudaFreeAsync, so the fallback when
// no private pool could be made is the device's default stream-ordered pool.
cudaError_t dev_alloc(void** p, size_t bytes, int dev, cudaStream_t st) {
  cudaMemPool_t pool = lib_pool(dev);
  if (!pool) return cudaMallocAsync(p, bytes, st);
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

}  // namespace
}  // namespace bilu

struct bilu_ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  int nb = 0, nnzb = 0, bs = 0;
  long long n = 0;
  int *Arow = nullptr, *Acol = nullptr, *diag = nullptr;
  double *Aval = nullptr, *LU = nullptr;
  double* rdiag = nullptr;  // 1 / pivots of the factor's U_II (nb x bs), written by BILU(0)
  float *LU32 = nullptr, *rdiag32 = nullptr;  // FP32 copies for the mixed exact-ILU apply
  // A, M_L, M_U: SpMV layout words from the setup (bit 0: the pattern has
  // rows of more than 64 blocks, which the CTA then shares; bit 1: more
  // than 5 blocks a row on average)
  int spmv_layout[3] = {0, 0, 0};
  int *Lrow = nullptr, *Lcol = nullptr, *Urow = nullptr, *Ucol = nullptr;
  double *Lval = nullptr, *Uval = nullptr;
  float *Lval32 = nullptr, *Uval32 = nullptr;
  float* Aval32 = nullptr;  // FP32 copy of A for the Arnoldi products (BILU_FP32_INNER)
  int nnzL = 0, nnzU = 0;
  int isai_level = 1;                     // ISAI(k): M patterns from pattern(A^k)
  int schedule = -1;  // BILU(0) and exact-ILU solves: -1 recommended, 0 level, 1 sync-free
  int *Prow = nullptr, *Pcol = nullptr;   // pattern(A^k) when isai_level > 1
  int nnzP = 0;
  bool ready = false;
  // exact BILU(0) apply (BILU_ILU): level analyses of the lower and upper
  // DAGs, and the barrier / error words of the launch-only solves
  int *ordL = nullptr, *lvlL = nullptr, *nlevL = nullptr;
  int *ordU = nullptr, *lvlU = nullptr, *nlevU = nullptr;
  unsigned* ilu_words = nullptr;
  int nlev_host[2] = {0, 0};
  int ilu_sched[2] = {0, 0};    // per triangle: 0 level schedule, 1 sync-free
  int ilu_maxdeg[2] = {0, 0};   // per triangle: largest dependency count
  int* ilu_flags = nullptr;     // ready flags + ticket of the sync-free solves
  // solver buffers
  int m_alloc = 0;
  long long ldv = 0;  // stride of the basis vectors in V and Z (n rounded up to 32)
  double *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr, *tmp = nullptr;
  float* v32 = nullptr;  // FP32 copy of the newest basis vector (mixed apply input)
  float* z32 = nullptr;  // FP32 copy of z_j (input of the FP32 operator product)
  double *partial = nullptr, *dscal = nullptr, *dcoef = nullptr;
  double* hpin = nullptr;  // pinned host mirror of dscal
  cudaEvent_t ev = nullptr;
  unsigned* counter = nullptr;  // arrival counter of the MGS sweep reductions
  unsigned* step_words = nullptr;  // barrier count, exit count, error word of mgs_step
  long long steps = 0, restarts = 0;  // Arnoldi steps and cycles of the last solve
  // nested (GMRES-IR) mode: FP32 inner GMRES of inner_k steps per outer
  // step; its basis U32 ((k+1) vectors, U32[0] = the outer basis vector in
  // FP32), the preconditioned vectors Q32 (k), the working vector w32 and
  // the small FP64 arrays (raw Hessenberg (k+1) x k, ||w||^2 per step, y)
  int inner_k = 8, inner_alloc = 0;
  long long inner_steps = 0;  // inner steps of the last solve
  float *U32 = nullptr, *Q32 = nullptr, *w32 = nullptr;
  double* inner_small = nullptr;
  std::vector<void*> setup_bufs;
  void free_setup() {
    for (void* p : setup_bufs) cudaFreeAsync(p, st);
    setup_bufs.clear();
    Arow = Acol = diag = Lrow = Lcol = Urow = Ucol = nullptr;
    Aval = LU = Lval = Uval = nullptr;
    rdiag = nullptr;
    LU32 = rdiag32 = nullptr;
    Lval32 = Uval32 = nullptr;
    Aval32 = nullptr;
    ordL = lvlL = nlevL = ordU = lvlU = nlevU = nullptr;
    ilu_flags = nullptr;
    Prow = Pcol = nullptr;
    ilu_words = nullptr;
    ready = false;
  }
  void free_solver() {
    for (void* p : {(void*)V, (void*)Z, (void*)w, (void*)r, (void*)tmp, (void*)v32, (void*)z32,
                    (void*)partial, (void*)dscal, (void*)dcoef, (void*)counter,
                    (void*)step_words, (void*)U32,
                    (void*)Q32, (void*)w32, (void*)inner_small})
      if (p) cudaFreeAsync(p, st);
    U32 = Q32 = w32 = nullptr;
    inner_small = nullptr;
    inner_alloc = 0;
    v32 = nullptr;
    z32 = nullptr;
    counter = nullptr;
    step_words = nullptr;
    if (hpin) cudaFreeHost(hpin);
    if (ev) cudaEventDestroy(ev);
    ev = nullptr;
    V = Z = w = r = tmp = partial = dscal = dcoef = hpin = nullptr;
    m_alloc = 0;
  }
  template <class T>
  int alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = bilu::dev_alloc((void**)p, sizeof(T) * count, dev, st);
    if (e != cudaSuccess) return cuda_status(e);
    setup_bufs.push_back(*p);
    return BILU_OK;
  }
  // a setup buffer no longer needed goes back to the pool now (stream
  // ordered), so the solver's buffers reuse its memory
  void release(void* p) {
    if (!p) return;
    for (size_t i = 0; i < setup_bufs.size(); ++i)
      if (setup_bufs[i] == p) {
        setup_bufs[i] = setup_bufs.back();
        setup_bufs.pop_back();
        cudaFreeAsync(p, st);
        return;
      }
  }
};

extern "C" int bilu_ctx_create(bilu_ctx** ctx, bilu_stream_t stream) {
  if (!ctx) return BILU_ERR_ARG;
  bilu_ctx* c = new (std::nothrow) bilu_ctx();
  if (!c) return BILU_ERR_ARG;
  cudaGetDevice(&c->dev);
  c->st = S(stream);
  *ctx = c;
  return BILU_OK;
}

extern "C" int bilu_ctx_destroy(bilu_ctx* ctx) {
  if (!ctx) return BILU_OK;
  cudaStreamSynchronize(ctx->st);
  ctx->free_setup();
  ctx->free_solver();
  delete ctx;
  return BILU_OK;
}

namespace {

struct Timer {
  cudaEvent_t e[6];
  cudaStream_t st;
  explicit Timer(cudaStream_t s) : st(s) {
    for (auto& x : e) cudaEventCreate(&x);
  }
  ~Timer() {
    for (auto& x : e) cudaEventDestroy(x);
  }
  void mark(int i) { cudaEventRecord(e[i], st); }
  double ms(int a, int b) {
    float v = 0;
    cudaEventSynchronize(e[b]);
    cudaEventElapsedTime(&v, e[a], e[b]);
    return v;
  }
};

// The structure of one ISAI side: M's BCSC pattern (Mptr, Mind), its BCSR
// view (Trow, Tcol) with the BCSC -> BCSR map, and the pair lists.
struct IsaiSym {
  int *Mptr = nullptr, *Mind = nullptr, *Trow = nullptr, *Tcol = nullptr, *map = nullptr;
  int *pp = nullptr, *pl = nullptr, *ps = nullptr;
  int mnnz = 0;
};

// Structure only (A's pattern, or pattern(A^k) for ISAI(k)): may run before
// the values are on the device.
int build_isai_sym(bilu_ctx* c, int lower, Carver& ws, IsaiSym& y, double* t_pattern) {
  cudaStream_t st = c->st;
  int nb = c->nb;
  // the M patterns come from pattern(A^k) for ISAI(k); the pair lists, Dinv
  // and the column solves still read the factor on A's pattern
  const int* pr = c->Prow ? c->Prow : c->Arow;
  const int* pc = c->Pcol ? c->Pcol : c->Acol;
  Timer tm(st);
  tm.mark(0);
  BILU_TRY(c->alloc(&y.Mptr, nb + 1));
  BILU_TRY(c->alloc(&y.Trow, nb + 1));
  int mnnz = 0, tnnz = 0;
  {
    Carver w2 = ws;
    BILU_TRY(isai_pattern_colptr_impl(nb, pr, pc, lower, y.Mptr, &mnnz, w2, st));
  }
  {
    Carver w2 = ws;
    BILU_TRY(tri_pattern_rowptr_impl(nb, pr, pc, lower, y.Trow, &tnnz, w2, st));
  }
  // the reference's guard (main.cu:537-546): both views must hold the same
  // blocks, i.e. every diagonal block is stored
  if (mnnz != tnnz) return BILU_ERR_PATTERN;
  BILU_TRY(c->alloc(&y.Mind, mnnz));
  BILU_TRY(c->alloc(&y.Tcol, tnnz));
  BILU_TRY(c->alloc(&y.map, mnnz));
  {
    Carver w2 = ws;
    if (!w2.take<int>(2)) return BILU_ERR_WORKSPACE;
    BILU_TRY(isai_pattern_fill_impl(nb, pr, pc, lower, y.Mptr, y.Mind, mnnz, w2, st));
  }
  BILU_TRY(tri_pattern_fill_impl(nb, pr, pc, lower, y.Trow, y.Tcol, st));
  {
    Carver w2 = ws;
    BILU_TRY(map_impl(nb, y.Mptr, y.Mind, y.Trow, y.Tcol, y.map, nullptr, w2, st));
  }
  BILU_TRY(c->alloc(&y.pp, (size_t)mnnz + 1));
  int total = 0;
  {
    Carver w2 = ws;
    BILU_TRY(pairs_ptr_impl(nb, c->Arow, c->Acol, y.Mptr, y.Mind, lower, y.pp, mnnz, &total,
                            nullptr, w2, st));
  }
  BILU_TRY(c->alloc(&y.pl, total));
  BILU_TRY(c->alloc(&y.ps, total));
  BILU_TRY(pairs_fill_impl(nb, c->Arow, c->Acol, y.Mptr, y.Mind, lower, y.pp, mnnz, y.pl, y.ps,
                           st));
  y.mnnz = mnnz;
  tm.mark(1);
  *t_pattern += tm.ms(0, 1);
  return BILU_OK;
}

// The values of one ISAI side on the factor: Dinv, the column solves into
// BCSC and the reorder into BCSR (with the FP32 copy when asked for).
int build_isai_num(bilu_ctx* c, int lower, const IsaiSym& y, int** orow, int** ocol,
                   double** oval, int* onnz, double* t_isai, float** oval32) {
  cudaStream_t st = c->st;
  int nb = c->nb, bs = c->bs, bs2 = bs * bs;
  Timer tm(st);
  tm.mark(0);
  double *Dinv, *Mcsc, *Mcsr;
  BILU_TRY(c->alloc(&Dinv, (size_t)nb * bs2));
  BILU_TRY(c->alloc(&Mcsc, (size_t)y.mnnz * bs2));
  BILU_TRY(c->alloc(&Mcsr, (size_t)y.mnnz * bs2));
  BILU_TRY(dinv_impl(nb, bs, c->Arow, c->Acol, c->LU, lower, Dinv, nullptr, st));
  BILU_TRY(isai_impl(nb, bs, c->LU, y.Mptr, y.Mind, lower, y.pp, y.pl, y.ps, Dinv, Mcsc, st));
  // the FP32 copy of the mixed apply is written by the same pass
  float* M32 = nullptr;
  if (oval32) BILU_TRY(c->alloc(&M32, (size_t)y.mnnz * bs2));
  BILU_TRY(reorder_impl(y.mnnz, bs, y.map, Mcsc, Mcsr, st, M32));
  if (oval32) *oval32 = M32;
  c->release(Mcsc);
  c->release(Dinv);
  tm.mark(1);
  *t_isai += tm.ms(0, 1);
  *orow = y.Trow;
  *ocol = y.Tcol;
  *oval = Mcsr;
  *onnz = y.mnnz;
  return BILU_OK;
}

}  // namespace

namespace {

// Setup in two phases.  Structure first (row pointers and column indices
// only): diagonal positions, BILU(0)'s level analysis, pattern(A^k), the
// ISAI patterns and pair lists of both sides, the SpMV layouts and the upper
// level analysis of the exact-ILU modes.  Then, after values_ready (an event
// the caller records when d_val is on the device; null: already there), the
// values: BILU(0), Dinv, the ISAI column solves, the reorders and the FP32
// copies.  The structure phase thus overlaps a host-to-device copy of the
// values that the caller issues on another stream.
// adopt_val: d_val is a buffer of the library's pool that the handle takes
// over as its copy of A (the host-buffer entry point's upload), instead of
// copying it.
int ctx_setup(bilu_ctx* c, int nb, int nnzb, int bs, const int* d_row, const int* d_col,
              const double* d_val, int prec_mask, double* h_times, cudaEvent_t values_ready,
              bool adopt_val = false) {
  if (!c || nb < 1 || nnzb < nb || !d_row || !d_col || !d_val) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = c->st;
  c->free_setup();
  // solver buffers are sized for n: a new system size reallocates them
  if (c->n != (long long)nb * bs) c->free_solver();
  c->nb = nb;
  c->nnzb = nnzb;
  c->bs = bs;
  c->n = (long long)nb * bs;
  size_t bs2 = (size_t)bs * bs;
  Timer tm(st);
  tm.mark(0);
  BILU_TRY(c->alloc(&c->Arow, nb + 1));
  BILU_TRY(c->alloc(&c->Acol, nnzb));
  BILU_TRY(c->alloc(&c->diag, nb + 1));
  BILU_TRY_CUDA(cudaMemcpyAsync(c->Arow, d_row, sizeof(int) * (nb + 1), cudaMemcpyDeviceToDevice, st));
  BILU_TRY_CUDA(cudaMemcpyAsync(c->Acol, d_col, sizeof(int) * nnzb, cudaMemcpyDeviceToDevice, st));
  // scratch shared by every step
  size_t wsb = std::max({isai_pattern_ws(nb, nnzb), bilu0_ws(nb, nnzb), pairs_ws(nnzb + nb),
                         levels_ws(nb, nnzb), pattern_product_ws(nb),
                         scan_ws_bytes(nnzb + nb + 1)}) + (1 << 16);
  void* wsp = nullptr;
  void* wsq = nullptr;  // a larger scratch for the pattern(A^k) steps
  BILU_TRY(c->alloc((char**)&wsp, wsb));
  Carver ws(wsp, wsb);
  {
    Carver w2 = ws;
    BILU_TRY(diag_positions(nb, c->Arow, c->Acol, c->diag, nullptr, w2, st));
  }
  // BILU(0)'s analysis of the lower DAG, kept: the exact-ILU apply's lower
  // solves reuse it
  const int ilu_bits = (1 << BILU_ILU) | (1 << BILU_ILU_FP32);
  const bool ilu = (prec_mask & ilu_bits) != 0;
  BILU_TRY(c->alloc(&c->ordL, (size_t)nb + 1));
  BILU_TRY(c->alloc(&c->lvlL, (size_t)nb + 2));
  BILU_TRY(c->alloc(&c->nlevL, 4));
  LevelOut keepL;
  keepL.order = c->ordL;
  keepL.lvl = c->lvlL;
  keepL.nlev = c->nlevL;
  tm.mark(1);
  {
    Carver w2 = ws;
    BILU_TRY(bilu0_analyze(nb, nnzb, c->Arow, c->Acol, c->diag, keepL, w2, st));
  }
  // the level-order factorisation's match lists (which A_IJ each L_IK
  // updates, with U_KJ), built here from the pattern instead of searched
  // for inside every row's dependency chain; at most 4 pairs a block.  The
  // sync-free factorisation (long rows) keeps its searches: on the
  // power-law system the lists cost as much to build as they saved.
  int* mptr = nullptr;
  int2* mpair = nullptr;
  const int fsched = (c->schedule == 0 || c->schedule == 1) ? c->schedule : keepL.h_fsched;
  if (fsched == 0) {
    BILU_TRY(c->alloc(&mptr, (size_t)nnzb + 1));
    long long total = 0;
    const long long cap = 4ll * nnzb;
    {
      Carver w2 = ws;
      BILU_TRY(bilu0_match_count(nb, nnzb, c->Arow, c->Acol, c->diag, mptr, cap, &total, w2, st));
    }
    if (total <= cap && total <= (long long)INT_MAX) {
      BILU_TRY(c->alloc(&mpair, (size_t)total));
      BILU_TRY(bilu0_match_fill(nb, nnzb, c->Arow, c->Acol, c->diag, mptr, mpair, st));
      keepL.mptr = mptr;
      keepL.mpair = mpair;
    } else {
      c->release(mptr);
      mptr = nullptr;
    }
  }
  tm.mark(2);
  double t_pat = 0, t_isai = 0;
  // a mask of exact-ILU modes alone builds no ISAI
  const bool isai = (prec_mask & ~ilu_bits) != 0 || (prec_mask & ilu_bits) == 0;
  if (isai && c->isai_level > 1) {
    // pattern(A^k) by repeated symbolic products with A
    const int *xr = c->Arow, *xc = c->Acol;
    for (int k = 2; k <= c->isai_level; ++k) {
      int *cr = nullptr, *cc = nullptr, nnz = 0;
      BILU_TRY(c->alloc(&cr, (size_t)nb + 1));
      {
        Carver w2 = ws;
        BILU_TRY(pattern_product_rowptr(nb, xr, xc, c->Arow, c->Acol, cr, &nnz, nullptr, w2, st));
      }
      BILU_TRY(c->alloc(&cc, (size_t)nnz));
      {
        Carver w2 = ws;
        BILU_TRY(pattern_product_fill(nb, xr, xc, c->Arow, c->Acol, cr, cc, w2, st));
      }
      xr = cr;
      xc = cc;
      c->Prow = cr;
      c->Pcol = cc;
      c->nnzP = nnz;
    }
    // the pattern steps below scale with nnz(pattern(A^k))
    long long np = c->nnzP;
    size_t need = std::max({isai_pattern_ws(nb, np), pairs_ws(np + nb),
                            scan_ws_bytes(np + nb + 1)}) + (1 << 16);
    if (need > wsb) {
      BILU_TRY(c->alloc((char**)&wsq, need));
      ws = Carver(wsq, need);
    }
  }
  IsaiSym symL, symU;
  if (isai) {
    BILU_TRY(build_isai_sym(c, 1, ws, symL, &t_pat));
    BILU_TRY(build_isai_sym(c, 0, ws, symU, &t_pat));
  }
  {
    Carver w2 = ws;
    int* words = w2.take<int>(1);
    if (!words) return BILU_ERR_WORKSPACE;
    BILU_TRY(spmv_layout_of(nb, bs, c->Arow, words, st, &c->spmv_layout[0]));
    c->spmv_layout[1] = c->spmv_layout[2] = 0;
    if (isai) {
      BILU_TRY(spmv_layout_of(nb, bs, symL.Trow, words, st, &c->spmv_layout[1]));
      BILU_TRY(spmv_layout_of(nb, bs, symU.Trow, words, st, &c->spmv_layout[2]));
    }
  }
  if (ilu) {
    // level analyses of both triangles of the packed factor for the exact
    // BILU(0) apply (two level-order triangular solves per apply): the
    // lower one is BILU(0)'s, the upper one is built here
    c->nlev_host[0] = keepL.h_nlev;
    c->ilu_sched[0] = keepL.h_sched;
    c->ilu_maxdeg[0] = keepL.h_maxdeg;
    BILU_TRY(c->alloc(&c->ordU, (size_t)nb + 1));
    BILU_TRY(c->alloc(&c->lvlU, (size_t)nb + 2));
    BILU_TRY(c->alloc(&c->nlevU, 4));
    {
      Carver w2 = ws;
      BILU_TRY(level_analysis(nb, nnzb, c->Arow, c->Acol, c->diag, 0, c->ordU, c->lvlU, c->nlevU,
                              &c->nlev_host[1], w2, st, &c->ilu_sched[1], &c->ilu_maxdeg[1]));
    }
    for (int t = 0; t < 2; ++t)
      if (c->schedule == 0 || c->schedule == 1) c->ilu_sched[t] = c->schedule;
  }
  // the values
  if (values_ready) BILU_TRY_CUDA(cudaStreamWaitEvent(st, values_ready, 0));
  tm.mark(3);
  if (adopt_val) {
    c->Aval = const_cast<double*>(d_val);
    c->setup_bufs.push_back(c->Aval);
  } else {
    BILU_TRY(c->alloc(&c->Aval, nnzb * bs2));
    BILU_TRY_CUDA(cudaMemcpyAsync(c->Aval, d_val, sizeof(double) * nnzb * bs2,
                                  cudaMemcpyDeviceToDevice, st));
  }
  BILU_TRY(c->alloc(&c->LU, nnzb * bs2));
  BILU_TRY(c->alloc(&c->rdiag, (size_t)nb * bs + 1));
  BILU_TRY_CUDA(cudaMemcpyAsync(c->LU, d_val, sizeof(double) * nnzb * bs2, cudaMemcpyDeviceToDevice, st));
  {
    Carver w2 = ws;
    int zp = -1;
    int rc = bilu0_factor(nb, nnzb, bs, c->Arow, c->Acol, c->diag, c->LU, &zp, w2, st,
                          c->schedule, c->rdiag, keepL);
    if (rc != BILU_OK) return rc;
  }
  c->release(mptr);
  c->release(mpair);
  keepL.mptr = nullptr;
  keepL.mpair = nullptr;
  tm.mark(4);
  if (isai) {
    const bool want32 =
        (prec_mask & ((1 << BILU_FP32) | (1 << BILU_FP32_INNER) | (1 << BILU_NESTED))) != 0;
    BILU_TRY(build_isai_num(c, 1, symL, &c->Lrow, &c->Lcol, &c->Lval, &c->nnzL, &t_isai,
                            want32 ? &c->Lval32 : nullptr));
    BILU_TRY(build_isai_num(c, 0, symU, &c->Urow, &c->Ucol, &c->Uval, &c->nnzU, &t_isai,
                            want32 ? &c->Uval32 : nullptr));
  }
  if (prec_mask & ((1 << BILU_FP32_INNER) | (1 << BILU_NESTED))) {
    BILU_TRY(c->alloc(&c->Aval32, (size_t)nnzb * bs2));
    BILU_TRY(bilu_convert_f64_to_f32((size_t)nnzb * bs2, c->Aval, c->Aval32, st));
  }
  if (ilu) {
    BILU_TRY(c->alloc(&c->ilu_flags, (size_t)nb + 2));
    BILU_TRY(c->alloc(&c->ilu_words, 4));
    BILU_TRY_CUDA(cudaMemsetAsync(c->ilu_words, 0, sizeof(unsigned) * 4, st));
    // FP32 factor for the mixed exact-ILU apply (the level-order kernel has
    // an FP32 form for rows of up to 32 dependencies)
    if ((prec_mask & (1 << BILU_ILU_FP32)) && c->ilu_maxdeg[0] <= 32 && c->ilu_maxdeg[1] <= 32) {
      BILU_TRY(c->alloc(&c->LU32, (size_t)nnzb * bs2));
      BILU_TRY(c->alloc(&c->rdiag32, (size_t)nb * bs));
      BILU_TRY(bilu_convert_f64_to_f32((size_t)nnzb * bs2, c->LU, c->LU32, st));
      BILU_TRY(bilu_convert_f64_to_f32((size_t)nb * bs, c->rdiag, c->rdiag32, st));
    }
  }

  // the structure of the ISAI columns, the pair lists and the scratch are
  // not read after the setup
  for (IsaiSym* y : {&symL, &symU})
    for (void* p : {(void*)y->Mptr, (void*)y->Mind, (void*)y->map, (void*)y->pp, (void*)y->pl,
                    (void*)y->ps})
      c->release(p);
  c->release(wsp);
  c->release(wsq);
  tm.mark(5);
  // factor: BILU(0)'s analysis and factorisation
  double t_factor = tm.ms(1, 2) + tm.ms(3, 4), t_total = tm.ms(0, 5);
  BILU_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_times) {
    h_times[0] = t_factor;
    h_times[1] = t_pat;
    h_times[2] = t_isai;
    h_times[3] = t_total;
  }
  c->ready = true;
  return BILU_OK;
}

}  // namespace

extern "C" int bilu_ctx_setup(bilu_ctx* c, int nb, int nnzb, int bs, const int* d_row,
                              const int* d_col, const double* d_val, int prec_mask,
                              double* h_times) {
  return ctx_setup(c, nb, nnzb, bs, d_row, d_col, d_val, prec_mask, h_times, nullptr);
}

extern "C" int bilu_ctx_set_schedule(bilu_ctx* c, int schedule) {
  if (!c || schedule < -1 || schedule > 1) return BILU_ERR_ARG;
  c->schedule = schedule;
  return BILU_OK;
}

extern "C" int bilu_ctx_set_isai_level(bilu_ctx* c, int k) {
  if (!c || k < 1 || k > 3) return BILU_ERR_ARG;
  c->isai_level = k;
  return BILU_OK;
}

extern "C" int bilu_ctx_get(bilu_ctx* c, int which, const void** d_ptr, long long* h_count) {
  if (!c || !d_ptr || !c->ready) return BILU_ERR_ARG;
  long long bs2 = (long long)c->bs * c->bs;
  const void* p = nullptr;
  long long cnt = 0;
  switch (which) {
    case 0: p = c->LU; cnt = c->nnzb * bs2; break;
    case 1: p = c->Lrow; cnt = p ? c->nb + 1 : 0; break;
    case 2: p = c->Lcol; cnt = p ? c->nnzL : 0; break;
    case 3: p = c->Lval; cnt = p ? c->nnzL * bs2 : 0; break;
    case 4: p = c->Urow; cnt = p ? c->nb + 1 : 0; break;
    case 5: p = c->Ucol; cnt = p ? c->nnzU : 0; break;
    case 6: p = c->Uval; cnt = p ? c->nnzU * bs2 : 0; break;
    case 7: p = c->Lval32; cnt = c->Lval32 ? c->nnzL * bs2 : 0; break;
    case 8: p = c->Uval32; cnt = c->Uval32 ? c->nnzU * bs2 : 0; break;
    default: return BILU_ERR_ARG;
  }
  *d_ptr = p;
  if (h_count) *h_count = cnt;
  return BILU_OK;
}

namespace {

int ensure_solver(bilu_ctx* c, int m) {
  if (c->m_alloc >= m && c->V) return BILU_OK;
  c->free_solver();
  size_t n = (size_t)c->n;
  // basis vectors start on 256-byte boundaries (16-byte vector loads)
  c->ldv = (long long)((n + 31) & ~(size_t)31);
  auto get = [&](auto** p, size_t bytes) {
    return dev_alloc((void**)p, bytes, c->dev, c->st);
  };
  BILU_TRY_CUDA(get(&c->V, sizeof(double) * c->ldv * (m + 1)));
  BILU_TRY_CUDA(get(&c->Z, sizeof(double) * c->ldv * m));
  BILU_TRY_CUDA(get(&c->w, sizeof(double) * n));
  BILU_TRY_CUDA(get(&c->r, sizeof(double) * n));
  BILU_TRY_CUDA(get(&c->tmp, sizeof(double) * n));
  BILU_TRY_CUDA(get(&c->v32, sizeof(float) * n));
  BILU_TRY_CUDA(get(&c->z32, sizeof(float) * n));
  BILU_TRY_CUDA(get(&c->partial, sizeof(double) * kRedCTAs * kPartStride));
  BILU_TRY_CUDA(get(&c->dscal, sizeof(double) * 6 * kPartStride));
  BILU_TRY_CUDA(get(&c->dcoef, sizeof(double) * kPartStride));
  BILU_TRY_CUDA(cudaMallocHost(&c->hpin, sizeof(double) * 6 * kPartStride));
  BILU_TRY_CUDA(get(&c->counter, sizeof(unsigned)));
  BILU_TRY_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->st));
  BILU_TRY_CUDA(get(&c->step_words, sizeof(unsigned) * 4));
  BILU_TRY_CUDA(cudaMemsetAsync(c->step_words, 0, sizeof(unsigned) * 4, c->st));
  c->m_alloc = m;
  return BILU_OK;
}

// ||v||^2 into dscal[slot] (device) and, if host != null, to the host.
int norm2(bilu_ctx* c, const double* v, double* dslot, double* host) {
  BILU_TRY(multidot(c->n, nullptr, 0, 0, v, true, c->partial, c->st));
  BILU_TRY(reduce_partials(c->partial, 1, dslot, c->st));
  if (host) {
    BILU_TRY_CUDA(cudaMemcpyAsync(host, dslot, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    BILU_TRY_CUDA(cudaStreamSynchronize(c->st));
  }
  return BILU_OK;
}

// whether the setup built what a preconditioner mode needs (-1: none)
bool mode_built(const bilu_ctx* c, int prec) {
  switch (prec) {
    case -1: return true;
    case BILU_FP64: return c->Lval != nullptr;
    case BILU_FP32: return c->Lval32 != nullptr;
    case BILU_ILU: return c->ilu_words != nullptr;
    case BILU_FP32_INNER: return c->Aval32 != nullptr;
    case BILU_ILU_FP32: return c->LU32 != nullptr;
    case BILU_NESTED: return c->Aval32 != nullptr && c->Lval32 != nullptr;
    default: return false;
  }
}

// modes whose apply starts from the FP32 copy of the basis vector
bool uses_v32(int prec) {
  return prec == BILU_FP32 || prec == BILU_FP32_INNER || prec == BILU_ILU_FP32 ||
         prec == BILU_NESTED;
}

// where the normalisation kernel writes that FP32 copy: the nested mode's
// inner basis starts with it
float* v32_of(bilu_ctx* c, int prec) {
  if (!uses_v32(prec)) return nullptr;
  return prec == BILU_NESTED ? c->U32 : c->v32;
}

int ensure_inner(bilu_ctx* c) {
  const int k = c->inner_k;
  if (c->inner_alloc >= k && c->U32) return BILU_OK;
  for (void* p : {(void*)c->U32, (void*)c->Q32, (void*)c->w32, (void*)c->inner_small})
    if (p) cudaFreeAsync(p, c->st);
  c->U32 = c->Q32 = c->w32 = nullptr;
  c->inner_small = nullptr;
  c->inner_alloc = 0;
  const size_t ld = (size_t)c->ldv;
  BILU_TRY_CUDA(dev_alloc((void**)&c->U32, sizeof(float) * ld * (k + 1), c->dev, c->st));
  BILU_TRY_CUDA(dev_alloc((void**)&c->Q32, sizeof(float) * ld * k, c->dev, c->st));
  BILU_TRY_CUDA(dev_alloc((void**)&c->w32, sizeof(float) * ld, c->dev, c->st));
  BILU_TRY_CUDA(dev_alloc((void**)&c->inner_small,
                          sizeof(double) * ((size_t)(k + 1) * k + 2 * (size_t)k), c->dev, c->st));
  c->inner_alloc = k;
  return BILU_OK;
}

// The nested mode's preconditioner: inner_k steps of right-preconditioned
// FP32 GMRES on A z = v from z = 0, with the FP32-stored A and ISAI, the
// basis starting from u_0 = v in FP32 (U32[0], written by the kernel that
// normalised v; v has unit norm, so beta = 1: flexible GMRES accepts any
// scaling of z).  Every step: q_i = M_U (M_L u_i) into Q32[i], w = A q_i,
// then one cooperative launch of the i + 2 fused FP32 Gram-Schmidt sweeps
// writing h_0i..h_ii and ||w||^2, and u_{i+1} = w / ||w||.  Then the
// Hessenberg least-squares problem on the device and z = Q y widened to
// FP64.  Nothing waits on the host: the whole inner solve is queued on the
// stream.
int inner_solve(bilu_ctx* c, double* z) {
  cudaStream_t st = c->st;
  const long long n = c->n;
  const size_t ld = (size_t)c->ldv;
  const int k = c->inner_k;
  double* H = c->inner_small;                // (k+1) x k, H[i*k + j]
  double* ww = H + (size_t)(k + 1) * k;      // ||w_j||^2
  double* y = ww + k;
  float* t32 = reinterpret_cast<float*>(c->tmp);
  for (int j = 0; j < k; ++j) {
    const float* uj = c->U32 + ld * j;
    float* qj = c->Q32 + ld * j;
    BILU_TRY(spmv_any(c->nb, c->bs, BILU_FP32, c->Lrow, c->Lcol, c->Lval32, uj, 1, t32, 1, st,
                      c->spmv_layout[1]));
    BILU_TRY(spmv_any(c->nb, c->bs, BILU_FP32, c->Urow, c->Ucol, c->Uval32, t32, 1, qj, 1, st,
                      c->spmv_layout[2]));
    BILU_TRY(spmv_any(c->nb, c->bs, BILU_FP32, c->Arow, c->Acol, c->Aval32, qj, 1, c->w32, 1, st,
                      c->spmv_layout[0]));
    // the j+2 FP32 sweeps and u_{j+1} = w / ||w|| in one cooperative launch
    BILU_TRY(mgs_step_f32(n, c->U32, (long long)ld, j, c->w32, H + j, k, ww + j, c->partial,
                          c->step_words, j + 1 < k ? c->U32 + ld * (j + 1) : nullptr, st));
  }
  BILU_TRY(inner_lsq(k, H, ww, y, st));
  return combine_f32(n, c->Q32, (long long)ld, k, y, z, st);
}

int apply_prec(bilu_ctx* c, int prec, const double* v, double* z) {
  if (prec == BILU_ILU_FP32) {
    // z = U^-1 (L^-1 v) in FP32 on the FP32 factor: L from the FP32 copy of
    // v (written with v by the normalisation kernel) into t32, U from t32
    // into x32 with z as its FP64 copy (tmp holds n doubles = 2n floats)
    float* t32 = reinterpret_cast<float*>(c->tmp);
    float* x32 = t32 + c->n;
    BILU_TRY(sptrsv_flow_f32_async(c->nb, c->bs, c->Arow, c->Acol, c->diag, c->ordL, c->lvlL,
                                   c->nlevL, c->LU32, 1, 1, c->v32, t32, nullptr, c->ilu_words,
                                   c->st, nullptr, c->ilu_maxdeg[0]));
    return sptrsv_flow_f32_async(c->nb, c->bs, c->Arow, c->Acol, c->diag, c->ordU, c->lvlU,
                                 c->nlevU, c->LU32, 0, 0, t32, x32, z, c->ilu_words, c->st,
                                 c->rdiag32, c->ilu_maxdeg[1]);
  }
  if (prec == BILU_ILU) {
    // z = U^-1 (L^-1 v): unit-lower then upper solve on the packed factor,
    // each with the schedule its level analysis recommends
    for (int lower = 1; lower >= 0; --lower) {
      const double* in = lower ? v : c->tmp;
      double* out = lower ? c->tmp : z;
      const int* ord = lower ? c->ordL : c->ordU;
      if (c->ilu_sched[lower ? 0 : 1] == 1)
        BILU_TRY(sptrsv_syncfree_async(c->nb, c->bs, c->Arow, c->Acol, c->diag, ord, c->LU,
                                       lower, lower, in, out, c->ilu_flags,
                                       c->ilu_flags + c->nb + 1, (int*)c->ilu_words + 2, c->st,
                                       lower ? nullptr : c->rdiag));
      else
        BILU_TRY(sptrsv_levels_async(c->nb, c->bs, c->Arow, c->Acol, c->diag, ord,
                                     lower ? c->lvlL : c->lvlU, lower ? c->nlevL : c->nlevU,
                                     c->LU, lower, lower, in, out, c->ilu_words, c->st,
                                     lower ? nullptr : c->rdiag, c->ilu_maxdeg[lower ? 0 : 1]));
    }
    return BILU_OK;
  }
  if (prec < 0) {
    BILU_TRY_CUDA(cudaMemcpyAsync(z, v, sizeof(double) * c->n, cudaMemcpyDeviceToDevice, c->st));
    return BILU_OK;
  }
  if (prec == BILU_NESTED) return inner_solve(c, z);
  if (prec == BILU_FP32 || prec == BILU_FP32_INNER) {
    // v32 (written with v by the normalisation kernel) is the FP32 copy of v
    if (!c->Lval32 || !c->Uval32) return BILU_ERR_ARG;
    return isai_apply_f32_staged(c->nb, c->bs, c->Lrow, c->Lcol, c->Lval32, c->Urow, c->Ucol,
                                 c->Uval32, c->v32, (float*)c->tmp, z, c->st,
                                 prec == BILU_FP32_INNER ? c->z32 : nullptr, c->spmv_layout[1],
                                 c->spmv_layout[2]);
  }
  return isai_apply_impl(c->nb, c->bs, prec, c->Lrow, c->Lcol, c->Lval, c->Urow, c->Ucol,
                         c->Uval, v, c->tmp, z, c->st, c->spmv_layout[1], c->spmv_layout[2]);
}

}  // namespace

namespace {

// Launches z_j = M v_j and w = A z_j.
int arnoldi_front(bilu_ctx* c, int prec, int j) {
  size_t ld = (size_t)c->ldv;
  double* zj = c->Z + ld * j;
  BILU_TRY(apply_prec(c, prec, c->V + ld * j, zj));
  if (prec == BILU_FP32_INNER)  // FP32-stored A and z (written by the apply), FP64 w
    return spmv_any(c->nb, c->bs, BILU_FP32, c->Arow, c->Acol, c->Aval32, c->z32, 1, c->w, 0,
                    c->st, c->spmv_layout[0]);
  return spmv_any(c->nb, c->bs, BILU_FP64, c->Arow, c->Acol, c->Aval, zj, 0, c->w, 0, c->st,
                  c->spmv_layout[0]);
}

// Orthogonalises w against V_0..V_j by modified Gram-Schmidt: j+2 fused
// sweeps (w -= h_{i-1} v_{i-1} together with h_i = v_i . w; the last one
// gives ||w||^2) and V_{j+1} = w / ||w|| in one cooperative launch, each
// sum reduced in a fixed order on the device; the Hessenberg column and
// the launch's error word are queued to hpin.
// s[0..j] = h, s[kPartStride] = ||w||^2.
int arnoldi_back(bilu_ctx* c, int j, int prec) {
  cudaStream_t st = c->st;
  long long n = c->n;
  size_t ld = (size_t)c->ldv;
  double* s = c->dscal;
  const double* V = c->V;
  BILU_TRY(mgs_step(n, V, (long long)ld, j, c->w, s, 1, s + kPartStride, c->partial,
                    c->step_words, c->V + ld * (j + 1), v32_of(c, prec), st));
  BILU_TRY_CUDA(cudaMemcpyAsync(c->hpin, s, sizeof(double) * (kPartStride + 1),
                                cudaMemcpyDeviceToHost, st));
  // the barrier error word of this step's (and the inner solver's) launches
  BILU_TRY_CUDA(cudaMemcpyAsync(c->hpin + kPartStride + 1, c->step_words + 2, sizeof(unsigned),
                                cudaMemcpyDeviceToHost, st));
  return BILU_OK;
}

}  // namespace

extern "C" int bilu_ctx_solve(bilu_ctx* c, int prec, const double* d_b, double* d_x, int restart,
                              double tol, int maxit, int* h_iters, double* h_relres,
                              double* h_hist) {
  if (!c || !c->ready || !d_b || !d_x || restart < 1 || restart > kMaxVec - 1 || maxit < 0)
    return BILU_ERR_ARG;
  if (prec != -1 && prec != BILU_FP64 && prec != BILU_FP32 && prec != BILU_ILU &&
      prec != BILU_FP32_INNER && prec != BILU_ILU_FP32 && prec != BILU_NESTED)
    return BILU_ERR_ARG;
  if (!mode_built(c, prec)) return BILU_ERR_ARG;  // the setup did not build this preconditioner
  BILU_TRY(ensure_solver(c, restart));
  if (prec == BILU_NESTED) BILU_TRY(ensure_inner(c));
  c->inner_steps = 0;
  cudaStream_t st = c->st;
  const bool ilu_mode = prec == BILU_ILU || prec == BILU_ILU_FP32;
  if (ilu_mode) BILU_TRY_CUDA(cudaMemsetAsync(c->ilu_words, 0, sizeof(unsigned) * 4, st));
  BILU_TRY_CUDA(cudaMemsetAsync(c->step_words, 0, sizeof(unsigned) * 4, st));
  const int m = restart;
  const long long n = c->n;
  double* s = c->dscal;
  double* hp = c->hpin;
  if (!c->ev) BILU_TRY_CUDA(cudaEventCreateWithFlags(&c->ev, cudaEventDisableTiming));
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m);
  BILU_TRY_CUDA(cudaMemsetAsync(d_x, 0, sizeof(double) * n, st));
  double bb = 0;
  BILU_TRY(norm2(c, d_b, s, &bb));
  double bnorm = std::sqrt(bb);
  if (bnorm == 0.0) bnorm = 1.0;
  BILU_TRY_CUDA(cudaMemcpyAsync(c->r, d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  double rr = 0;
  BILU_TRY(norm2(c, c->r, s + 5 * kPartStride, &rr));
  double beta = std::sqrt(rr);
  int total = 0, status = BILU_ERR_NOT_CONVERGED;
  c->steps = 0;
  c->restarts = 0;
  double res = beta / bnorm;
  if (h_hist) h_hist[0] = res;
  if (res <= tol) status = BILU_OK;
  while (status != BILU_OK && total < maxit) {
    // V_0 = r / beta (beta^2 sits in s[5*kPartStride])
    BILU_TRY(scale_rsqrt(n, c->r, s + 5 * kPartStride, c->V, st, v32_of(c, prec)));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int jlast = -1;
    BILU_TRY(arnoldi_front(c, prec, 0));
    for (int j = 0; j < m && total < maxit; ++j) {
      BILU_TRY(arnoldi_back(c, j, prec));
      BILU_TRY_CUDA(cudaEventRecord(c->ev, st));
      // the next basis vector's apply and SpMV do not depend on the host
      // Givens step: queue them before waiting (discarded if this step
      // converges).  The nested mode's front is a whole inner solve, so it
      // waits for the host's convergence test instead (one round trip per
      // outer step, against an inner solve of milliseconds).
      const bool speculate = prec != BILU_NESTED;
      if (speculate && j + 1 < m && total + 1 < maxit) BILU_TRY(arnoldi_front(c, prec, j + 1));
      BILU_TRY_CUDA(cudaEventSynchronize(c->ev));
      unsigned step_err = 0;
      std::memcpy(&step_err, hp + kPartStride + 1, sizeof(unsigned));
      if (step_err != 0) {  // a grid barrier of the orthogonalisation timed out
        cudaStreamSynchronize(st);
        cudaMemsetAsync(c->step_words, 0, sizeof(unsigned) * 4, st);
        cudaStreamSynchronize(st);
        return (int)step_err;
      }
      for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hp[i];
      double hn = std::sqrt(hp[kPartStride]);
      H[(size_t)(j + 1) * m + j] = hn;
      for (int i = 0; i < j; ++i) {
        double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
        H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
        H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
      }
      double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
      double den = std::sqrt(a * a + b * b);
      cs[j] = den != 0.0 ? a / den : 1.0;
      sn[j] = den != 0.0 ? b / den : 0.0;
      H[(size_t)j * m + j] = cs[j] * a + sn[j] * b;
      H[(size_t)(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++total;
      jlast = j;
      res = std::fabs(g[j + 1]) / bnorm;
      if (h_hist) h_hist[total] = res;
      if (res <= tol || hn == 0.0) break;
      if (!speculate && j + 1 < m && total < maxit) BILU_TRY(arnoldi_front(c, prec, j + 1));
    }
    c->steps += jlast + 1;
    c->restarts += 1;
    for (int i = jlast; i >= 0; --i) {
      double v = g[i];
      for (int k = i + 1; k <= jlast; ++k) v -= H[(size_t)i * m + k] * y[k];
      y[i] = v / H[(size_t)i * m + i];
    }
    if (jlast >= 0) {
      BILU_TRY_CUDA(cudaMemcpyAsync(c->dcoef, y.data(), sizeof(double) * (jlast + 1),
                                    cudaMemcpyHostToDevice, st));
      BILU_TRY(multiaxpy_norm(n, c->Z, c->ldv, jlast + 1, c->dcoef, 1.0, d_x, nullptr, nullptr, st));
    }
    BILU_TRY(spmv_any(c->nb, c->bs, BILU_FP64, c->Arow, c->Acol, c->Aval, d_x, 0, c->w, 0, st,
                      c->spmv_layout[0]));
    BILU_TRY(residual_norm(n, d_b, c->w, c->r, c->partial, st));
    BILU_TRY(reduce_partials(c->partial, 1, s + 5 * kPartStride, st));
    BILU_TRY_CUDA(cudaMemcpyAsync(&rr, s + 5 * kPartStride, sizeof(double), cudaMemcpyDeviceToHost, st));
    int ilu_err = 0;
    if (ilu_mode)
      BILU_TRY_CUDA(cudaMemcpyAsync(&ilu_err, c->ilu_words + 2, sizeof(int),
                                    cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
    if (ilu_err != 0) return ilu_err;  // a triangular-solve barrier timed out
    beta = std::sqrt(rr);
    res = beta / bnorm;
    if (res <= tol) status = BILU_OK;
    if (beta == 0.0) break;
  }
  if (prec == BILU_NESTED) c->inner_steps = (long long)total * c->inner_k;
  if (h_iters) *h_iters = total;
  if (h_relres) *h_relres = res;
  return status;
}

extern "C" int bilu_ctx_stats(bilu_ctx* c, long long* h_out) {
  if (!c || !h_out) return BILU_ERR_ARG;
  h_out[0] = c->steps;
  h_out[1] = c->restarts;
  return BILU_OK;
}

extern "C" int bilu_ctx_set_inner(bilu_ctx* c, int k) {
  if (!c || k < 1 || k > kMaxVec) return BILU_ERR_ARG;
  c->inner_k = k;
  return BILU_OK;
}

extern "C" int bilu_ctx_inner_steps(bilu_ctx* c, long long* h_steps) {
  if (!c || !h_steps) return BILU_ERR_ARG;
  *h_steps = c->inner_steps;
  return BILU_OK;
}

// Preconditioner switch by measurement: up to `cycles` restart cycles (fewer
// if it reaches tol) of the solve from x0 = 0 with every choice in `mask` (bits 1 << BILU_FP64 /
// BILU_FP32 / BILU_ILU / BILU_FP32_INNER that the setup built), timed with
// events on the handle's stream.  The score is the residual reduction per
// second over the last cycle run (decimal digits / s): restarted GMRES gains
// most in its first cycle, so a one-cycle rate flatters the weaker
// preconditioner.  Returns the best choice in *h_choice and the scores in
// h_rate[4] (0 for choices not tried).
extern "C" int bilu_ctx_select(bilu_ctx* c, const double* d_b, int restart, int cycles,
                               double tol, int mask, int* h_choice, double* h_rate) {
  if (!c || !c->ready || !d_b || !h_choice || cycles < 1 || restart < 1) return BILU_ERR_ARG;
  double* x = nullptr;
  BILU_TRY_CUDA(cudaMalloc(&x, sizeof(double) * c->n));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<double> hist((size_t)restart * cycles + 1);
  int best = -1, rc = BILU_OK;
  double best_rate = -1.0;
  // h_rate has entries up to the highest choice the mask asks for (at
  // least four)
  int nrate = 4;
  for (int p = BILU_ILU_FP32; p <= BILU_NESTED; ++p)
    if (mask >> p) nrate = p + 1;
  for (int p = 0; p < nrate && rc == BILU_OK; ++p) {
    if (h_rate) h_rate[p] = 0.0;
    if (!(mask & (1 << p))) continue;
    if (!mode_built(c, p)) continue;
    int it = 0;
    double rr = 1.0;
    cudaEventRecord(e0, c->st);
    int st = bilu_ctx_solve(c, p, d_b, x, restart, tol, restart * cycles, &it, &rr, hist.data());
    cudaEventRecord(e1, c->st);
    cudaEventSynchronize(e1);
    if (st != BILU_OK && st != BILU_ERR_NOT_CONVERGED) {
      rc = st;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (it < 1) continue;
    // last cycle: iterations (it - 1) / restart * restart .. it
    int first = ((it - 1) / restart) * restart;
    double r0 = hist[first] > 0.0 ? hist[first] : 1.0;
    double r1 = rr > 0.0 ? rr : 1e-300;
    double digits = std::max(0.0, std::log10(r0) - std::log10(r1));
    double sec = ms * 1e-3 * (double)(it - first) / (double)it;
    double rate = sec > 0.0 ? digits / sec : 0.0;
    if (h_rate) h_rate[p] = rate;
    if (rate > best_rate) {
      best_rate = rate;
      best = p;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  if (rc != BILU_OK) return rc;
  if (best < 0) return BILU_ERR_ARG;
  *h_choice = best;
  return BILU_OK;
}

extern "C" int bilu_solve_host(int nb, int nnzb, int bs, const int* h_row, const int* h_col,
                               const double* h_val, const double* h_b, double* h_x, int prec,
                               int restart, double tol, int maxit, int* h_iters, double* h_relres,
                               double* h_times, bilu_stream_t stream) {
  if (nb < 1 || nnzb < 1 || !h_row || !h_col || !h_val || !h_b || !h_x) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  cudaStream_t st = S(stream);
  size_t bs2 = (size_t)bs * bs, n = (size_t)nb * bs;
  int *row = nullptr, *col = nullptr;
  double *val = nullptr, *b = nullptr, *x = nullptr;
  bilu_ctx* c = nullptr;
  int rc = BILU_OK;
  auto cu = [&](cudaError_t e) {
    if (rc == BILU_OK && e != cudaSuccess) rc = cuda_status(e);
  };
  int dev = 0;
  cu(cudaGetDevice(&dev));
  cu(dev_alloc((void**)&row, sizeof(int) * (nb + 1), dev, st));
  cu(dev_alloc((void**)&col, sizeof(int) * nnzb, dev, st));
  cu(dev_alloc((void**)&val, sizeof(double) * nnzb * bs2, dev, st));
  cu(dev_alloc((void**)&b, sizeof(double) * n, dev, st));
  cu(dev_alloc((void**)&x, sizeof(double) * n, dev, st));
  // the pattern on the caller's stream, the values (most of the bytes) and
  // b on a second stream: the setup's structure phase runs while they copy
  cudaStream_t side = nullptr;
  cudaEvent_t ev = nullptr;
  cu(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  cu(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (rc == BILU_OK) {
    cu(cudaEventRecord(ev, st));  // the buffers were allocated on st
    cu(cudaStreamWaitEvent(side, ev, 0));
    cu(cudaMemcpyAsync(row, h_row, sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st));
    cu(cudaMemcpyAsync(col, h_col, sizeof(int) * nnzb, cudaMemcpyHostToDevice, st));
    cu(cudaMemcpyAsync(val, h_val, sizeof(double) * nnzb * bs2, cudaMemcpyHostToDevice, side));
    cu(cudaMemcpyAsync(b, h_b, sizeof(double) * n, cudaMemcpyHostToDevice, side));
    cu(cudaEventRecord(ev, side));
  }
  if (rc == BILU_OK) rc = bilu_ctx_create(&c, stream);
  if (rc == BILU_OK) {
    // the handle keeps the uploaded values as its copy of A (one device
    // copy and 8 bytes per value less) and frees them with its other buffers
    rc = ctx_setup(c, nb, nnzb, bs, row, col, val, prec > 0 ? (1 << prec) : 0, h_times, ev,
                   true);
    if (c->Aval == val) val = nullptr;
  }
  int src = BILU_OK;
  if (rc == BILU_OK) {
    src = bilu_ctx_solve(c, prec, b, x, restart, tol, maxit, h_iters, h_relres, nullptr);
    if (src != BILU_OK && src != BILU_ERR_NOT_CONVERGED) rc = src;
  }
  if (rc == BILU_OK) {
    cu(cudaMemcpyAsync(h_x, x, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    cu(cudaStreamSynchronize(st));
  }
  bilu_ctx_destroy(c);
  // the side stream's copies are finished before the buffers go back (on a
  // failed setup the solve never waited for them)
  if (ev) cudaStreamWaitEvent(st, ev, 0);
  for (void* p : {(void*)row, (void*)col, (void*)val, (void*)b, (void*)x})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (ev) cudaEventDestroy(ev);
  if (side) cudaStreamDestroy(side);
  return rc != BILU_OK ? rc : src;
}
