// Sync-free block triangular solve that allocates nothing.
//
// Callers that cannot allocate device memory -- hosts whose device memory is
// owned by a fixed arena or budget, or plugins that may only touch the
// buffers they are given -- cannot provide the workspace bilu_sptrsv asks
// for.  This variant takes only the inputs and the output and keeps its
// scratch in one file-scope device array of fixed size, so it never calls
// cudaMalloc, cudaFree or any allocating routine.  It waits on its stream
// (to read the pattern check and the error word back), like bilu_sptrsv.
#include <mutex>

#include "common.cuh"

namespace bilu {

size_t syncfree_ws(int nb);
int diag_positions(int nb, const int* row, const int* col, int* diag, int* h_bad, Carver& ws,
                   cudaStream_t st);
int sptrsv_impl(int nb, int bs, const int* row, const int* col, const int* diag,
                const double* val, int lower, int unit, const double* b, double* x, Carver& ws,
                cudaStream_t st, long long spin, int withhold);

namespace {

// Scratch of the no-allocation solve: ready flags, level order, level
// counts, diagonal positions and scan sums for up to kNoAllocMaxRows block
// rows.  Every device that loads the library holds these bytes until exit.
constexpr int kNoAllocMaxRows = 262144;
constexpr size_t kNoAllocBytes = 6u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The first
// call on a device resolves it with cudaGetSymbolAddress (no allocation);
// later calls reuse the cached address.
int noalloc_scratch(void** out) {
  int dev = 0;
  BILU_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return BILU_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    BILU_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return BILU_OK;
}

}  // namespace

}  // namespace bilu

using namespace bilu;

extern "C" int bilu_sptrsv_noalloc_max_rows(void) { return kNoAllocMaxRows; }

extern "C" int bilu_sptrsv_noalloc(int nb, int bs, const int* d_row, const int* d_col,
                                   const double* d_val, int lower, const double* d_b, double* d_x,
                                   bilu_stream_t stream) {
  if (nb < 0 || (nb > 0 && (!d_row || !d_col || !d_val || !d_b || !d_x))) return BILU_ERR_ARG;
  // b is read while x is written: they may not share memory
  if (nb > 0 && (const void*)d_b == (const void*)d_x) return BILU_ERR_ARG;
  if (!bs_supported(bs)) return BILU_ERR_UNSUPPORTED;
  if (nb > kNoAllocMaxRows) return BILU_ERR_WORKSPACE;
  size_t need = syncfree_ws(nb) + carve_size(sizeof(int) * ((size_t)nb + 1));
  if (need > kNoAllocBytes) return BILU_ERR_WORKSPACE;
  void* scratch = nullptr;
  BILU_TRY(noalloc_scratch(&scratch));
  Carver ws(scratch, kNoAllocBytes);
  int* diag = ws.take<int>((size_t)nb + 1);
  if (!diag) return BILU_ERR_WORKSPACE;
  BILU_TRY(diag_positions(nb, d_row, d_col, diag, nullptr, ws, S(stream)));
  return sptrsv_impl(nb, bs, d_row, d_col, diag, d_val, lower != 0, lower != 0, d_b, d_x, ws,
                     S(stream), kSpinLimit, -1);
}
