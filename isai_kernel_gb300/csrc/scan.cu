// Device-wide exclusive scan of int32: tile sums -> single-CTA scan of the
// tile sums -> per-tile scan with offset.  Replaces thrust::exclusive_scan
// (main.cu:684) and the cub::DeviceScan of bcsc2bcsrAndSpMV.h:101.
#include "scan.cuh"

namespace bilu {

namespace {

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int warp_tot[kScanThreads / 32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;
    if (lane == kScanThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  int r = incl - v + warp_tot[warp];
  __syncthreads();
  return r;
}

__global__ void k_tile_sums(const int* __restrict__ in, long long n, int* __restrict__ sums) {
  long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    long long idx = base + (long long)i * kScanThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  __shared__ int tot;
  block_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int* sums, int ntiles, int* out_total) {
  __shared__ int carry_s;
  __shared__ int tot;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += kScanThreads) {
    int idx = base + threadIdx.x;
    int v = idx < ntiles ? sums[idx] : 0;
    int ex = block_exclusive_scan(v, &tot);
    int carry = carry_s;
    if (idx < ntiles) sums[idx] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *out_total = carry_s;
}

__global__ void k_tile_scan(const int* in, int* out, long long n, const int* __restrict__ sums) {
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    long long idx = base + i;
    v[i] = idx < n ? in[idx] : 0;
    s += v[i];
  }
  __shared__ int tot;
  int ex = block_exclusive_scan(s, &tot) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    long long idx = base + i;
    if (idx < n) out[idx] = ex;
    ex += v[i];
  }
}

}  // namespace

size_t scan_ws_bytes(long long n) {
  long long tiles = (n + kScanTile - 1) / kScanTile;
  return carve_size(sizeof(int) * (size_t)(tiles + 1));
}

int scan_exclusive(const int* in, int* out, long long n, int* h_total, Carver& ws,
                   cudaStream_t st) {
  if (n < 0) return BILU_ERR_ARG;
  long long tiles = (n + kScanTile - 1) / kScanTile;
  int* sums = ws.take<int>((size_t)tiles + 1);
  if (!sums) return BILU_ERR_WORKSPACE;
  if (tiles > 0) {
    k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, sums);
    BILU_LAUNCH_CHECK();
  }
  // the tile-scan reads in[] before writing out[] within each tile, and the
  // total goes to out[n] only after every tile has been read
  k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, (int)tiles, sums + tiles);
  BILU_LAUNCH_CHECK();
  if (tiles > 0) {
    k_tile_scan<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
    BILU_LAUNCH_CHECK();
  }
  BILU_TRY_CUDA(cudaMemcpyAsync(out + n, sums + tiles, sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (h_total) {
    BILU_TRY_CUDA(cudaMemcpyAsync(h_total, sums + tiles, sizeof(int), cudaMemcpyDeviceToHost, st));
    BILU_TRY_CUDA(cudaStreamSynchronize(st));
  }
  return BILU_OK;
}

}  // namespace bilu
