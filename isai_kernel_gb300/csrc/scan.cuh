// Device-wide exclusive scan of int32 (three passes over 2048-item tiles).
#pragma once
#include "common.cuh"

namespace bilu {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Scratch bytes for scan_exclusive over n items.
size_t scan_ws_bytes(long long n);

// out[0..n) = exclusive prefix sums of in[0..n), out[n] = total.  in may
// alias out.  If h_total is non-null the total is copied to the host (this
// synchronises the stream).  Scratch comes from the carver.
int scan_exclusive(const int* in, int* out, long long n, int* h_total, Carver& ws,
                   cudaStream_t st);

}  // namespace bilu
