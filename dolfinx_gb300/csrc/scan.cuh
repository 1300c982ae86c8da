// Device exclusive prefix sum of int64 counts, used by the device-side
// structure builders (sparsity pattern, sliced-ELL slice pointers).
// Three launches: per-block scans with the block totals, one block that
// scans the totals in order, and the add-back. Deterministic (integer).
#pragma once

#include "common.cuh"

namespace dfx
{
constexpr int kScanBlock = 1024;

// int64 scratch entries the scan of n values needs.
inline int64_t scan_scratch_count(int64_t n) { return (n + kScanBlock - 1) / kScanBlock + 1; }

// out[0..n] = exclusive prefix sums of in[0..n-1]; out[n] = total. out may
// alias in. scratch: scan_scratch_count(n) int64.
int exclusive_scan(const int64_t* in, int64_t* out, int64_t n, int64_t* scratch,
                   cudaStream_t s);
} // namespace dfx
