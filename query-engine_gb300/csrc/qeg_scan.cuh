// qeg_scan.cuh -- device exclusive prefix sum over uint32 counts into uint64
// offsets (three phases: per-tile scan, scan of tile totals, add-back).
#pragma once

#include "qeg_internal.h"

namespace qeg {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void scan_tiles_kernel(const uint32_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ out,
                                  uint64_t* __restrict__ tile_sums);
__global__ void scan_add_kernel(uint64_t* __restrict__ out, uint64_t n, const uint64_t* __restrict__ tile_offs);
__global__ void scan_u64_tiles_kernel(const uint64_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ out,
                                      uint64_t* __restrict__ tile_sums);

// out[i] = sum(in[0..i)), out[n] = total. `out` holds n+1 entries. Returns the
// total (synchronises the stream).
uint64_t exclusive_scan(qeg_ctx* ctx, const uint32_t* in, uint64_t n, uint64_t* out);

}  // namespace qeg
