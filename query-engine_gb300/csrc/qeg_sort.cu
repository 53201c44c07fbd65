// qeg_sort.cu -- stable LSD radix sort (8-bit digits) of (hi, lo, val) items.
//
// One pass per digit: a per-tile digit histogram (digit-major, tile-minor), an
// exclusive scan of it (qeg_scan), then a scatter in which each tile ranks its
// items stably: each warp walks its own contiguous eighth of the tile in
// 32-item chunks, lanes with equal digits rank among themselves with
// __match_any_sync, and per-warp digit counters (prefixed over the warps of
// the tile) keep the input order across chunks and warps.
#include "qeg_scan.cuh"
#include "qeg_sort.h"

namespace qeg {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortChunks = 16;                             // 32-item chunks per warp
constexpr int kSortTile = kSortThreads * kSortChunks;       // items per tile
constexpr int kWarpSpan = kSortTile / kSortWarps;           // items per warp
constexpr int kRadix = 256;
static_assert(kSortThreads == kRadix, "one thread per digit in the histogram and prefix steps");

struct PassK {
  SortItems in, out;
  uint64_t n;
  uint32_t ntiles;
  int use_hi, shift;
  uint32_t* hist;       // [kRadix][ntiles]
  const uint64_t* off;  // exclusive scan of hist
};

__device__ __forceinline__ uint32_t digit_of(const PassK& P, uint64_t i) {
  return P.use_hi ? ((P.in.hi[i] >> P.shift) & (kRadix - 1))
                  : static_cast<uint32_t>((P.in.lo[i] >> P.shift) & (kRadix - 1));
}

__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const PassK P) {
  __shared__ uint32_t cnt[kRadix];
  for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(tile) * kSortTile;
    for (int k = 0; k < kSortChunks; ++k) {
      const uint64_t i = base + static_cast<uint64_t>(k) * kSortThreads + threadIdx.x;
      if (i < P.n) atomicAdd(&cnt[digit_of(P, i)], 1u);
    }
    __syncthreads();
    P.hist[static_cast<uint64_t>(threadIdx.x) * P.ntiles + tile] = cnt[threadIdx.x];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const PassK P) {
  __shared__ uint32_t pos[kSortWarps][kRadix];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    for (int d = threadIdx.x; d < kSortWarps * kRadix; d += kSortThreads) (&pos[0][0])[d] = 0;
    __syncthreads();
    const uint64_t wbase = static_cast<uint64_t>(tile) * kSortTile + static_cast<uint64_t>(warp) * kWarpSpan;
    // Digit counts of this warp's items.
    for (int c = 0; c < kSortChunks; ++c) {
      const uint64_t i = wbase + c * 32 + lane;
      const uint32_t d = i < P.n ? digit_of(P, i) : kRadix;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      if (d < kRadix && (peers & lt) == 0) pos[warp][d] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // Global start of each (warp, digit) run: the tile's scanned offset plus
    // the counts of the earlier warps.
    {
      const int d = threadIdx.x;
      uint64_t run = P.off[static_cast<uint64_t>(d) * P.ntiles + tile];
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = pos[w][d];
        pos[w][d] = static_cast<uint32_t>(run);
        run += c;
      }
    }
    __syncthreads();
    for (int c = 0; c < kSortChunks; ++c) {
      const uint64_t i = wbase + c * 32 + lane;
      const bool ok = i < P.n;
      const uint32_t d = ok ? digit_of(P, i) : kRadix;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      uint32_t at = 0;
      if (ok) at = pos[warp][d] + __popc(peers & lt);
      __syncwarp();
      if (ok && (peers & lt) == 0) pos[warp][d] += __popc(peers);
      __syncwarp();
      if (ok) {
        P.out.lo[at] = P.in.lo[i];
        P.out.hi[at] = P.in.hi[i];
        P.out.val[at] = P.in.val[i];
      }
    }
    __syncthreads();
  }
}

}  // namespace

SortItems radix_sort_items(qeg_ctx* ctx, SortItems a, SortItems b, uint64_t n, int lo_bits, int hi_bits) {
  require(n < 0xffffffffull, "radix sort holds at most 2^32-2 items");
  if (n <= 1) return a;
  PassK P{};
  P.n = n;
  P.ntiles = static_cast<uint32_t>((n + kSortTile - 1) / kSortTile);
  const uint64_t nh = static_cast<uint64_t>(kRadix) * P.ntiles;
  DevBuf hist(nh * 4, ctx->stream), off((nh + 1) * 8, ctx->stream);
  P.hist = hist.get<uint32_t>();
  P.off = off.get<uint64_t>();
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(P.ntiles, static_cast<uint64_t>(ctx->sms) * 8));
  SortItems src = a, dst = b;
  auto pass = [&](int use_hi, int shift) {
    P.in = src;
    P.out = dst;
    P.use_hi = use_hi;
    P.shift = shift;
    radix_hist_kernel<<<grid, kSortThreads, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    exclusive_scan(ctx, P.hist, nh, off.get<uint64_t>());
    radix_scatter_kernel<<<grid, kSortThreads, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    std::swap(src, dst);
  };
  for (int s = 0; s < lo_bits; s += 8) pass(0, s);
  for (int s = 0; s < hi_bits; s += 8) pass(1, s);
  return src;
}

}  // namespace qeg
