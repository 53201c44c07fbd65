// qeg_scan.cu -- exclusive prefix sum (see qeg_scan.cuh).
#include "qeg_scan.cuh"

namespace qeg {

namespace {

// Block-wide inclusive scan of one value per thread (warp shuffles + smem).
__device__ __forceinline__ uint64_t block_inclusive_scan(uint64_t v, uint64_t* warp_sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sums[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += warp_sums[warp - 1];
  return v;
}

template <class T>
__device__ void scan_tile(const T* __restrict__ in, uint64_t n, uint64_t* __restrict__ out,
                          uint64_t* __restrict__ tile_sums) {
  __shared__ uint64_t warp_sums[32];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + static_cast<uint64_t>(threadIdx.x) * kScanItems;
  uint64_t v[kScanItems];
  uint64_t local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? static_cast<uint64_t>(in[base + i]) : 0;
    local += v[i];
  }
  const uint64_t incl = block_inclusive_scan(local, warp_sums);
  uint64_t run = incl - local;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == blockDim.x - 1) tile_sums[blockIdx.x] = incl;
}

}  // namespace

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const uint32_t* __restrict__ in, uint64_t n,
                                                                   uint64_t* __restrict__ out,
                                                                   uint64_t* __restrict__ tile_sums) {
  scan_tile<uint32_t>(in, n, out, tile_sums);
}

__global__ void __launch_bounds__(kScanThreads) scan_u64_tiles_kernel(const uint64_t* __restrict__ in, uint64_t n,
                                                                       uint64_t* __restrict__ out,
                                                                       uint64_t* __restrict__ tile_sums) {
  scan_tile<uint64_t>(in, n, out, tile_sums);
}

__global__ void scan_add_kernel(uint64_t* __restrict__ out, uint64_t n, const uint64_t* __restrict__ tile_offs) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] += tile_offs[i / kScanTile];
}

namespace {

// Exclusive scan of n uint64 tile totals in place (recursive).
void scan_u64_inplace(qeg_ctx* ctx, uint64_t* data, uint64_t n) {
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  DevBuf sums(tiles * 8 + 8, ctx->stream);
  DevBuf tmp(n * 8, ctx->stream);
  scan_u64_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(data, n, tmp.get<uint64_t>(),
                                                                          sums.get<uint64_t>());
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  if (tiles > 1) {
    scan_u64_inplace(ctx, sums.get<uint64_t>(), tiles);
    scan_add_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(tmp.get<uint64_t>(), n, sums.get<uint64_t>());
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  QEG_CUDA(cudaMemcpyAsync(data, tmp.get(), n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
}

}  // namespace

uint64_t exclusive_scan(qeg_ctx* ctx, const uint32_t* in, uint64_t n, uint64_t* out) {
  uint64_t total = 0;
  if (n == 0) {
    QEG_CUDA(cudaMemsetAsync(out, 0, 8, ctx->stream));
    return 0;
  }
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  DevBuf sums(tiles * 8, ctx->stream);
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(in, n, out, sums.get<uint64_t>());
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  // Tile totals -> exclusive offsets, then the grand total.
  DevBuf last(8, ctx->stream);
  QEG_CUDA(cudaMemcpyAsync(last.get(), sums.get<uint64_t>() + tiles - 1, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  scan_u64_inplace(ctx, sums.get<uint64_t>(), tiles);
  if (tiles > 1) {
    scan_add_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(out, n, sums.get<uint64_t>());
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  uint64_t last_off = 0, last_sum = 0;
  QEG_CUDA(cudaMemcpyAsync(&last_off, sums.get<uint64_t>() + tiles - 1, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaMemcpyAsync(&last_sum, last.get(), 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  total = last_off + last_sum;
  QEG_CUDA(cudaMemcpyAsync(out + n, &total, 8, cudaMemcpyHostToDevice, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  return total;
}

}  // namespace qeg
