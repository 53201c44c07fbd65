// qeg_sketch.cu -- on-device sketch of a key column: HyperLogLog registers,
// a count-min sketch and heavy-hitter candidates over a strided sample. The
// sketch is the input of the distinct-group estimator that sizes the GROUP BY
// table and picks its strategy (the reference sizes by growth only,
// ops/hashtable.h:83-94; results never depend on the estimate, because an
// overflowing table is grown and the affected rows replayed).
#include <algorithm>
#include <cmath>

#include "qeg_agg.h"

namespace qeg {

namespace {

constexpr int kHllP = 14;
constexpr int kHllM = 1 << kHllP;
constexpr int kCmsDepth = 4;
constexpr int kCmsWidth = 2048;
constexpr int kCandLocal = 1024;
constexpr int kCandGlobal = 8192;
constexpr int kSampleBlock = 256;

struct SketchK {
  DevCol key;
  const uint32_t* sel;
  uint64_t nrows, len;
  uint64_t stride;   // rows between the starts of consecutive sample blocks
  uint64_t nblocks;  // sample blocks
  uint32_t* hll;     // kHllM
  uint32_t* cms;     // kCmsDepth * kCmsWidth
  unsigned long long* cand_key;  // kCandGlobal
  unsigned long long* cand_cnt;  // kCandGlobal
  unsigned long long* stats;     // [0] sampled rows, [1] sampled nulls
  uint32_t* err;
};

__device__ __forceinline__ uint64_t sketch_hash(uint64_t w) { return mix64(w ^ 0x243F6A8885A308D3ull); }

__global__ void __launch_bounds__(kSampleBlock) sketch_kernel(const SketchK P) {
  extern __shared__ uint32_t sh[];
  uint32_t* hll = sh;                                  // kHllM
  uint32_t* cms = hll + kHllM;                         // kCmsDepth * kCmsWidth
  unsigned long long* ck = reinterpret_cast<unsigned long long*>(cms + kCmsDepth * kCmsWidth);
  uint32_t* cc = reinterpret_cast<uint32_t*>(ck + kCandLocal);
  for (int i = threadIdx.x; i < kHllM + kCmsDepth * kCmsWidth; i += blockDim.x) sh[i] = 0;
  for (int i = threadIdx.x; i < kCandLocal; i += blockDim.x) {
    ck[i] = 0;
    cc[i] = 0;
  }
  __shared__ unsigned long long s_rows, s_nulls;
  if (threadIdx.x == 0) s_rows = s_nulls = 0;
  __syncthreads();
  unsigned long long rows = 0, nulls = 0;
  for (uint64_t b = blockIdx.x; b < P.nblocks; b += gridDim.x) {
    const uint64_t i = b * P.stride + threadIdx.x;
    if (i >= P.nrows) continue;
    uint64_t p = i;
    if (P.sel) {
      p = P.sel[i];
      if (p >= P.len) {
        atomicOr(P.err, kDevBadInput);
        continue;
      }
    }
    ++rows;
    if (!col_valid(P.key, p)) {
      ++nulls;
      continue;
    }
    const uint64_t w = key_word(P.key, p);
    const uint64_t h = sketch_hash(w);
    const uint32_t idx = static_cast<uint32_t>(h >> (64 - kHllP));
    const uint64_t rest = (h << kHllP) | (1ull << (kHllP - 1));
    const uint32_t rho = static_cast<uint32_t>(__clzll(static_cast<long long>(rest))) + 1;
    atomicMax(&hll[idx], rho);
#pragma unroll
    for (int d = 0; d < kCmsDepth; ++d) {
      const uint32_t c = static_cast<uint32_t>(mix64(h + 0x9E3779B97F4A7C15ull * (d + 1)) >> 40) & (kCmsWidth - 1);
      atomicAdd(&cms[d * kCmsWidth + c], 1u);
    }
    // First-come candidate table: a key seen early and often stays resident.
    uint32_t s = static_cast<uint32_t>(h) & (kCandLocal - 1);
    const unsigned long long kk = w + 1;  // 0 marks an empty candidate slot
    for (int t = 0; t < 8; ++t) {
      unsigned long long cur = ck[s];
      if (cur == 0) cur = atomicCAS(&ck[s], 0ull, kk);
      if (cur == 0 || cur == kk) {
        atomicAdd(&cc[s], 1u);
        break;
      }
      s = (s + 1) & (kCandLocal - 1);
    }
  }
  atomicAdd(&s_rows, rows);
  atomicAdd(&s_nulls, nulls);
  __syncthreads();
  for (int i = threadIdx.x; i < kHllM; i += blockDim.x)
    if (hll[i]) atomicMax(&P.hll[i], hll[i]);
  for (int i = threadIdx.x; i < kCmsDepth * kCmsWidth; i += blockDim.x)
    if (cms[i]) atomicAdd(&P.cms[i], cms[i]);
  for (int i = threadIdx.x; i < kCandLocal; i += blockDim.x) {
    if (cc[i] < 2) continue;
    const unsigned long long kk = ck[i];
    uint32_t s = static_cast<uint32_t>(mix64(kk)) & (kCandGlobal - 1);
    for (int t = 0; t < 32; ++t) {
      unsigned long long cur = atomicCAS(&P.cand_key[s], 0ull, kk);
      if (cur == 0 || cur == kk) {
        atomicAdd(&P.cand_cnt[s], static_cast<unsigned long long>(cc[i]));
        break;
      }
      s = (s + 1) & (kCandGlobal - 1);
    }
  }
  if (threadIdx.x == 0) {
    atomicAdd(&P.stats[0], s_rows);
    atomicAdd(&P.stats[1], s_nulls);
  }
}

// Exact counts of the sampled keys (the heavy-hitter candidates of a GROUP BY
// are the sample's most frequent keys): a linear-probing table of key words
// (0 = empty; key word 0 has a side row in the aggregation and is skipped)
// and counts, over the same strided sample blocks as sketch_kernel.
constexpr int kHeavyBins = 4096;

struct HeavyK {
  DevCol key;
  const uint32_t* sel;
  uint64_t nrows, len, stride, nblocks;
  unsigned long long* keys;  // [cap]
  unsigned int* cnt;         // [cap]
  uint64_t cap;              // power of two, >= 2 x the sampled rows
  unsigned int* hist;        // [kHeavyBins] keys per count (the last bin: >= kHeavyBins - 1)
  unsigned long long* out;   // [2 * out_cap] (key, count) of the kept keys
  unsigned int* nout;
  uint32_t out_cap, min_count;
  uint32_t* err;
};

__global__ void __launch_bounds__(kSampleBlock) heavy_count_kernel(const HeavyK P) {
  for (uint64_t b = blockIdx.x; b < P.nblocks; b += gridDim.x) {
    const uint64_t i = b * P.stride + threadIdx.x;
    if (i >= P.nrows) continue;
    uint64_t p = i;
    if (P.sel) {
      p = P.sel[i];
      if (p >= P.len) continue;  // reported by sketch_kernel
    }
    if (!col_valid(P.key, p)) continue;
    const uint64_t w = key_word(P.key, p);
    if (w == 0) continue;
    uint64_t s = mix64(w ^ 0x3C6EF372FE94F82Bull) & (P.cap - 1);
    for (uint64_t t = 0; t < P.cap; ++t) {  // at most half full: ends at a free slot
      unsigned long long cur = P.keys[s];
      if (cur == 0) cur = atomicCAS(P.keys + s, 0ull, static_cast<unsigned long long>(w));
      if (cur == 0 || cur == w) {
        atomicAdd(P.cnt + s, 1u);
        break;
      }
      s = (s + 1) & (P.cap - 1);
    }
  }
}

__global__ void heavy_hist_kernel(const HeavyK P) {
  __shared__ unsigned int h[kHeavyBins];
  for (int b = threadIdx.x; b < kHeavyBins; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < P.cap; s += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned int c = P.cnt[s];
    if (c) atomicAdd(&h[min(c, kHeavyBins - 1u)], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kHeavyBins; b += blockDim.x)
    if (h[b]) atomicAdd(P.hist + b, h[b]);
}

__global__ void heavy_compact_kernel(const HeavyK P) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < P.cap; s += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned int c = P.cnt[s];
    if (c < P.min_count) continue;
    const unsigned int o = atomicAdd(P.nout, 1u);
    if (o < P.out_cap) {
      P.out[2 * o] = P.keys[s];
      P.out[2 * o + 1] = c;
    }
  }
}

double hll_estimate(const std::vector<uint32_t>& regs) {
  const double m = kHllM;
  double sum = 0;
  int zeros = 0;
  for (uint32_t r : regs) {
    sum += std::ldexp(1.0, -static_cast<int>(r));
    if (r == 0) ++zeros;
  }
  const double alpha = 0.7213 / (1.0 + 1.079 / m);
  double e = alpha * m * m / sum;
  if (e <= 2.5 * m && zeros > 0) e = m * std::log(m / zeros);  // linear counting
  return e;
}

}  // namespace

void sketch_key_column(qeg_ctx* ctx, const DevCol& key, const uint32_t* sel, uint64_t nrows, uint64_t len,
                       uint64_t sample_target, int want_heavy, SketchResult& out) {
  out = SketchResult{};
  out.total_rows = static_cast<double>(nrows);
  const uint64_t target_blocks = std::max<uint64_t>(1, sample_target / kSampleBlock);
  uint64_t stride = kSampleBlock;
  uint64_t nblocks = (nrows + kSampleBlock - 1) / kSampleBlock;
  if (nblocks > target_blocks) {
    stride = ((nrows / target_blocks) / kSampleBlock) * kSampleBlock;
    if (stride < kSampleBlock) stride = kSampleBlock;
    nblocks = (nrows + stride - 1) / stride;
  }
  const size_t words = kHllM + kCmsDepth * kCmsWidth;
  DevBuf buf(words * 4 + kCandGlobal * 16 + 16, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(buf.get(), 0, buf.bytes(), ctx->stream));
  SketchK P{};
  P.key = key;
  P.sel = sel;
  P.nrows = nrows;
  P.len = len;
  P.stride = stride;
  P.nblocks = nblocks;
  P.hll = buf.get<uint32_t>();
  P.cms = P.hll + kHllM;
  P.cand_key = reinterpret_cast<unsigned long long*>(P.cms + kCmsDepth * kCmsWidth);
  P.cand_cnt = P.cand_key + kCandGlobal;
  P.stats = P.cand_cnt + kCandGlobal;
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());
  const size_t sb = words * 4 + kCandLocal * 12;
  raise_dynamic_smem(reinterpret_cast<const void*>(sketch_kernel), sb);
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(nblocks, ctx->sms * 2ull));
  if (nblocks > 0) {
    sketch_kernel<<<grid, kSampleBlock, sb, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  std::vector<uint32_t> regs(words);
  std::vector<unsigned long long> cand(2 * kCandGlobal + 2);
  QEG_CUDA(cudaMemcpyAsync(regs.data(), buf.get(), words * 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaMemcpyAsync(cand.data(), P.cand_key, cand.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  check_device_error(ctx);

  const std::vector<uint32_t> hll(regs.begin(), regs.begin() + kHllM);
  out.sample_rows = static_cast<double>(cand[2 * kCandGlobal]);
  const double nulls = static_cast<double>(cand[2 * kCandGlobal + 1]);
  out.null_frac = out.sample_rows > 0 ? nulls / out.sample_rows : 0;
  const double nonnull = out.sample_rows - nulls;
  out.hll_estimate = nonnull > 0 ? hll_estimate(hll) : 0;

  // Candidates ranked by their count-min estimate.
  auto cms_est = [&](uint64_t w) {
    const uint64_t h = mix64(w ^ 0x243F6A8885A308D3ull);
    uint32_t best = UINT32_MAX;
    for (int d = 0; d < kCmsDepth; ++d) {
      const uint32_t c = static_cast<uint32_t>(mix64(h + 0x9E3779B97F4A7C15ull * (d + 1)) >> 40) & (kCmsWidth - 1);
      best = std::min(best, regs[kHllM + d * kCmsWidth + c]);
    }
    return best;
  };
  std::vector<std::pair<uint32_t, uint64_t>> ranked;
  for (int i = 0; i < kCandGlobal; ++i)
    if (cand[i]) ranked.push_back({cms_est(cand[i] - 1), cand[i] - 1});
  std::sort(ranked.begin(), ranked.end(), [](auto& a, auto& b) { return a.first > b.first; });

  // Features: 64 normalised HLL register-value bins, then 16 frequency features.
  float* f = out.features;
  for (int i = 0; i < kSketchFeatures; ++i) f[i] = 0;
  for (uint32_t r : hll) f[std::min<uint32_t>(r, 63)] += 1.0f / kHllM;
  double cum = 0;
  size_t k = 0;
  for (int i = 0; i < 12; ++i) {
    const size_t upto = size_t(1) << i;
    while (k < ranked.size() && k < upto) cum += ranked[k++].first;
    out.top_share[i] = nonnull > 0 ? std::min(1.0, cum / nonnull) : 0;
  }
  for (int i = 0; i < 10; ++i) f[64 + i] = static_cast<float>(out.top_share[i]);
  double f2 = 0;
  for (int c = 0; c < kCmsWidth; ++c) {
    const double v = regs[kHllM + c];
    f2 += v * v;
  }
  f[74] = nonnull > 0 ? static_cast<float>(f2 / (nonnull * nonnull)) : 0.f;
  f[75] = static_cast<float>(std::log2(1.0 + out.sample_rows) / 32.0);
  f[76] = static_cast<float>(std::log2(1.0 + out.total_rows) / 32.0);
  f[77] = out.total_rows > 0 ? static_cast<float>(out.sample_rows / out.total_rows) : 1.f;
  f[78] = static_cast<float>(out.null_frac);
  f[79] = nonnull > 0 ? static_cast<float>(std::min(1.0, out.hll_estimate / nonnull)) : 0.f;

  if (want_heavy <= 0 || nblocks == 0) return;
  // Heavy hitters: the sample's want_heavy most frequent keys, by exact counts.
  HeavyK H{};
  H.key = key;
  H.sel = sel;
  H.nrows = nrows;
  H.len = len;
  H.stride = stride;
  H.nblocks = nblocks;
  H.cap = 1;
  while (H.cap < 2 * nblocks * kSampleBlock) H.cap <<= 1;
  H.out_cap = static_cast<uint32_t>(4 * want_heavy);
  const size_t head = H.cap * 12 + kHeavyBins * 4 + 16;
  DevBuf hb(head + static_cast<size_t>(H.out_cap) * 16, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(hb.get(), 0, head, ctx->stream));
  H.keys = hb.get<unsigned long long>();
  H.cnt = reinterpret_cast<unsigned int*>(H.keys + H.cap);
  H.hist = H.cnt + H.cap;
  H.nout = H.hist + kHeavyBins;
  H.out = reinterpret_cast<unsigned long long*>(hb.get<uint8_t>() + head);
  H.err = P.err;
  heavy_count_kernel<<<grid, kSampleBlock, 0, ctx->stream>>>(H);
  heavy_hist_kernel<<<grid_for(ctx, H.cap, 256, 4), 256, 0, ctx->stream>>>(H);
  std::vector<uint32_t> hist(kHeavyBins);
  QEG_CUDA(cudaMemcpyAsync(hist.data(), H.hist, kHeavyBins * 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  // The smallest count threshold that keeps at most out_cap keys (whole bins
  // only, so the kept set does not depend on the order of the atomics; the
  // top bin holds at most sample/(kHeavyBins-1) keys, fewer than out_cap).
  uint64_t kept = 0;
  uint32_t c = kHeavyBins - 1;
  while (c > 1 && kept + hist[c] <= H.out_cap) kept += hist[c--];
  if (c == 1 && kept + hist[1] <= H.out_cap) c = 0;
  H.min_count = c + 1;
  heavy_compact_kernel<<<grid_for(ctx, H.cap, 256, 4), 256, 0, ctx->stream>>>(H);
  ctx->launches += 3;
  QEG_CUDA(cudaGetLastError());
  uint32_t n = 0;
  QEG_CUDA(cudaMemcpyAsync(&n, H.nout, 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  n = std::min(n, H.out_cap);
  std::vector<unsigned long long> kc(2 * static_cast<size_t>(n));
  if (n) {
    QEG_CUDA(cudaMemcpyAsync(kc.data(), H.out, kc.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  std::vector<std::pair<uint64_t, uint64_t>> top(n);
  for (uint32_t i = 0; i < n; ++i) top[i] = {kc[2 * i + 1], kc[2 * i]};
  std::sort(top.begin(), top.end(), [](const auto& a, const auto& b) {
    return a.first != b.first ? a.first > b.first : a.second < b.second;
  });
  const size_t nh = std::min<size_t>(top.size(), static_cast<size_t>(want_heavy));
  for (size_t i = 0; i < nh; ++i) out.heavy.push_back(top[i].second);
}

// ---------------------------------------------------------------------------
// Batched sketch: one CTA per query of a batch (qeg_batch.cu). The CTA walks
// the query's whole sample (the same strided 256-row sample blocks as
// sketch_key_column), builds HyperLogLog registers, the count-min sketch and a
// first-come candidate table in shared memory, and computes the 80 features
// itself, so planning a batch costs one launch and one small copy back.
// ---------------------------------------------------------------------------
namespace {

constexpr int kBSThreads = 1024;
constexpr int kBSCand = 2048;

struct BatchSketchOut {
  float f[kSketchFeatures];
  double hll, rows, nulls;
  double top[12];
};

struct BatchSketchK {
  DevCol key;
  const uint64_t* offs;  // nq + 1 row offsets
  uint64_t sample_target;
  BatchSketchOut* out;
};

__global__ void __launch_bounds__(kBSThreads) batch_sketch_kernel(const BatchSketchK P) {
  extern __shared__ uint32_t sh[];
  uint32_t* hll = sh;                                                   // kHllM
  uint32_t* cms = hll + kHllM;                                          // kCmsDepth * kCmsWidth
  unsigned long long* ck = reinterpret_cast<unsigned long long*>(cms + kCmsDepth * kCmsWidth);  // kBSCand
  uint32_t* cc = reinterpret_cast<uint32_t*>(ck + kBSCand);             // kBSCand
  __shared__ unsigned long long s_rows, s_nulls;
  __shared__ uint32_t s_hist[64];
  __shared__ unsigned long long s_bucket[12];
  __shared__ double s_sum, s_f2;
  __shared__ uint32_t s_zeros;
  const int tid = threadIdx.x;
  for (int i = tid; i < kHllM + kCmsDepth * kCmsWidth; i += blockDim.x) sh[i] = 0;
  for (int i = tid; i < kBSCand; i += blockDim.x) {
    ck[i] = 0;
    cc[i] = 0;
  }
  if (tid < 64) s_hist[tid] = 0;
  if (tid < 12) s_bucket[tid] = 0;
  if (tid == 0) {
    s_rows = s_nulls = 0;
    s_sum = s_f2 = 0;
    s_zeros = 0;
  }
  __syncthreads();

  const uint64_t base = P.offs[blockIdx.x];
  const uint64_t n = P.offs[blockIdx.x + 1] - base;
  const uint64_t target_blocks = P.sample_target / kSampleBlock > 0 ? P.sample_target / kSampleBlock : 1;
  uint64_t stride = kSampleBlock;
  uint64_t nblocks = (n + kSampleBlock - 1) / kSampleBlock;
  if (nblocks > target_blocks) {
    stride = ((n / target_blocks) / kSampleBlock) * kSampleBlock;
    if (stride < kSampleBlock) stride = kSampleBlock;
    nblocks = (n + stride - 1) / stride;
  }
  unsigned long long rows = 0, nulls = 0;
  for (uint64_t j = tid; j < nblocks * kSampleBlock; j += blockDim.x) {
    const uint64_t i = (j / kSampleBlock) * stride + (j % kSampleBlock);
    if (i >= n) continue;
    const uint64_t p = base + i;
    ++rows;
    if (!col_valid(P.key, p)) {
      ++nulls;
      continue;
    }
    const uint64_t w = key_word(P.key, p);
    const uint64_t h = sketch_hash(w);
    const uint32_t idx = static_cast<uint32_t>(h >> (64 - kHllP));
    const uint64_t rest = (h << kHllP) | (1ull << (kHllP - 1));
    const uint32_t rho = static_cast<uint32_t>(__clzll(static_cast<long long>(rest))) + 1;
    atomicMax(&hll[idx], rho);
#pragma unroll
    for (int d = 0; d < kCmsDepth; ++d) {
      const uint32_t c = static_cast<uint32_t>(mix64(h + 0x9E3779B97F4A7C15ull * (d + 1)) >> 40) & (kCmsWidth - 1);
      atomicAdd(&cms[d * kCmsWidth + c], 1u);
    }
    uint32_t s = static_cast<uint32_t>(h) & (kBSCand - 1);
    const unsigned long long kk = w + 1;
    for (int t = 0; t < 8; ++t) {
      unsigned long long cur = ck[s];
      if (cur == 0) cur = atomicCAS(&ck[s], 0ull, kk);
      if (cur == 0 || cur == kk) {
        atomicAdd(&cc[s], 1u);
        break;
      }
      s = (s + 1) & (kBSCand - 1);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    rows += __shfl_down_sync(0xffffffffu, rows, o);
    nulls += __shfl_down_sync(0xffffffffu, nulls, o);
  }
  if ((tid & 31) == 0) {
    atomicAdd(&s_rows, rows);
    atomicAdd(&s_nulls, nulls);
  }
  __syncthreads();

  // Register histogram, HyperLogLog sum and zero count, F2 of CMS row 0.
  double hsum = 0, f2 = 0;
  uint32_t zeros = 0;
  for (int i = tid; i < kHllM; i += blockDim.x) {
    const uint32_t r = hll[i];
    atomicAdd(&s_hist[r < 63 ? r : 63], 1u);
    hsum += ldexp(1.0, -static_cast<int>(r));
    zeros += r == 0;
  }
  for (int c = tid; c < kCmsWidth; c += blockDim.x) {
    const double v = cms[c];
    f2 += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    hsum += __shfl_down_sync(0xffffffffu, hsum, o);
    f2 += __shfl_down_sync(0xffffffffu, f2, o);
    zeros += __shfl_down_sync(0xffffffffu, zeros, o);
  }
  if ((tid & 31) == 0) {
    atomicAdd(&s_sum, hsum);
    atomicAdd(&s_f2, f2);
    atomicAdd(&s_zeros, zeros);
  }
  // Count-min estimate of every candidate seen at least twice (0 otherwise),
  // into cc, then a descending bitonic sort of those estimates.
  for (int i = tid; i < kBSCand; i += blockDim.x) {
    uint32_t est = 0;
    if (cc[i] >= 2) {
      const uint64_t h = sketch_hash(ck[i] - 1);
      est = UINT32_MAX;
#pragma unroll
      for (int d = 0; d < kCmsDepth; ++d) {
        const uint32_t c = static_cast<uint32_t>(mix64(h + 0x9E3779B97F4A7C15ull * (d + 1)) >> 40) & (kCmsWidth - 1);
        est = min(est, cms[d * kCmsWidth + c]);
      }
    }
    cc[i] = est;
  }
  __syncthreads();
  for (int k = 2; k <= kBSCand; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < kBSCand; i += blockDim.x) {
        const int x = i ^ j;
        if (x > i) {
          const uint32_t a = cc[i], b = cc[x];
          if (((i & k) == 0) ? (a < b) : (a > b)) {
            cc[i] = b;
            cc[x] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  // Sum of the top 2^b estimates: the estimate at sorted position j counts
  // toward every prefix longer than j, i.e. bucket bitlength(j) and above.
  for (int j = tid; j < kBSCand; j += blockDim.x) {
    const int b = j == 0 ? 0 : 32 - __clz(j);
    if (b < 12 && cc[j]) atomicAdd(&s_bucket[b], static_cast<unsigned long long>(cc[j]));
  }
  __syncthreads();
  if (tid == 0) {
    BatchSketchOut& o = P.out[blockIdx.x];
    const double srows = static_cast<double>(s_rows), snulls = static_cast<double>(s_nulls);
    const double nonnull = srows - snulls;
    const double m = kHllM;
    double e = (0.7213 / (1.0 + 1.079 / m)) * m * m / s_sum;
    if (e <= 2.5 * m && s_zeros > 0) e = m * log(m / s_zeros);
    o.hll = nonnull > 0 ? e : 0;
    o.rows = srows;
    o.nulls = snulls;
    for (int i = 0; i < kSketchFeatures; ++i) o.f[i] = 0;
    for (int r = 0; r < 64; ++r) o.f[r] = static_cast<float>(s_hist[r]) / kHllM;
    double cum = 0;
    for (int i = 0; i < 12; ++i) {
      cum += static_cast<double>(s_bucket[i]);
      o.top[i] = nonnull > 0 ? fmin(1.0, cum / nonnull) : 0;
    }
    for (int i = 0; i < 10; ++i) o.f[64 + i] = static_cast<float>(o.top[i]);
    o.f[74] = nonnull > 0 ? static_cast<float>(s_f2 / (nonnull * nonnull)) : 0.f;
    o.f[75] = static_cast<float>(log2(1.0 + srows) / 32.0);
    o.f[76] = static_cast<float>(log2(1.0 + static_cast<double>(n)) / 32.0);
    o.f[77] = n > 0 ? static_cast<float>(srows / static_cast<double>(n)) : 1.f;
    o.f[78] = srows > 0 ? static_cast<float>(snulls / srows) : 0.f;
    o.f[79] = nonnull > 0 ? static_cast<float>(fmin(1.0, o.hll / nonnull)) : 0.f;
  }
}

}  // namespace

void batch_sketch(qeg_ctx* ctx, const DevCol& key, const uint64_t* d_offsets, const std::vector<uint64_t>& offsets,
                  uint64_t sample_target, std::vector<SketchResult>& out) {
  const uint32_t nq = static_cast<uint32_t>(offsets.size() - 1);
  out.assign(nq, SketchResult{});
  if (nq == 0) return;
  DevBuf buf(static_cast<size_t>(nq) * sizeof(BatchSketchOut), ctx->stream);
  BatchSketchK P{};
  P.key = key;
  P.offs = d_offsets;
  P.sample_target = sample_target;
  P.out = buf.get<BatchSketchOut>();
  const size_t sb = (kHllM + kCmsDepth * kCmsWidth) * 4 + kBSCand * 12;
  raise_dynamic_smem(reinterpret_cast<const void*>(batch_sketch_kernel), sb);
  batch_sketch_kernel<<<nq, kBSThreads, sb, ctx->stream>>>(P);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  std::vector<BatchSketchOut> h(nq);
  QEG_CUDA(cudaMemcpyAsync(h.data(), buf.get(), nq * sizeof(BatchSketchOut), cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  check_device_error(ctx);
  for (uint32_t q = 0; q < nq; ++q) {
    SketchResult& r = out[q];
    std::copy(h[q].f, h[q].f + kSketchFeatures, r.features);
    r.hll_estimate = h[q].hll;
    r.sample_rows = h[q].rows;
    r.total_rows = static_cast<double>(offsets[q + 1] - offsets[q]);
    r.null_frac = h[q].rows > 0 ? h[q].nulls / h[q].rows : 0;
    for (int i = 0; i < 12; ++i) r.top_share[i] = h[q].top[i];
  }
}

double classic_estimate(const SketchResult& s) {
  // Distinct count of the sample from HyperLogLog, scaled to the population by
  // inverting E[d_sample] = D (1 - (1 - 1/D)^m) (a uniform-frequency model),
  // plus the NULL group. Skewed data breaks the uniform model; that is what the
  // learned estimator corrects.
  const double nonnull_rows = s.total_rows * (1.0 - s.null_frac);
  const double m = s.sample_rows * (1.0 - s.null_frac);
  double d = s.hll_estimate;
  if (m <= 0) return s.null_frac > 0 ? 1.0 : 0.0;
  if (s.sample_rows < s.total_rows && d > 0) {
    if (d >= m * 0.999) {
      d = nonnull_rows;  // every sampled row distinct: assume all distinct
    } else {
      double lo = d, hi = std::max(d, nonnull_rows);
      for (int it = 0; it < 100; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double e = mid * (1.0 - std::exp(m * std::log1p(-1.0 / std::max(mid, 1.0 + 1e-9))));
        if (e < d) lo = mid;
        else hi = mid;
      }
      d = 0.5 * (lo + hi);
    }
  }
  d = std::min(d, nonnull_rows);
  return d + (s.null_frac > 0 ? 1.0 : 0.0);
}

double AggState::estimate_groups(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len,
                                 const uint32_t* dsel) {
  if (mode != 1 || nrows == 0) {
    // Composite keys: bounded by the row count (grown on overflow).
    return static_cast<double>(std::min<uint64_t>(std::max<uint64_t>(nrows, 1), 1ull << 22));
  }
  SketchResult s;
  // Heavy hitters are wanted for preloading (hot_keys > 0) and by the
  // partitioned strategy, which the estimate may choose.
  const bool part_possible = (cfg.strategy == QEG_AGG_AUTO || cfg.strategy == QEG_AGG_PARTITIONED) &&
                             part_eligible(staged);
  const int want_heavy = (cfg.hot_keys > 0 || part_possible) ? 4096 : 0;
  if (packed) {
    // A packed window's (partition key, bucket) words are clustered by time,
    // which a strided sample cannot extrapolate: estimate the partition key's
    // distinct count instead and multiply by the buckets the time range
    // spans (at most one group per row).
    sketch_key_column(ctx, staged[keys[0]].dev, dsel, nrows, len, 1u << 20, 0, s);
    double keys_est = 0, share = 0;
    if (!learned_estimate(ctx, s, &keys_est, &share)) keys_est = classic_estimate(s);
    hot_share = 0;
    const double buckets = static_cast<double>(pack_qmax - pack_qmin + 1);
    return std::max(1.0, std::min(static_cast<double>(nrows), std::max(keys_est, 1.0) * buckets));
  }
  sketch_key_column(ctx, key_col(staged, 0), dsel, nrows, len, 1u << 20, want_heavy, s);
  double groups = 0, share = 0;
  if (learned_estimate(ctx, s, &groups, &share)) {
    hot_share = share;
  } else {
    groups = classic_estimate(s);
    hot_share = s.top_share[11];
  }
  heavy_candidates = s.heavy;
  return std::max(groups, 1.0);
}

}  // namespace qeg
