// qeg_mlp.cu -- the learned cardinality / skew estimator: an MLP 80 -> 64 -> 64
// -> 2 with ReLU hidden layers, BF16 weights and FP32 accumulation, with
// hand-written forward, backward and Adam kernels.
//
// Inputs are the 80 sketch features of a key column (qeg_sketch.cu: 64 HLL
// register-value bins + 16 frequency features). Outputs:
//   y0 = log2(1 + distinct groups) / 32
//   y1 = share of rows carried by the 2048 most frequent keys
// The prediction only sizes tables and picks strategies; results never depend
// on it (an undersized table grows and replays, qeg_agg.cu).
//
// Parameter layout (fp32 master copy, and a bf16 copy used by the kernels):
//   W1[64][80] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
#include <cuda_bf16.h>

#include <cmath>
#include <random>

#include "qeg_mlp.h"

namespace qeg {

namespace {

constexpr int kTile = 32;  // samples per block

__device__ __forceinline__ float bf(const __nv_bfloat16* p, int i) { return __bfloat162float(p[i]); }

struct Acts {  // per-sample activations kept for the backward pass
  float* z1;  // [B][H]
  float* z2;  // [B][H]
  float* y;   // [B][OUT]
};

// Forward pass: one block of kHid threads per kTile samples.
__global__ void __launch_bounds__(kHid) mlp_forward_kernel(const __nv_bfloat16* __restrict__ w, const float* __restrict__ x,
                                                          int B, Acts A) {
  __shared__ float sx[kTile][kIn];
  __shared__ float sh1[kTile][kHid];
  __shared__ float sh2[kTile][kHid];
  const int h = threadIdx.x;
  const int s0 = blockIdx.x * kTile;
  for (int i = h; i < kTile * kIn; i += kHid) {
    const int s = i / kIn, f = i % kIn;
    sx[s][f] = (s0 + s < B) ? x[(size_t)(s0 + s) * kIn + f] : 0.f;
  }
  __syncthreads();
  const __nv_bfloat16* W1 = w + kOffW1;
  const __nv_bfloat16* W2 = w + kOffW2;
  const __nv_bfloat16* W3 = w + kOffW3;
  float wr[kIn];
#pragma unroll
  for (int f = 0; f < kIn; ++f) wr[f] = bf(W1, h * kIn + f);
  const float b1 = bf(w, kOffB1 + h);
  for (int s = 0; s < kTile; ++s) {
    float acc = b1;
#pragma unroll
    for (int f = 0; f < kIn; ++f) acc = fmaf(sx[s][f], wr[f], acc);
    sh1[s][h] = fmaxf(acc, 0.f);
    if (s0 + s < B) A.z1[(size_t)(s0 + s) * kHid + h] = acc;
  }
  __syncthreads();
  float wr2[kHid];
#pragma unroll
  for (int k = 0; k < kHid; ++k) wr2[k] = bf(W2, h * kHid + k);
  const float b2 = bf(w, kOffB2 + h);
  for (int s = 0; s < kTile; ++s) {
    float acc = b2;
#pragma unroll
    for (int k = 0; k < kHid; ++k) acc = fmaf(sh1[s][k], wr2[k], acc);
    sh2[s][h] = fmaxf(acc, 0.f);
    if (s0 + s < B) A.z2[(size_t)(s0 + s) * kHid + h] = acc;
  }
  __syncthreads();
  // Output layer: thread (s, o) for s < kTile, o < kOut.
  for (int t = h; t < kTile * kOut; t += kHid) {
    const int s = t / kOut, o = t % kOut;
    float acc = bf(w, kOffB3 + o);
    for (int k = 0; k < kHid; ++k) acc = fmaf(sh2[s][k], bf(W3, o * kHid + k), acc);
    if (s0 + s < B) A.y[(size_t)(s0 + s) * kOut + o] = acc;
  }
}

// Loss (mean squared error over batch and outputs) and its gradient dY.
__global__ void mlp_loss_kernel(const float* __restrict__ y, const float* __restrict__ t, int B, float* __restrict__ dy,
                                float* __restrict__ loss) {
  float l = 0;
  const float scale = 1.f / (static_cast<float>(B) * kOut);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * kOut; i += gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = 2.f * d * scale;
    l += d * d * scale;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Backward pass: one block of kHid threads per kTile samples; per-block partial
// weight gradients are added into `g` (fp32, master layout) with atomics.
__global__ void __launch_bounds__(kHid) mlp_backward_kernel(const __nv_bfloat16* __restrict__ w,
                                                           const float* __restrict__ x, int B, Acts A,
                                                           const float* __restrict__ dy, float* __restrict__ g) {
  __shared__ float sx[kTile][kIn];
  __shared__ float sh1[kTile][kHid];
  __shared__ float sh2[kTile][kHid];
  __shared__ float sdz2[kTile][kHid];
  __shared__ float sdz1[kTile][kHid];
  __shared__ float sdy[kTile][kOut];
  const int h = threadIdx.x;
  const int s0 = blockIdx.x * kTile;
  for (int i = h; i < kTile * kIn; i += kHid) {
    const int s = i / kIn, f = i % kIn;
    sx[s][f] = (s0 + s < B) ? x[(size_t)(s0 + s) * kIn + f] : 0.f;
  }
  for (int s = 0; s < kTile; ++s) {
    const bool ok = s0 + s < B;
    sh1[s][h] = ok ? fmaxf(A.z1[(size_t)(s0 + s) * kHid + h], 0.f) : 0.f;
    sh2[s][h] = ok ? fmaxf(A.z2[(size_t)(s0 + s) * kHid + h], 0.f) : 0.f;
  }
  for (int t = h; t < kTile * kOut; t += kHid) {
    const int s = t / kOut, o = t % kOut;
    sdy[s][o] = (s0 + s < B) ? dy[(size_t)(s0 + s) * kOut + o] : 0.f;
  }
  __syncthreads();
  const __nv_bfloat16* W2 = w + kOffW2;
  const __nv_bfloat16* W3 = w + kOffW3;
  // dZ2[s][h] = (sum_o dY[s][o] W3[o][h]) * relu'(z2)
  for (int s = 0; s < kTile; ++s) {
    float d = 0;
    for (int o = 0; o < kOut; ++o) d = fmaf(sdy[s][o], bf(W3, o * kHid + h), d);
    sdz2[s][h] = sh2[s][h] > 0.f ? d : 0.f;
  }
  __syncthreads();
  // dZ1[s][k=h] = (sum_j dZ2[s][j] W2[j][h]) * relu'(z1)
  for (int s = 0; s < kTile; ++s) {
    float d = 0;
    for (int j = 0; j < kHid; ++j) d = fmaf(sdz2[s][j], bf(W2, j * kHid + h), d);
    sdz1[s][h] = sh1[s][h] > 0.f ? d : 0.f;
  }
  __syncthreads();
  // Weight gradients, thread h owns row h of W1/W2 and the matching biases.
  for (int f = 0; f < kIn; ++f) {
    float a = 0;
    for (int s = 0; s < kTile; ++s) a = fmaf(sdz1[s][h], sx[s][f], a);
    atomicAdd(g + kOffW1 + h * kIn + f, a);
  }
  for (int k = 0; k < kHid; ++k) {
    float a = 0;
    for (int s = 0; s < kTile; ++s) a = fmaf(sdz2[s][h], sh1[s][k], a);
    atomicAdd(g + kOffW2 + h * kHid + k, a);
  }
  float gb1 = 0, gb2 = 0;
  for (int s = 0; s < kTile; ++s) {
    gb1 += sdz1[s][h];
    gb2 += sdz2[s][h];
  }
  atomicAdd(g + kOffB1 + h, gb1);
  atomicAdd(g + kOffB2 + h, gb2);
  for (int o = 0; o < kOut; ++o) {
    float a = 0;
    for (int s = 0; s < kTile; ++s) a = fmaf(sdy[s][o], sh2[s][h], a);
    atomicAdd(g + kOffW3 + o * kHid + h, a);
  }
  if (h < kOut) {
    float a = 0;
    for (int s = 0; s < kTile; ++s) a += sdy[s][h];
    atomicAdd(g + kOffB3 + h, a);
  }
}

// Adam step on the fp32 master weights; refreshes the bf16 copy.
__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                                float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] -= upd;
    wb[i] = __float2bfloat16(p[i]);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ p, __nv_bfloat16* __restrict__ wb, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) wb[i] = __float2bfloat16(p[i]);
}

}  // namespace

void Mlp::ensure(qeg_ctx* c, int max_batch) {
  ctx = c;
  if (!master.get()) {
    master.alloc(kParams * 4, ctx->stream);
    grad.alloc(kParams * 4, ctx->stream);
    m1.alloc(kParams * 4, ctx->stream);
    m2.alloc(kParams * 4, ctx->stream);
    wbf.alloc(kParams * 2, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(m1.get(), 0, kParams * 4, ctx->stream));
    QEG_CUDA(cudaMemsetAsync(m2.get(), 0, kParams * 4, ctx->stream));
  }
  if (max_batch > cap_batch) {
    cap_batch = max_batch;
    x.alloc((size_t)max_batch * kIn * 4, ctx->stream);
    t.alloc((size_t)max_batch * kOut * 4, ctx->stream);
    z1.alloc((size_t)max_batch * kHid * 4, ctx->stream);
    z2.alloc((size_t)max_batch * kHid * 4, ctx->stream);
    y.alloc((size_t)max_batch * kOut * 4, ctx->stream);
    dy.alloc((size_t)max_batch * kOut * 4, ctx->stream);
    loss.alloc(4, ctx->stream);
  }
}

void Mlp::set_master(const float* host) {
  QEG_CUDA(cudaMemcpyAsync(master.get(), host, kParams * 4, cudaMemcpyHostToDevice, ctx->stream));
  to_bf16_kernel<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(master.get<float>(), wbf.get<__nv_bfloat16>(),
                                                                 kParams);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  loaded = true;
}

void Mlp::init_random(uint64_t seed) {
  std::mt19937_64 rng(seed);
  std::vector<float> p(kParams, 0.f);
  auto fill = [&](int off, int fan_in, int n) {
    std::normal_distribution<float> d(0.f, std::sqrt(2.f / fan_in));
    for (int i = 0; i < n; ++i) p[off + i] = d(rng);
  };
  fill(kOffW1, kIn, kHid * kIn);
  fill(kOffW2, kHid, kHid * kHid);
  fill(kOffW3, kHid, kOut * kHid);
  set_master(p.data());
  QEG_CUDA(cudaMemsetAsync(m1.get(), 0, kParams * 4, ctx->stream));
  QEG_CUDA(cudaMemsetAsync(m2.get(), 0, kParams * 4, ctx->stream));
  step = 0;
}

void Mlp::forward(const float* dx, int B) {
  Acts A{z1.get<float>(), z2.get<float>(), y.get<float>()};
  mlp_forward_kernel<<<(B + kTile - 1) / kTile, kHid, 0, ctx->stream>>>(wbf.get<__nv_bfloat16>(), dx, B, A);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
}

float Mlp::loss_and_grad(const float* dx, const float* dt, int B, bool want_loss) {
  QEG_CUDA(cudaMemsetAsync(grad.get(), 0, kParams * 4, ctx->stream));
  QEG_CUDA(cudaMemsetAsync(loss.get(), 0, 4, ctx->stream));
  forward(dx, B);
  mlp_loss_kernel<<<std::max(1, std::min(64, (B * kOut + 255) / 256)), 256, 0, ctx->stream>>>(
      y.get<float>(), dt, B, dy.get<float>(), loss.get<float>());
  ctx->launches++;
  Acts A{z1.get<float>(), z2.get<float>(), y.get<float>()};
  mlp_backward_kernel<<<(B + kTile - 1) / kTile, kHid, 0, ctx->stream>>>(wbf.get<__nv_bfloat16>(), dx, B, A,
                                                                       dy.get<float>(), grad.get<float>());
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  float l = 0;
  if (want_loss) {
    QEG_CUDA(cudaMemcpyAsync(&l, loss.get(), 4, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return l;
}

void Mlp::adam(float lr) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, static_cast<float>(step));
  const float c2 = 1.f - std::pow(b2, static_cast<float>(step));
  mlp_adam_kernel<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(master.get<float>(), grad.get<float>(),
                                                                  m1.get<float>(), m2.get<float>(),
                                                                  wbf.get<__nv_bfloat16>(), lr, b1, b2, 1e-8f, c1, c2);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
}

}  // namespace qeg
