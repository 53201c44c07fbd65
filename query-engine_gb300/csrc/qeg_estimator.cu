// qeg_estimator.cu -- C ABI of the sketch + learned estimator, and the hook the
// GROUP BY uses to size its table (learned_estimate).
#include <dlfcn.h>

#include <algorithm>
#include <cstdlib>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <random>

#include "qeg_agg.h"
#include "qeg_mlp.h"

namespace qeg {

namespace {

Mlp& mlp_of(qeg_ctx* ctx) {
  if (!ctx->mlp) ctx->mlp = std::make_shared<Mlp>();
  return *ctx->mlp;
}

std::vector<float> predict_host(qeg_ctx* ctx, const float* feats, uint32_t n) {
  Mlp& m = mlp_of(ctx);
  m.ensure(ctx, static_cast<int>(n));
  QEG_CUDA(cudaMemcpyAsync(m.x.get(), feats, (size_t)n * kIn * 4, cudaMemcpyHostToDevice, ctx->stream));
  m.forward(m.x.get<float>(), static_cast<int>(n));
  std::vector<float> out((size_t)n * kOut);
  QEG_CUDA(cudaMemcpyAsync(out.data(), m.y.get(), out.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  return out;
}

}  // namespace

// The network predicts a correction to the classic estimate in log space:
// log2(1 + groups) = log2(1 + classic non-null groups) + 32 * out0.
double learned_groups(const SketchResult& s, float out0, double deadband) {
  const double classic = classic_estimate(s) - (s.null_frac > 0 ? 1.0 : 0.0);
  // The network's log2 correction, less a dead band of its own resolution:
  // small corrections are noise of the BF16 network where the classic
  // estimate is already close (a sample that covers most of the column),
  // while the large ones fix its underestimates on sparsely sampled skewed
  // columns. The band is chosen by the trainer on its training columns.
  double c = 32.0 * static_cast<double>(out0);
  c = c > deadband ? c - deadband : (c < -deadband ? c + deadband : 0.0);
  const double lg = std::log2(1.0 + std::max(classic, 0.0)) + c;
  return std::exp2(std::min(40.0, std::max(0.0, lg))) - 1.0;
}

bool learned_estimate(qeg_ctx* ctx, const SketchResult& s, double* groups, double* hot_share) {
  if (!ctx->mlp || !ctx->mlp->loaded) return false;
  const std::vector<float> y = predict_host(ctx, s.features, 1);
  double g = learned_groups(s, y[0], ctx->mlp->deadband);
  // Never below what the sample itself proves, never above the non-null rows.
  const double nonnull = s.total_rows * (1.0 - s.null_frac);
  g = std::max(g, s.hll_estimate * 0.95);
  g = std::min(g, std::max(nonnull, 1.0));
  *groups = g + (s.null_frac > 0 ? 1.0 : 0.0);
  *hot_share = std::min(1.0, std::max(0.0, static_cast<double>(y[1])));
  return true;
}

// Loads estimator weights from `path` (kParams little-endian float32, then
// optionally the correction's dead band as one more float32).
bool load_weights_file(qeg_ctx* ctx, const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::vector<float> p(kParams);
  f.read(reinterpret_cast<char*>(p.data()), kParams * 4);
  if (f.gcount() != kParams * 4) return false;
  float band = static_cast<float>(kCorrectionDeadband);
  f.read(reinterpret_cast<char*>(&band), 4);
  if (f.gcount() != 4 || !(band >= 0.0f && band <= 4.0f)) band = static_cast<float>(kCorrectionDeadband);
  Mlp& m = mlp_of(ctx);
  m.ensure(ctx, 1);
  m.set_master(p.data());
  m.deadband = band;
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  return true;
}

// Default weights: $QEG_ESTIMATOR_WEIGHTS, else estimator_weights.f32 next to
// libqeg.so. Without weights the classic estimator is used.
void load_default_weights(qeg_ctx* ctx) {
  const char* env = std::getenv("QEG_ESTIMATOR_WEIGHTS");
  if (env && *env) {
    load_weights_file(ctx, env);
    return;
  }
  Dl_info info{};
  if (dladdr(reinterpret_cast<void*>(&load_default_weights), &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const size_t slash = p.rfind('/');
    p = (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/estimator_weights.f32";
    load_weights_file(ctx, p);
  }
}

}  // namespace qeg

using namespace qeg;

extern "C" {

qeg_status qeg_sketch(qeg_ctx* ctx, const qeg_column* key, uint64_t sample_rows, float* features,
                      double* classic_groups, double* top_share) {
  qeg::NvtxRange nvtx_range("qeg_sketch");
  return guarded(ctx, [&] {
    require(ctx && key && features, "NULL argument");
    QEG_CUDA(cudaSetDevice(ctx->device));
    StagedCol s;
    stage_column(ctx, *key, s);
    SketchResult r;
    sketch_key_column(ctx, s.dev, nullptr, key->len, key->len, sample_rows ? sample_rows : (1u << 20), 0, r);
    for (int i = 0; i < kSketchFeatures; ++i) features[i] = r.features[i];
    if (classic_groups) *classic_groups = classic_estimate(r);
    if (top_share) *top_share = r.top_share[11];
  });
}

qeg_status qeg_sketch_batch(qeg_ctx* ctx, const qeg_column* key, uint32_t nqueries, const uint64_t* row_offsets,
                            uint64_t sample_rows, float* features, double* classic_groups) {
  return guarded(ctx, [&] {
    require(ctx && key && row_offsets && features, "NULL argument");
    require(nqueries >= 1 && row_offsets[nqueries] == key->len, "row offsets must cover the column");
    for (uint32_t q = 0; q < nqueries; ++q) require(row_offsets[q] <= row_offsets[q + 1], "row offsets must ascend");
    QEG_CUDA(cudaSetDevice(ctx->device));
    StagedCol s;
    stage_column(ctx, *key, s);
    std::vector<uint64_t> offs(row_offsets, row_offsets + nqueries + 1);
    DevBuf doffs((nqueries + 1) * 8, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(doffs.get(), offs.data(), (nqueries + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<SketchResult> r;
    batch_sketch(ctx, s.dev, doffs.get<uint64_t>(), offs, sample_rows ? sample_rows : (1u << 16), r);
    for (uint32_t q = 0; q < nqueries; ++q) {
      std::copy(r[q].features, r[q].features + kSketchFeatures, features + static_cast<size_t>(q) * kSketchFeatures);
      if (classic_groups) classic_groups[q] = classic_estimate(r[q]);
    }
  });
}

qeg_status qeg_estimator_init(qeg_ctx* ctx, uint64_t seed) {
  return guarded(ctx, [&] {
    require(ctx, "NULL ctx");
    QEG_CUDA(cudaSetDevice(ctx->device));
    Mlp& m = mlp_of(ctx);
    m.ensure(ctx, 1);
    m.init_random(seed);
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qeg_status qeg_estimator_set_weights(qeg_ctx* ctx, const float* params) {
  return guarded(ctx, [&] {
    require(ctx && params, "NULL argument");
    QEG_CUDA(cudaSetDevice(ctx->device));
    Mlp& m = mlp_of(ctx);
    m.ensure(ctx, 1);
    m.set_master(params);
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qeg_status qeg_estimator_set_deadband(qeg_ctx* ctx, double band) {
  return guarded(ctx, [&] {
    require(ctx != nullptr, "NULL argument");
    require(band >= 0.0 && band <= 4.0, "the dead band lies in [0, 4] (log2 units)");
    mlp_of(ctx).deadband = band;
  });
}

qeg_status qeg_estimator_get_deadband(qeg_ctx* ctx, double* band) {
  return guarded(ctx, [&] {
    require(ctx != nullptr && band != nullptr, "NULL argument");
    *band = ctx->mlp ? ctx->mlp->deadband : kCorrectionDeadband;
  });
}

qeg_status qeg_estimator_get_weights(qeg_ctx* ctx, float* params) {
  return guarded(ctx, [&] {
    require(ctx && params, "NULL argument");
    require(ctx->mlp && ctx->mlp->master.get(), "no estimator weights in this context");
    QEG_CUDA(cudaMemcpyAsync(params, ctx->mlp->master.get(), kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qeg_status qeg_estimator_predict(qeg_ctx* ctx, const float* features, uint32_t n, float* out) {
  return guarded(ctx, [&] {
    require(ctx && features && out, "NULL argument");
    require(ctx->mlp && ctx->mlp->master.get(), "no estimator weights in this context");
    QEG_CUDA(cudaSetDevice(ctx->device));
    if (n == 0) return;
    const std::vector<float> y = predict_host(ctx, features, n);
    std::memcpy(out, y.data(), y.size() * 4);
  });
}

qeg_status qeg_estimator_grad(qeg_ctx* ctx, const float* x, const float* t, uint32_t n, float* loss, float* grad) {
  return guarded(ctx, [&] {
    require(ctx && x && t && loss && grad, "NULL argument");
    require(ctx->mlp && ctx->mlp->master.get(), "no estimator weights in this context");
    require(n > 0, "empty batch");
    QEG_CUDA(cudaSetDevice(ctx->device));
    Mlp& m = mlp_of(ctx);
    m.ensure(ctx, static_cast<int>(n));
    QEG_CUDA(cudaMemcpyAsync(m.x.get(), x, (size_t)n * kIn * 4, cudaMemcpyHostToDevice, ctx->stream));
    QEG_CUDA(cudaMemcpyAsync(m.t.get(), t, (size_t)n * kOut * 4, cudaMemcpyHostToDevice, ctx->stream));
    *loss = m.loss_and_grad(m.x.get<float>(), m.t.get<float>(), static_cast<int>(n), true);
    QEG_CUDA(cudaMemcpyAsync(grad, m.grad.get(), kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qeg_status qeg_estimator_train(qeg_ctx* ctx, const float* x, const float* t, uint32_t n, uint32_t epochs,
                               uint32_t batch, float lr, uint64_t seed, float* final_loss) {
  return guarded(ctx, [&] {
    require(ctx && x && t && final_loss, "NULL argument");
    require(n > 0 && batch > 0, "empty training set");
    require(ctx->mlp && ctx->mlp->master.get(), "initialise or load the estimator first");
    QEG_CUDA(cudaSetDevice(ctx->device));
    Mlp& m = mlp_of(ctx);
    m.ensure(ctx, static_cast<int>(batch));
    DevBuf dx((size_t)n * kIn * 4, ctx->stream), dt((size_t)n * kOut * 4, ctx->stream);
    // Shuffled copies per epoch are made on the host; the data set is small.
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    std::mt19937_64 rng(seed);
    std::vector<float> sx((size_t)n * kIn), st((size_t)n * kOut);
    float l = 0;
    for (uint32_t e = 0; e < epochs; ++e) {
      std::shuffle(order.begin(), order.end(), rng);
      for (uint32_t i = 0; i < n; ++i) {
        std::memcpy(&sx[(size_t)i * kIn], x + (size_t)order[i] * kIn, kIn * 4);
        std::memcpy(&st[(size_t)i * kOut], t + (size_t)order[i] * kOut, kOut * 4);
      }
      QEG_CUDA(cudaMemcpyAsync(dx.get(), sx.data(), sx.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
      QEG_CUDA(cudaMemcpyAsync(dt.get(), st.data(), st.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
      double el = 0;
      uint32_t nb = 0;
      for (uint32_t b0 = 0; b0 < n; b0 += batch) {
        const int B = static_cast<int>(std::min(batch, n - b0));
        const bool last_epoch = (e + 1 == epochs);
        const float li = m.loss_and_grad(dx.get<float>() + (size_t)b0 * kIn, dt.get<float>() + (size_t)b0 * kOut, B,
                                         last_epoch);
        m.adam(lr);
        el += li;
        ++nb;
      }
      l = static_cast<float>(el / std::max<uint32_t>(nb, 1));
    }
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    *final_loss = l;
  });
}

}  // extern "C"
