// qeg_mlp.h -- the estimator network (see qeg_mlp.cu).
#pragma once

#include "qeg_internal.h"

namespace qeg {

constexpr int kIn = 80;
constexpr int kHid = 64;
constexpr int kOut = 2;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kOut * kHid;
constexpr int kParams = kOffB3 + kOut;  // 9474

// Heavy-hitter count the second output refers to (share of rows carried by
// the this-many most frequent keys).
constexpr int kHotTopK = 2048;

// Dead band (log2 units) subtracted from the magnitude of the network's
// group-count correction when the weights carry none: train_estimator.py
// picks one on its training columns and stores it after the parameters in
// the weights file (Mlp::deadband).
constexpr double kCorrectionDeadband = 0.125;

struct Mlp {
  qeg_ctx* ctx = nullptr;
  DevBuf master, grad, m1, m2, wbf;         // params (fp32), grads, Adam moments, bf16 copy
  DevBuf x, t, z1, z2, y, dy, loss;         // batch buffers
  int cap_batch = 0;
  int step = 0;
  bool loaded = false;
  double deadband = kCorrectionDeadband;  // of the loaded weights

  void ensure(qeg_ctx* c, int max_batch);
  void set_master(const float* host);
  void init_random(uint64_t seed);
  void forward(const float* dx, int B);                                  // -> y
  float loss_and_grad(const float* dx, const float* dt, int B, bool want_loss);  // -> grad
  void adam(float lr);
};

}  // namespace qeg
