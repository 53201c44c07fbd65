// qeg_ctx.cu -- context, staging of host inputs, result fetch, device error word.
#include <mutex>

#include "qeg_internal.h"

thread_local std::string g_qeg_tls_err;

namespace qeg {

namespace {

// Packs one byte per row (1 = valid) into 64-bit validity words, LSB-first
// (core/validity.h:21-40). Padding bits of the last word are set to 1, the
// reference's canonical representation (core/validity.h:53-58).
__global__ void pack_validity_kernel(const uint8_t* __restrict__ valid, uint64_t n,
                                     uint64_t* __restrict__ words, uint32_t* __restrict__ any_null) {
  const uint64_t nw = (n + 63) / 64;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t bits = ~0ull;
    const uint64_t base = w * 64;
    for (int b = 0; b < 64; ++b) {
      const uint64_t r = base + b;
      if (r < n && !valid[r]) bits &= ~(1ull << b);
    }
    words[w] = bits;
    if (bits != ~0ull) atomicOr(any_null, 1u);
  }
}

// One thread waits, with the bounded wait every composite-key table uses, on
// a row state word that is claimed and never published.
__global__ void stuck_claim_kernel(uint64_t* word, int polls, uint32_t* err) {
  *word = kRowClaimed;
  __threadfence();
  wait_published(word, kRowClaimed, polls, err);
}

}  // namespace

void stage_column(qeg_ctx* ctx, const qeg_column& c, StagedCol& out) {
  require(c.type >= QEG_I32 && c.type <= QEG_STR, "unknown column type");
  out.len = c.len;
  out.dev.type = c.type;
  out.dev.all_valid = (c.all_valid || c.validity == nullptr) ? 1 : 0;
  const size_t w = type_width(c.type);
  if (c.len == 0) {
    out.dev.data = nullptr;
    out.dev.validity = nullptr;
  } else if (is_device_ptr(c.data)) {
    out.dev.data = c.data;
  } else {
    require(c.data != nullptr, "column data is NULL");
    out.data.alloc(c.len * w, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(out.data.get(), c.data, c.len * w, cudaMemcpyHostToDevice, ctx->stream));
    out.dev.data = out.data.get();
  }
  if (!out.dev.all_valid && c.len > 0) {
    const size_t vb = ((c.len + 63) / 64) * 8;
    if (is_device_ptr(c.validity)) {
      out.dev.validity = c.validity;
    } else {
      out.validity.alloc(vb, ctx->stream);
      QEG_CUDA(cudaMemcpyAsync(out.validity.get(), c.validity, vb, cudaMemcpyHostToDevice, ctx->stream));
      out.dev.validity = out.validity.get<uint64_t>();
    }
  } else {
    out.dev.validity = nullptr;
  }
  out.dev.code_map = nullptr;
  if (c.type == QEG_STR && c.code_map != nullptr && c.code_map_len > 0) {
    if (is_device_ptr(c.code_map)) {
      out.dev.code_map = c.code_map;
    } else {
      out.code_map.alloc(c.code_map_len * 4, ctx->stream);
      QEG_CUDA(cudaMemcpyAsync(out.code_map.get(), c.code_map, c.code_map_len * 4,
                               cudaMemcpyHostToDevice, ctx->stream));
      out.dev.code_map = out.code_map.get<int32_t>();
    }
  }
}

void stage_sel(qeg_ctx* ctx, const uint32_t* sel, uint64_t n, DevBuf& buf, const uint32_t** dev) {
  if (sel == nullptr || n == 0) {
    *dev = nullptr;
    return;
  }
  if (is_device_ptr(sel)) {
    *dev = sel;
    return;
  }
  buf.alloc(n * 4, ctx->stream);
  QEG_CUDA(cudaMemcpyAsync(buf.get(), sel, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  *dev = buf.get<uint32_t>();
}

void check_device_error(qeg_ctx* ctx) {
  uint32_t e = 0;
  QEG_CUDA(cudaMemcpyAsync(&e, ctx->dev_err.get(), 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  raise_device_error(ctx, e);
}

void read_words_and_error(qeg_ctx* ctx, const void* dev_words, size_t nwords, uint64_t* out) {
  uint8_t* pin = static_cast<uint8_t*>(ctx->pinned_in.reserve(nwords * 8 + 16));
  if (nwords)
    QEG_CUDA(cudaMemcpyAsync(pin + 16, dev_words, nwords * 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaMemcpyAsync(pin, ctx->dev_err.get(), 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  uint32_t e;
  std::memcpy(&e, pin, 4);
  if (nwords) std::memcpy(out, pin + 16, nwords * 8);
  raise_device_error(ctx, e);
}

namespace {
// The shared-memory attribute belongs to the function (for every thread of the
// process), so it is only ever raised: the largest size set so far is kept
// per (device, kernel), and a request for more raises it. A launch of `smem`
// bytes after its own request therefore always fits, whatever other threads
// request meanwhile. The occupancy answers are cached per (device, kernel,
// block, shared bytes).
struct SmemAttr {
  const void* kern;
  int dev;
  size_t smem;
};
struct SmemOcc {
  const void* kern;
  int dev, block;
  size_t smem;
  int per_sm;
};
std::mutex g_smem_mu;
std::vector<SmemAttr> g_smem_attrs;
std::vector<SmemOcc> g_smem_occs;

void raise_locked(const void* kern, int dev, size_t smem) {
  if (smem <= 48 * 1024) return;
  SmemAttr* a = nullptr;
  for (SmemAttr& x : g_smem_attrs)
    if (x.kern == kern && x.dev == dev) a = &x;
  if (a && a->smem >= smem) return;
  QEG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  if (a) a->smem = smem;
  else g_smem_attrs.push_back(SmemAttr{kern, dev, smem});
}
}  // namespace

void raise_dynamic_smem(const void* kern, size_t smem) {
  int dev = 0;
  QEG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_smem_mu);
  raise_locked(kern, dev, smem);
}

int blocks_per_sm(const void* kern, int block, size_t smem) {
  int dev = 0;
  QEG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_smem_mu);
  raise_locked(kern, dev, smem);
  for (const SmemOcc& o : g_smem_occs)
    if (o.kern == kern && o.dev == dev && o.block == block && o.smem == smem) return o.per_sm;
  int per_sm = 0;
  QEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
  g_smem_occs.push_back(SmemOcc{kern, dev, block, smem, per_sm});
  return per_sm;
}

void raise_device_error(qeg_ctx* ctx, uint32_t e) {
  if (e == kDevOk) return;
  QEG_CUDA(cudaMemsetAsync(ctx->dev_err.get(), 0, 4, ctx->stream));
  if (e & kDevSpinTimeout)
    throw Error(QEG_ERR_TIMEOUT, "a bounded device-side wait ran out (slot publication)");
  if (e & kDevBadInput)
    throw Error(QEG_ERR_INVALID, "an input index (selection or dictionary code) is out of range");
  throw Error(QEG_ERR_CUDA, "device error word " + std::to_string(e));
}

void fetch_column(qeg_ctx* ctx, const void* dev_vals, const uint8_t* dev_valid, size_t width,
                  uint64_t first, uint64_t count, const qeg_out_column& out) {
  if (count == 0) {
    if (out.all_valid) *out.all_valid = 1;
    return;
  }
  const bool dev_out = is_device_ptr(out.data);
  const auto kind = dev_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (out.data)
    QEG_CUDA(cudaMemcpyAsync(out.data, static_cast<const uint8_t*>(dev_vals) + first * width,
                             count * width, kind, ctx->stream));
  const uint64_t nw = (count + 63) / 64;
  DevBuf words(nw * 8 + 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(words.get<uint8_t>() + nw * 8, 0, 4, ctx->stream));
  uint32_t* any_null = reinterpret_cast<uint32_t*>(words.get<uint8_t>() + nw * 8);
  pack_validity_kernel<<<grid_for(ctx, nw, 256, 4), 256, 0, ctx->stream>>>(dev_valid + first, count,
                                                                         words.get<uint64_t>(), any_null);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  uint32_t has_null = 0;
  if (out.validity) {
    const auto vk = is_device_ptr(out.validity) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    QEG_CUDA(cudaMemcpyAsync(out.validity, words.get(), nw * 8, vk, ctx->stream));
  }
  QEG_CUDA(cudaMemcpyAsync(&has_null, any_null, 4, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (out.all_valid) *out.all_valid = has_null ? 0 : 1;
}

}  // namespace qeg

extern "C" {

qeg_status qeg_ctx_create(int device, qeg_ctx** out) {
  return qeg::guarded(nullptr, [&] {
    qeg::require(out != nullptr, "out is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      throw qeg::Error(QEG_ERR_NO_DEVICE, "no CUDA device available");
    }
    qeg::require(device >= 0 && device < n, "device index out of range");
    QEG_CUDA(cudaSetDevice(device));
    auto c = std::make_unique<qeg_ctx>();
    c->device = device;
    cudaDeviceProp p{};
    QEG_CUDA(cudaGetDeviceProperties(&p, device));
    c->sms = p.multiProcessorCount;
    c->smem_optin = p.sharedMemPerBlockOptin;
    QEG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    // QEG_L2_FETCH_BYTES (32..128): the largest L2 fetch from DRAM on an L2
    // miss, a limit of this process's CUDA context (for measuring random
    // table reads; unset leaves the context's default).
    if (const char* e = std::getenv("QEG_L2_FETCH_BYTES")) {
      const size_t v = static_cast<size_t>(std::atoi(e));
      if (v >= 32 && v <= 128) QEG_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, v));
    }
    // Keep freed stream-ordered allocations cached in this process's pool, so a
    // query's tables and scratch are re-used instead of re-mapped every call.
    cudaMemPool_t pool;
    QEG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    QEG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    c->dev_err.alloc(64, c->stream);
    QEG_CUDA(cudaMemsetAsync(c->dev_err.get(), 0, 64, c->stream));
    QEG_CUDA(cudaStreamSynchronize(c->stream));
    qeg::load_default_weights(c.get());
    *out = c.release();
  });
}

void qeg_ctx_destroy(qeg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  // Every buffer owned by the context is freed on its stream: release them
  // all while the stream still exists, then destroy it.
  ctx->dev_err.release();
  ctx->mlp.reset();
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
    cudaEventDestroy(ctx->side_in);
    cudaEventDestroy(ctx->side_out);
  }
  delete ctx;
}

const char* qeg_last_error(const qeg_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_qeg_tls_err.c_str();
}

void* qeg_ctx_stream(qeg_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

qeg_status qeg_ctx_synchronize(qeg_ctx* ctx) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr, "ctx is NULL");
    qeg::check_device_error(ctx);
  });
}

uint64_t qeg_ctx_kernel_launches(const qeg_ctx* ctx) { return ctx ? ctx->launches : 0; }

qeg_status qeg_host_alloc(uint64_t bytes, void** out) {
  return qeg::guarded(nullptr, [&] {
    qeg::require(out != nullptr, "out is NULL");
    *out = nullptr;
    if (bytes == 0) return;
    const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *out = nullptr;
      throw qeg::Error(QEG_ERR_OOM, std::string("page-locked host allocation: ") + cudaGetErrorString(e));
    }
  });
}

void qeg_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

qeg_status qeg_dev_alloc(qeg_ctx* ctx, uint64_t bytes, void** out) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr && out != nullptr, "ctx/out is NULL");
    *out = nullptr;
    if (bytes == 0) return;
    QEG_CUDA(cudaSetDevice(ctx->device));
    const cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *out = nullptr;
      throw qeg::Error(QEG_ERR_OOM, std::string("device allocation: ") + cudaGetErrorString(e));
    }
  });
}

qeg_status qeg_dev_upload(qeg_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr, "ctx is NULL");
    if (bytes == 0) return;
    qeg::require(dst != nullptr && src != nullptr, "dst/src is NULL");
    qeg::require(qeg::is_device_ptr(dst), "upload destination is not device memory");
    QEG_CUDA(cudaSetDevice(ctx->device));
    QEG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qeg_status qeg_dev_download(qeg_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr, "ctx is NULL");
    if (bytes == 0) return;
    qeg::require(dst != nullptr && src != nullptr, "dst/src is NULL");
    qeg::require(qeg::is_device_ptr(src), "download source is not device memory");
    QEG_CUDA(cudaSetDevice(ctx->device));
    QEG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

void qeg_dev_free(void* p) {
  if (p) cudaFree(p);
}

qeg_status qeg_ctx_check_bounded_wait(qeg_ctx* ctx, int32_t polls) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr, "ctx is NULL");
    qeg::require(polls >= 0 && polls <= (1 << 20), "polls must lie in [0, 2^20]");
    qeg::DevBuf word(8, ctx->stream);
    qeg::stuck_claim_kernel<<<1, 1, 0, ctx->stream>>>(word.get<uint64_t>(), polls, ctx->dev_err.get<uint32_t>());
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    qeg::check_device_error(ctx);
  });
}

}  // extern "C"
