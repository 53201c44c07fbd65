// qeg_internal.h -- host-side internals shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/qeg.h"
#include "qeg_device.cuh"

namespace qeg {

// A named NVTX range around one C-ABI call, for timelines of Nsight tools
// (a no-op when no tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Error carrying a qeg_status; thrown inside the library, converted to a status
// code at the C-ABI boundary (no exception crosses it).
struct Error : std::runtime_error {
  qeg_status code;
  Error(qeg_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation)
    throw Error(QEG_ERR_OOM, std::string(what) + ": out of device memory");
  throw Error(QEG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define QEG_CUDA(x) ::qeg::cuda_check((x), #x)

inline void require(bool ok, const std::string& msg) {
  if (!ok) throw Error(QEG_ERR_INVALID, msg);
}
// The same for a message literal: the message string is only built on
// failure (checks inside per-row host loops cost nothing when they pass).
inline void require(bool ok, const char* msg) {
  if (!ok) throw Error(QEG_ERR_INVALID, std::string(msg));
}

// Stream-ordered device buffer (cudaMallocAsync on the context stream).
class DevBuf {
 public:
  DevBuf() = default;
  DevBuf(size_t bytes, cudaStream_t s) { alloc(bytes, s); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { swap(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    release();
    swap(o);
    return *this;
  }
  void alloc(size_t bytes, cudaStream_t s) {
    release();
    stream_ = s;
    bytes_ = bytes;
    if (bytes) QEG_CUDA(cudaMallocAsync(&ptr_, bytes, s));
  }
  void release() {
    if (ptr_) cudaFreeAsync(ptr_, stream_);
    ptr_ = nullptr;
    bytes_ = 0;
  }
  void swap(DevBuf& o) noexcept {
    std::swap(ptr_, o.ptr_);
    std::swap(bytes_, o.bytes_);
    std::swap(stream_, o.stream_);
  }
  template <class T = void>
  T* get() const { return static_cast<T*>(ptr_); }
  size_t bytes() const { return bytes_; }

 private:
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
  cudaStream_t stream_ = nullptr;
};

inline size_t type_width(int32_t t) {
  switch (t) {
    case QEG_I32: return 4;
    case QEG_I64: return 8;
    case QEG_F64: return 8;
    case QEG_BOOL: return 1;
    case QEG_TS: return 8;
    case QEG_STR: return 4;
  }
  return 0;
}

inline bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct Mlp;

}  // namespace qeg

namespace qeg {
// Grow-only page-locked host buffer (one per context): small host<->device
// staging that runs asynchronously on the context stream.
class PinnedBuf {
 public:
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { release(); }
  // At least `bytes` bytes (the previous contents are not kept).
  void* reserve(size_t bytes) {
    if (bytes > bytes_) {
      release();
      const size_t want = std::max<size_t>(bytes, size_t{1} << 16);
      if (cudaHostAlloc(&ptr_, want, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        ptr_ = nullptr;
        throw Error(QEG_ERR_OOM, "page-locked host buffer allocation failed");
      }
      bytes_ = want;
    }
    return ptr_;
  }
  void release() {
    if (ptr_) cudaFreeHost(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
  }

 private:
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};
}  // namespace qeg

struct qeg_ctx {
  int device = 0;
  int sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  uint64_t launches = 0;
  qeg::DevBuf dev_err;  // uint32 device error word (qeg::DevError bits)
  cudaStream_t side = nullptr;  // copies that overlap the context stream's kernels (created on first use)
  cudaEvent_t side_in = nullptr, side_out = nullptr;  // fork / join of the side stream
  std::shared_ptr<qeg::Mlp> mlp;  // the learned estimator, when weights are loaded
  qeg::PinnedBuf pinned_in, pinned_out;  // small staging of a call (device -> host, host -> device)
};

namespace qeg {
// Loads the shipped estimator weights into a new context (qeg_estimator.cu).
void load_default_weights(qeg_ctx* ctx);
}  // namespace qeg

namespace qeg {

// Resolves a caller column to device pointers: device pointers are used in
// place; host pointers are copied into buffers owned by this object.
struct StagedCol {
  DevCol dev{};
  DevBuf data, validity, code_map;
  uint64_t len = 0;
};

void stage_column(qeg_ctx* ctx, const qeg_column& c, StagedCol& out);
void stage_sel(qeg_ctx* ctx, const uint32_t* sel, uint64_t n, DevBuf& buf, const uint32_t** dev);

// Checks and clears the context's device error word (syncs the stream).
void check_device_error(qeg_ctx* ctx);
// Copies `nwords` 64-bit words from the device and the context's device error
// word in one stream synchronisation, then checks the error word as
// check_device_error does.
void read_words_and_error(qeg_ctx* ctx, const void* dev_words, size_t nwords, uint64_t* out);
// Throws the error an error word `e` (read from the device) stands for, after
// clearing the device copy; returns for no error.
void raise_device_error(qeg_ctx* ctx, uint32_t e);
// Raises `kern`'s dynamic shared-memory attribute on the current device to
// `smem` bytes when it is lower (never lowers it), under one process-wide
// lock: operator instances in several threads launch the same kernels with
// different sizes. Every setting of that attribute goes through here.
void raise_dynamic_smem(const void* kern, size_t smem);
// Blocks per SM of `kern` at `block` threads and `smem` dynamic shared bytes
// on the current device, after raise_dynamic_smem(kern, smem); cached per
// (device, kernel, block, smem).
int blocks_per_sm(const void* kern, int block, size_t smem);

inline unsigned grid_for(qeg_ctx* ctx, uint64_t work_items, int block, int blocks_per_sm) {
  const uint64_t want = (work_items + block - 1) / block;
  const uint64_t cap = static_cast<uint64_t>(ctx->sms) * blocks_per_sm;
  uint64_t g = want < cap ? want : cap;
  return static_cast<unsigned>(g == 0 ? 1 : g);
}

// Copies `count` rows starting at `first` of a device column (values `width`
// bytes, validity as one byte per row) into a caller output column (host or
// device), packing validity into 64-bit words.
void fetch_column(qeg_ctx* ctx, const void* dev_vals, const uint8_t* dev_valid, size_t width,
                  uint64_t first, uint64_t count, const qeg_out_column& out);

template <class F>
qeg_status guarded(qeg_ctx* ctx, F&& fn);

}  // namespace qeg

extern thread_local std::string g_qeg_tls_err;

template <class F>
qeg_status qeg::guarded(qeg_ctx* ctx, F&& fn) {
  try {
    fn();
    return QEG_OK;
  } catch (const qeg::Error& e) {
    (ctx ? ctx->err : g_qeg_tls_err) = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    (ctx ? ctx->err : g_qeg_tls_err) = "out of host memory";
    return QEG_ERR_OOM;
  } catch (const std::exception& e) {
    (ctx ? ctx->err : g_qeg_tls_err) = e.what();
    return QEG_ERR_CUDA;
  }
}
