// qeg_noalloc.cu -- the inner-join COUNT(*)/SUM(probe payload) sink for callers
// that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all: engines whose
// device memory is owned by another allocator (a fixed arena handed out at
// start-up, which a stray cudaMalloc would fragment or exceed), plugins hosted
// by an application that accounts for every device byte itself, and latency-
// critical paths that must not risk an allocation stall or failure at query
// time. For them, qeg_join_count_sum_noalloc runs the whole join sink in a
// fixed scratch area that is part of this library's image: a file-scope
// `static __device__` array of kScratchBytes (about 24 MiB) that every GPU
// loading the library holds until the process exits. The build side is limited
// to kMaxBuildRows rows; larger builds are rejected before any GPU work.
//
// In host code `g_scratch` is only a host-side stand-in for the device array,
// not a device address: passing it to a kernel would fault (or silently use
// the wrong memory where the GPU can reach host memory). The device address
// is looked up once per device with cudaGetSymbolAddress, with that device
// current, the first time the entry point runs on that device; make that first
// call before any stream capture begins.
//
// Every call shares the one scratch array and leaves its contents behind; each
// call clears the parts that must start at zero. Calls whose GPU work overlaps
// (on different streams, or from different threads) race on the scratch and
// corrupt each other's results: serialise them.
#include <mutex>

#include "qeg_internal.h"

namespace qeg {
namespace {

constexpr uint64_t kMaxBuildRows = 1ull << 20;  // build side limit
constexpr uint64_t kCap = 1ull << 21;           // hash slots (load <= 0.5)
constexpr size_t kKeysOff = 0;                                  // (kCap + 1) u64 keys
constexpr size_t kCntOff = kKeysOff + (kCap + 1) * 8;           // (kCap + 1) u32 counts
constexpr size_t kAccOff = ((kCntOff + (kCap + 1) * 4 + 255) / 256) * 256;  // 4 u64
constexpr size_t kScratchBytes = kAccOff + 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {};

// Device address of g_scratch on `device` (which must be current).
void* scratch_address(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (device < 0 || device >= kMaxDevices) throw Error(QEG_ERR_INVALID, "device index out of range");
  if (!g_scratch_dev[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw Error(QEG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_dev[device] = p;
  }
  return g_scratch_dev[device];
}

__device__ __forceinline__ uint64_t slot_hash(uint64_t k) { return hash_fold(kHashSeed, k) & (kCap - 1); }

// out[3] flags.
constexpr unsigned long long kFlagOverflow = 1ull;  // the scratch table filled up
constexpr unsigned long long kFlagBadCode = 2ull;   // a STR code outside its code map

// Key word of row p: key_word(), except that a STR code is checked against its
// code map's length before the map is read (an out-of-range code raises
// kFlagBadCode and the row is skipped). `cm_len` is 0 when there is no map.
__device__ __forceinline__ bool na_key_word(const DevCol& c, uint64_t cm_len, uint64_t p, uint64_t& w,
                                            unsigned long long* acc) {
  if (c.type == kSTR && c.code_map) {
    const int32_t code = __ldg(static_cast<const int32_t*>(c.data) + p);
    if (code < 0 || static_cast<uint64_t>(code) >= cm_len) {
      atomicOr(acc + 3, kFlagBadCode);
      return false;
    }
    w = static_cast<uint32_t>(__ldg(c.code_map + code));
    return true;
  }
  w = key_word(c, p);
  return true;
}

// Counts the build rows of every distinct non-NULL key (key word 0 -> slot kCap).
__global__ void noalloc_build_kernel(DevCol key, uint64_t cm_len, uint64_t n, unsigned long long* keys, uint32_t* cnt,
                                     unsigned long long* acc) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    if (!col_valid(key, r)) continue;
    uint64_t k;
    if (!na_key_word(key, cm_len, r, k, acc)) continue;
    uint64_t s = kCap;
    if (k != 0) {
      s = slot_hash(k);
      uint64_t t = 0;
      for (; t < kCap; ++t) {
        const unsigned long long old = atomicCAS(keys + s, 0ull, static_cast<unsigned long long>(k));
        if (old == 0 || old == k) break;
        s = (s + 1) & (kCap - 1);
      }
      if (t == kCap) {  // cannot happen below the row limit; reported, never hangs
        atomicOr(acc + 3, kFlagOverflow);
        continue;
      }
    }
    atomicAdd(cnt + s, 1u);
  }
}

__global__ void noalloc_probe_kernel(DevCol key, uint64_t cm_len, DevCol val, uint64_t n,
                                     const unsigned long long* keys, const uint32_t* cnt, unsigned long long* acc) {
  unsigned long long c = 0, sum = 0, seen = 0;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
    if (!col_valid(key, p)) continue;
    uint64_t k;
    if (!na_key_word(key, cm_len, p, k, acc)) continue;
    uint64_t m = 0;
    if (k == 0) {
      m = cnt[kCap];
    } else {
      uint64_t s = slot_hash(k);
      for (uint64_t t = 0; t < kCap; ++t) {
        const unsigned long long cur = keys[s];
        if (cur == k) {
          m = cnt[s];
          break;
        }
        if (cur == 0) break;
        s = (s + 1) & (kCap - 1);
      }
    }
    if (!m) continue;
    c += m;
    if (col_valid(val, p)) {
      sum += static_cast<unsigned long long>(int_value(val, p)) * m;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    c += __shfl_down_sync(0xffffffffu, c, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (c) atomicAdd(acc + 0, c);
    if (sum) atomicAdd(acc + 1, sum);
    if (seen) atomicOr(acc + 2, seen);
  }
}

__global__ void noalloc_result_kernel(const unsigned long long* acc, int64_t* out) {
  out[0] = static_cast<int64_t>(acc[0]);
  out[1] = static_cast<int64_t>(acc[1]);
  out[2] = acc[2] ? 1 : 0;
  out[3] = static_cast<int64_t>(acc[3]);
}

DevCol device_column(const qeg_column& c, const char* what) {
  require(c.type >= QEG_I32 && c.type <= QEG_STR, std::string(what) + ": unknown column type");
  DevCol d{};
  d.type = c.type;
  d.all_valid = (c.all_valid || c.validity == nullptr) ? 1 : 0;
  d.data = c.data;
  d.validity = d.all_valid ? nullptr : c.validity;
  // As in the allocating path: a STR column's code map is used only when it
  // has entries.
  d.code_map = (c.type == QEG_STR && c.code_map != nullptr && c.code_map_len > 0) ? c.code_map : nullptr;
  if (c.len > 0) {
    require(is_device_ptr(c.data), std::string(what) + ": data must be a device pointer (no staging copies here)");
    require(d.all_valid || is_device_ptr(c.validity), std::string(what) + ": validity must be a device pointer");
    require(!d.code_map || is_device_ptr(d.code_map), std::string(what) + ": code_map must be a device pointer");
  }
  return d;
}

}  // namespace
}  // namespace qeg

extern "C" {

qeg_status qeg_join_count_sum_noalloc(void* stream, const qeg_column* build_key, const qeg_column* probe_key,
                                      const qeg_column* probe_val, int64_t* out) {
  using namespace qeg;
  return guarded(nullptr, [&] {
    require(build_key && probe_key && probe_val && out, "NULL argument");
    require(build_key->len <= kMaxBuildRows,
            "build side of " + std::to_string(build_key->len) +
                " rows exceeds the no-allocation limit of 1048576 rows; use qeg_join_build instead");
    require(build_key->type == probe_key->type, "HashJoin: join key column types must match positionally");
    require(probe_val->type != QEG_F64 && probe_val->type != QEG_STR, "the count/sum sink sums an integer column");
    require(probe_key->len == probe_val->len, "probe columns differ in length");
    require(is_device_ptr(out), "out must be a device pointer to 4 int64 values");
    const DevCol bk = device_column(*build_key, "build key");
    const DevCol pk = device_column(*probe_key, "probe key");
    const DevCol pv = device_column(*probe_val, "probe payload");
    int device = 0;
    QEG_CUDA(cudaGetDevice(&device));
    unsigned char* base = static_cast<unsigned char*>(scratch_address(device));
    auto* keys = reinterpret_cast<unsigned long long*>(base + kKeysOff);
    auto* cnt = reinterpret_cast<uint32_t*>(base + kCntOff);
    auto* acc = reinterpret_cast<unsigned long long*>(base + kAccOff);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Everything the kernels read before writing starts at zero: the keys, the
    // counts and the accumulators left by the previous call.
    QEG_CUDA(cudaMemsetAsync(base, 0, kScratchBytes, s));
    int sms = 0;
    QEG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const uint64_t nb = build_key->len, np = probe_key->len;
    if (nb > 0) {
      const unsigned g = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((nb + 255) / 256, sms * 8ull)));
      noalloc_build_kernel<<<g, 256, 0, s>>>(bk, bk.code_map ? build_key->code_map_len : 0, nb, keys, cnt, acc);
      QEG_CUDA(cudaGetLastError());
    }
    if (nb > 0 && np > 0) {
      const unsigned g = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((np + 255) / 256, sms * 8ull)));
      noalloc_probe_kernel<<<g, 256, 0, s>>>(pk, pk.code_map ? probe_key->code_map_len : 0, pv, np, keys, cnt, acc);
      QEG_CUDA(cudaGetLastError());
    }
    noalloc_result_kernel<<<1, 1, 0, s>>>(acc, out);
    QEG_CUDA(cudaGetLastError());
  });
}

}  // extern "C"
