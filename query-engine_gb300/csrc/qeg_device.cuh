// qeg_device.cuh -- device-side building blocks shared by the GROUP BY, join,
// sketch and pipeline kernels (sm_103a).
//
// Key semantics follow the reference's HashTable contract
// (ops/hashtable.h:24-44, ops/hash_internal.cpp:29-60):
//   * I32/STR-id keys zero-extend to a 64-bit word, I64/TS are their bits,
//     BOOL is its 0/1 byte;
//   * F64 keys canonicalise -0.0 to +0.0 and every NaN to one quiet NaN;
//   * NULL is tracked outside the word (a separate null flag / null slot).
// The hash itself is an internal detail (group ids and output order are not part
// of the contract); the splitmix64 finaliser is used because it is a bijection
// on 64 bits, so a single-column key never collides in the full hash.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace qeg {

enum ColType : int32_t { kI32 = 0, kI64 = 1, kF64 = 2, kBOOL = 3, kTS = 4, kSTR = 5 };
// Internal key type (never a column type): a tumbling window's I32 partition
// key and bucket index packed into one key word (see key_word).
constexpr int32_t kPackedKey = 16;

constexpr uint64_t kCanonNaN = 0x7ff8000000000000ull;
constexpr uint64_t kHashSeed = 0x51E57A11AB1E5EEDull;

// A column as the kernels see it: the reference's Column (core/column.h:55-67)
// with an optional code -> id translation for dictionary (STR) columns.
struct DevCol {
  const void* data;
  const uint64_t* validity;  // nullptr when all_valid
  const int32_t* code_map;   // STR only: dictionary code -> canonical value id
  int32_t type;
  int32_t all_valid;
  // Tumbling-window key (I32/I64/TS only): when > 0 the key word is the lower
  // edge of the value's bucket, (v / bucket) * bucket with C++ truncating
  // division, in the column's own type (tsx/window.cpp:318-330).
  int64_t bucket;
  // kPackedKey: `data` is the partition key (type `type1`), `data2` the time
  // column (type `type2`); the key word is (key << 32) | (t / bucket), both
  // halves as 32-bit integers (no NULLs, key values and bucket indexes within
  // int32).
  const void* data2;
  int32_t type2;
  int32_t type1;
};

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__host__ __device__ __forceinline__ uint64_t hash_fold(uint64_t acc, uint64_t w) {
  return mix64(acc ^ mix64(w));
}

__device__ __forceinline__ bool col_valid(const DevCol& c, uint64_t p) {
  if (c.all_valid) return true;
  return (__ldg(c.validity + (p >> 6)) >> (p & 63)) & 1ull;
}

// Canonical 64-bit key word of row p (valid rows only).
__device__ __forceinline__ uint64_t key_word(const DevCol& c, uint64_t p) {
  switch (c.type) {
    case kI32: {
      int32_t v = __ldg(static_cast<const int32_t*>(c.data) + p);
      if (c.bucket > 0) v = static_cast<int32_t>(static_cast<int64_t>(v) / c.bucket * c.bucket);
      return static_cast<uint32_t>(v);
    }
    case kSTR: {
      const int32_t code = __ldg(static_cast<const int32_t*>(c.data) + p);
      return static_cast<uint32_t>(c.code_map ? __ldg(c.code_map + code) : code);
    }
    case kI64:
    case kTS: {
      long long v = __ldg(static_cast<const long long*>(c.data) + p);
      if (c.bucket > 0) v = v / c.bucket * c.bucket;
      return static_cast<uint64_t>(v);
    }
    case kBOOL: return __ldg(static_cast<const uint8_t*>(c.data) + p);
    case kPackedKey: {
      const int32_t a = c.type1 == kI32 ? __ldg(static_cast<const int32_t*>(c.data) + p)
                                        : static_cast<int32_t>(__ldg(static_cast<const long long*>(c.data) + p));
      const long long t = c.type2 == kI32 ? static_cast<long long>(__ldg(static_cast<const int32_t*>(c.data2) + p))
                                          : __ldg(static_cast<const long long*>(c.data2) + p);
      const long long q = t / c.bucket;
      return (static_cast<uint64_t>(static_cast<uint32_t>(a)) << 32) |
             static_cast<uint32_t>(static_cast<int32_t>(q));
    }
    case kF64: {
      const uint64_t b = static_cast<uint64_t>(__ldg(static_cast<const long long*>(c.data) + p));
      const uint64_t mag = b & 0x7fffffffffffffffull;
      if (mag > 0x7ff0000000000000ull) return kCanonNaN;  // any NaN
      if (mag == 0) return 0;                             // -0.0 -> +0.0
      return b;
    }
  }
  return 0;
}

// Integer value of row p widened to int64 (I32/I64/TS/BOOL/STR-id).
__device__ __forceinline__ int64_t int_value(const DevCol& c, uint64_t p) {
  switch (c.type) {
    case kI32: return __ldg(static_cast<const int32_t*>(c.data) + p);
    case kSTR: {
      const int32_t code = __ldg(static_cast<const int32_t*>(c.data) + p);
      return c.code_map ? __ldg(c.code_map + code) : code;
    }
    case kI64:
    case kTS: return __ldg(static_cast<const long long*>(c.data) + p);
    case kBOOL: return __ldg(static_cast<const uint8_t*>(c.data) + p);
    default: return 0;
  }
}

__device__ __forceinline__ double f64_value(const DevCol& c, uint64_t p) {
  return __ldg(static_cast<const double*>(c.data) + p);
}

// ---------------------------------------------------------------------------
// Order-preserving encodings. Every MIN/MAX state is kept as an unsigned 64-bit
// word updated with atomicMax, so that an all-zero word is the identity of every
// aggregate state (COUNT 0, SUM 0 / 0.0, MIN, MAX): a table is initialised by a
// plain memset and never needs a per-slot init step.
//   MAX(int):  enc_i(v) = v ^ 2^63 (unsigned order == signed order)
//   MIN(int):  ~enc_i(v)
//   MAX(f64):  enc_f(d) = total-order bits, NaN canonicalised to the greatest
//   MIN(f64):  ~enc_f(d)
// The F64 order is the reference's NaN-greatest total order
// (ops/agg_internal.h:34-40); -0.0 orders below +0.0 here, which the reference's
// comparator (oracle/result_set.cpp:84-92) treats as equal.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t enc_i64(int64_t v) {
  return static_cast<uint64_t>(v) ^ 0x8000000000000000ull;
}
__host__ __device__ __forceinline__ int64_t dec_i64(uint64_t u) {
  return static_cast<int64_t>(u ^ 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ uint64_t enc_f64_bits(uint64_t b) {
  if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) b = kCanonNaN;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ uint64_t dec_f64_bits(uint64_t u) {
  return (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
}

// ---------------------------------------------------------------------------
// Bounded spin: every device-side wait on another thread's publication gives up
// after kSpinLimit polls and raises an error flag instead of hanging.
// ---------------------------------------------------------------------------
constexpr int kSpinLimit = 1 << 22;

enum DevError : uint32_t {
  kDevOk = 0,
  kDevSpinTimeout = 1u << 0,   // a bounded wait ran out
  kDevSpillOverflow = 1u << 1, // the overflow buffer itself filled up
  kDevBadInput = 1u << 2,      // an index outside its column (sel / code map)
};

// State word of a composite-key row in global memory: 0 empty, 1 claimed (the
// key words are being written), otherwise the published tag.
constexpr uint64_t kRowClaimed = 1;

// Waits until the global state word at `r` (last read as `st`) leaves the
// claimed state, polling at most `limit` times with acquire loads. Returns the
// state it then holds; on running out it raises kDevSpinTimeout in *err and
// returns kRowClaimed, and the caller gives up on the row.
__device__ __forceinline__ uint64_t wait_published(const uint64_t* r, uint64_t st, int limit, uint32_t* err) {
  for (int spins = 0; st == kRowClaimed; ++spins) {
    if (spins >= limit) {
      atomicOr(err, kDevSpinTimeout);
      return kRowClaimed;
    }
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(st) : "l"(r) : "memory");
  }
  return st;
}

}  // namespace qeg
