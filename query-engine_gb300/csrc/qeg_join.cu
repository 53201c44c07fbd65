// qeg_join.cu -- hash equi-join on sm_103a: replaces qe::HashJoin
// (ops/join.h:69-123, ops/join.cpp).
//
// Build (ops/join.cpp:133-197): every build batch is appended to a device
// BuildStore (column values + one validity byte per row, the GPU form of
// ops/join_internal.h:38-93). build_finish() then builds a CSR multiplicity
// map over the rows whose key tuple holds no NULL (NULL keys never match,
// NullPolicy::kNeverMatch, ops/hashtable.h:36-43):
//   slot  : a key's position in an open-addressing table (QEG_JOIN_HASH), or
//           value - min over the key range (QEG_JOIN_DENSE, chosen when the
//           non-null build keys are integers whose range is at most 4x their
//           count);
//   cnt   : build rows per slot; off: exclusive prefix sum of cnt;
//   rows  : build row ids grouped by slot (the group_rows lists of
//           ops/join.cpp:190-194, as one array).
// A build whose keys are all distinct also gets a bitmap (DENSE) or a
// "unique" flag (HASH) so a probe that only needs the match count reads one
// bit / one key word per row.
//
// Probe: per probe batch, a count kernel sizes each probe row's output (LEFT:
// at least one row), a scan turns the counts into offsets, an emit kernel
// writes (probe row, build row | NULL) pairs (build_pairs_for_probe,
// ops/join.cpp:199-247), and fetch() gathers the output columns, probe columns
// then build columns (ops/join_internal.h:136-179). The COUNT(*)/SUM(payload)
// sink is fused into one probe kernel.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "qeg_agg.h"
#include "qeg_scan.cuh"
#include "qeg_sort.h"

namespace qeg {

namespace {

constexpr uint32_t kNullRow = 0xffffffffu;  // ops/join_internal.h:31
// Hashed single-key tables of at least this many bytes (too large to stay in
// L2 beside the probe stream) get a Bloom filter of kBloomBitsPerKey bits per
// build row: 16 bits and four bits per key in one 64-bit word give a false
// positive rate of about 0.5%, in 32 MB for 16M build rows.
constexpr uint64_t kBloomMinTableBytes = 32ull << 20;
constexpr uint64_t kBloomBitsPerKey = 16;
// Learned sizing of hashed single-key builds (QEG_SIZE_LEARNED): build sides
// of at least kJoinSketchMinRows rows are sketched, and the table gets
// kJoinSlotsPerEstimatedKey slots per estimated distinct key (a power of two,
// never more than the row count's two per row): load 0.25 at the estimate,
// 0.5 at a two-fold underestimate. Inserts into such a table give up after
// kEstimatedTableProbeLimit slots; an overflow rebuilds it at full size.
constexpr uint64_t kJoinSketchMinRows = 1ull << 20;
constexpr double kJoinSlotsPerEstimatedKey = 4.0;
constexpr uint64_t kEstimatedTableProbeLimit = 1024;

struct JTable {
  int strategy;    // QEG_JOIN_HASH / QEG_JOIN_DENSE
  int nkeys;
  int kw;          // words per hash row: 1 (single key) or 1 + nkeys
  uint64_t* keys;  // hash rows; single key: slot cap holds key word 0
  uint64_t cap;    // hash: power of two; dense: range
  int64_t dmin;    // dense: smallest key value
  uint32_t* cnt;   // cap (+1 hash single key) entries
  const uint64_t* off;
  const uint32_t* rows;
  const uint64_t* bitmap;  // dense and unique: one bit per slot
  int unique;
  int shift;  // hash, single key: home slot = hash >> shift (64 - log2 cap)
  // Hash, single key: a blocked Bloom filter of the build keys (nullptr: none).
  // Key hash h selects word h >> bshift and sets the four bits bloom_mask(h).
  const uint64_t* bloom;
  int bshift;
};

__device__ __forceinline__ uint64_t ld_relaxed64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Acquire load of a composite row's state word: the key words published
// before its tag (a fence, then the atomic exchange) are visible after it.
__device__ __forceinline__ uint64_t ld_acquire64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Loads the key tuple of row p. Returns false when any key column is NULL.
// Slot hash of a key tuple: one splitmix64 round for a single key word, the
// seeded fold of every word for composite keys.
__device__ __forceinline__ uint64_t single_key_hash(uint64_t k) { return mix64(k ^ kHashSeed); }

// Bits of a key in its Bloom filter word: four positions from the low 24 bits
// of the key hash (the word is chosen by its top bits, the table's home slot by
// its top bits too, so the positions are independent of both).
__device__ __forceinline__ uint64_t bloom_mask(uint64_t h) {
  return (1ull << (h & 63)) | (1ull << ((h >> 6) & 63)) | (1ull << ((h >> 12) & 63)) | (1ull << ((h >> 18) & 63));
}

__device__ __forceinline__ bool load_key(const DevCol* kc, int nk, uint64_t p, uint64_t* w, uint64_t& h) {
  h = kHashSeed;
  for (int j = 0; j < nk; ++j) {
    if (!col_valid(kc[j], p)) return false;
    w[j] = key_word(kc[j], p);
    h = hash_fold(h, w[j]);
  }
  if (nk == 1) h = single_key_hash(w[0]);
  return true;
}

__device__ __forceinline__ int64_t dense_value(const DevCol& c, uint64_t p) { return int_value(c, p); }

// Finds (insert = true: or inserts) the slot of a key tuple. -1: absent / full.
// `existed` (may be null) is set when an insert found the key already there.
// Key word 0 of a single key has the side slot `cap`, which the caller tracks.
template <bool INSERT>
__device__ __forceinline__ int64_t hash_slot(const JTable& T, const uint64_t* w, uint64_t h, uint32_t* err,
                                             bool* existed = nullptr, uint64_t limit = ~0ull) {
  if (T.nkeys == 1) {
    const uint64_t k = w[0];
    if (k == 0) return static_cast<int64_t>(T.cap);
    uint64_t s = h >> T.shift;  // home slot: the top bits of the hash
    // (`limit`: an insert into a table sized from an estimate gives up after
    // that many slots; the build is then redone at full size.)
    for (uint64_t t = 0; t < T.cap && t < limit; ++t) {
      uint64_t* r = T.keys + s;
      uint64_t cur = ld_relaxed64(r);
      if (cur == k) {
        if (existed) *existed = true;
        return static_cast<int64_t>(s);
      }
      if (cur == 0) {
        if (!INSERT) return -1;
        cur = atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, static_cast<unsigned long long>(k));
        if (cur == k && existed) *existed = true;
        if (cur == 0 || cur == k) return static_cast<int64_t>(s);
      }
      s = (s + 1) & (T.cap - 1);
    }
    return -1;
  }
  const uint64_t tag = (h >> 32) | 2ull;
  uint64_t s = h & (T.cap - 1);
  for (uint64_t t = 0; t < T.cap; ++t) {
    uint64_t* r = T.keys + s * T.kw;
    uint64_t st = ld_acquire64(r);
    if (st == 0) {
      if (!INSERT) return -1;
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, 1ull);
      if (old == 0) {
        for (int j = 0; j < T.nkeys; ++j) r[1 + j] = w[j];
        __threadfence();
        atomicExch(reinterpret_cast<unsigned long long*>(r), static_cast<unsigned long long>(tag));
        return static_cast<int64_t>(s);
      }
      st = old;
    }
    st = wait_published(r, st, kSpinLimit, err);
    if (st == kRowClaimed) return -1;
    if (st == tag) {
      bool eq = true;
      for (int j = 0; eq && j < T.nkeys; ++j) eq = ld_relaxed64(r + 1 + j) == w[j];
      if (eq) {
        if (existed) *existed = true;
        return static_cast<int64_t>(s);
      }
    }
    s = (s + 1) & (T.cap - 1);
  }
  return -1;
}

struct BuildK {
  DevCol key[kMaxKeys];
  int nkeys;
  int no_count;  // insert keys only (the as-of join needs no per-slot row counts)
  // Hash table, counts deferred: the insert itself tells a repeated key (only
  // key word 0's side slot is counted); per-slot row counts are taken by a
  // second pass when a probe needs them.
  int presence;
  uint64_t n;
  JTable T;
  uint32_t* fill;
  uint32_t* rows_out;
  uint32_t* dup;
  unsigned long long* distinct;
  uint32_t* err;
  unsigned long long* bloom;  // single key: the Bloom filter to fill (nullptr: none)
  // Single key, table sized from an estimate: inserts give up after
  // probe_limit slots and raise *ovf (nullptr: full-size table, no limit).
  uint32_t* ovf;
  uint64_t probe_limit;
};

__global__ void build_count_kernel(BuildK P) {
  unsigned long long fresh = 0;
  uint32_t dup = 0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n; r += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t w[kMaxKeys], h;
    bool existed = false;
    if (!load_key(P.key, P.nkeys, r, w, h)) continue;
    if (P.bloom) atomicOr(P.bloom + (h >> P.T.bshift), static_cast<unsigned long long>(bloom_mask(h)));
    int64_t s;
    if (P.T.strategy == QEG_JOIN_DENSE) {
      s = dense_value(P.key[0], r) - P.T.dmin;
    } else {
      s = hash_slot<true>(P.T, w, h, P.err, &existed, P.ovf ? P.probe_limit : ~0ull);
      if (s < 0) {
        if (P.ovf) atomicExch(P.ovf, 1u);  // the table is too small: the host rebuilds it
        else atomicOr(P.err, kDevSpillOverflow);
        continue;
      }
    }
    if (P.no_count) continue;
    if (P.presence && !(P.T.nkeys == 1 && static_cast<uint64_t>(s) == P.T.cap)) {
      if (existed) dup = 1;
      else ++fresh;
      continue;
    }
    if (atomicAdd(&P.T.cnt[s], 1u) != 0) dup = 1;
    else ++fresh;
  }
  for (int o = 16; o > 0; o >>= 1) {
    fresh += __shfl_down_sync(0xffffffffu, fresh, o);
    dup |= __shfl_down_sync(0xffffffffu, dup, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (fresh) atomicAdd(P.distinct, fresh);
    if (dup) *P.dup = 1;
  }
}

__global__ void build_scatter_kernel(BuildK P) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n; r += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t w[kMaxKeys], h;
    if (!load_key(P.key, P.nkeys, r, w, h)) continue;
    int64_t s;
    if (P.T.strategy == QEG_JOIN_DENSE) {
      s = dense_value(P.key[0], r) - P.T.dmin;
    } else {
      s = hash_slot<false>(P.T, w, h, P.err);
      if (s < 0) continue;
    }
    const uint64_t pos = P.T.off[s] + atomicAdd(&P.fill[s], 1u);
    P.rows_out[pos] = static_cast<uint32_t>(r);
  }
}

// Dense build: sets the bit of every non-NULL build key (fire-and-forget
// reductions; the distinct count, and so uniqueness, comes from a population
// count of the bitmap afterwards).
__global__ void dense_mark_kernel(BuildK P, unsigned long long* __restrict__ bits) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n; r += (uint64_t)gridDim.x * blockDim.x) {
    if (!col_valid(P.key[0], r)) continue;
    const uint64_t s = static_cast<uint64_t>(dense_value(P.key[0], r) - P.T.dmin);
    atomicOr(bits + (s >> 6), 1ull << (s & 63));
  }
}

// Number of set bits of `nw` words, added to *out.
__global__ void popc_kernel(const unsigned long long* __restrict__ w, uint64_t nw, unsigned long long* out) {
  unsigned long long c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x)
    c += __popcll(w[i]);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// Range of the non-null values of one integer key column.
__global__ void minmax_kernel(DevCol c, uint64_t n, unsigned long long* out /* [0]=min enc, [1]=max enc, [2]=count */) {
  unsigned long long mn = ~0ull, mx = 0, cnt = 0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    if (!col_valid(c, r)) continue;
    const unsigned long long e = enc_i64(int_value(c, r));
    mn = e < mn ? e : mn;
    mx = e > mx ? e : mx;
    ++cnt;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  // One set of global atomics per CTA (per-warp atomics on three words
  // serialise at the L2).
  __shared__ unsigned long long smn[32], smx[32], scn[32];
  const unsigned warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    smn[warp] = mn;
    smx[warp] = mx;
    scn[warp] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned w = 1; w < nwarps; ++w) {
      mn = min(mn, smn[w]);
      mx = max(mx, smx[w]);
      cnt += scn[w];
    }
    if (cnt) {
      atomicMin(out + 0, mn);
      atomicMax(out + 1, mx);
      atomicAdd(out + 2, cnt);
    }
  }
}

// Slot of a probe key, or -1 on a miss (NULL keys are filtered by the caller).
__device__ __forceinline__ int64_t probe_slot(const JTable& T, const DevCol* kc, uint64_t p, const uint64_t* w,
                                              uint64_t h, uint32_t* err) {
  if (T.strategy == QEG_JOIN_DENSE) {
    const int64_t v = dense_value(kc[0], p);
    const uint64_t s = static_cast<uint64_t>(v) - static_cast<uint64_t>(T.dmin);
    if (v < T.dmin || s >= T.cap) return -1;
    return static_cast<int64_t>(s);
  }
  return hash_slot<false>(T, w, h, err);
}

struct ProbeK {
  DevCol key[kMaxKeys];
  int nkeys;
  DevCol val;  // count/sum sink payload
  uint64_t n;
  JTable T;
  int left;
  uint32_t* counts;    // per probe row output rows
  const uint64_t* starts;
  uint32_t* out_probe;
  uint32_t* out_build;
  unsigned long long* acc;  // sink: [0] count, [1] sum, [2] any payload
  uint32_t* err;
};

// Read-only lookup of one key in the finished table: match multiplicity.
template <typename KT, int STRAT, bool UNIQUE>
__device__ __forceinline__ uint64_t sink_lookup(const JTable& T, KT key) {
  if (STRAT == QEG_JOIN_DENSE) {
    const uint64_t s = static_cast<uint64_t>(static_cast<int64_t>(key)) - static_cast<uint64_t>(T.dmin);
    if (s >= T.cap) return 0;
    if (UNIQUE) return (__ldg(T.bitmap + (s >> 6)) >> (s & 63)) & 1ull;
    return __ldg(T.cnt + s);
  } else {
    const uint64_t k = sizeof(KT) == 4 ? static_cast<uint64_t>(static_cast<uint32_t>(key))
                                       : static_cast<uint64_t>(key);
    if (k == 0) return __ldg(T.cnt + T.cap);
    // Linear probing read four slots (one 32-byte sector) at a time: the
    // aligned group holding the home slot, then the following groups. Slots
    // before the home slot in the first group are not part of the probe.
    const uint64_t home = single_key_hash(k) >> T.shift;
    uint64_t g = home & ~3ull;
    int skip = static_cast<int>(home & 3);
    const ulonglong2* base = reinterpret_cast<const ulonglong2*>(T.keys);
    for (uint64_t t = 0; t < T.cap; t += 4) {
      const ulonglong2 a = __ldg(base + (g >> 1));
      const ulonglong2 b = __ldg(base + (g >> 1) + 1);
      const uint64_t c[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (i < skip) continue;
        if (c[i] == k) return UNIQUE ? 1 : __ldg(T.cnt + g + i);
        if (c[i] == 0) return 0;
      }
      skip = 0;
      g = (g + 4) & (T.cap - 1);
    }
    return 0;
  }
}

// Loads a 64-bit word with an L2 evict-last policy: the Bloom filter (and
// optionally the table) keeps its lines in L2 while the probe stream, loaded
// evict-first, passes through.
__device__ __forceinline__ uint64_t ld_keep_l2(const uint64_t* p, uint64_t pol) {
  uint64_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ ulonglong2 ld_keep_l2x2(const ulonglong2* p, uint64_t pol) {
  ulonglong2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.u64 {%0, %1}, [%2], %3;" : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ uint64_t evict_last_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// Hashed single-key lookup of key word k (nonzero, home slot `home`) whose
// first 32-byte slot group {a, b} (the aligned group holding the home slot) the
// caller has already loaded: resolves within it when it can, else walks on.
template <bool UNIQUE>
__device__ __forceinline__ uint64_t hashed_resolve(const JTable& T, uint64_t k, uint64_t home, ulonglong2 a,
                                                   ulonglong2 b) {
  uint64_t g = home & ~3ull;
  int skip = static_cast<int>(home & 3);
  const ulonglong2* base = reinterpret_cast<const ulonglong2*>(T.keys);
  for (uint64_t t = 0; t < T.cap; t += 4) {
    if (t) {
      a = __ldg(base + (g >> 1));
      b = __ldg(base + (g >> 1) + 1);
    }
    const uint64_t c[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i < skip) continue;
      if (c[i] == k) return UNIQUE ? 1 : __ldg(T.cnt + g + i);
      if (c[i] == 0) return 0;
    }
    skip = 0;
    g = (g + 4) & (T.cap - 1);
  }
  return 0;
}

// Match multiplicities of two probe keys against a hashed single-key table,
// with every memory access of the two rows issued before any is consumed: the
// two Bloom filter words (when the table has a filter), then the first slot
// group of each row that passed it. kv: the key is non-NULL.
template <typename KT, bool UNIQUE, bool BLOOM>
__device__ __forceinline__ void hashed_lookup2(const JTable& T, const KT (&key)[2], const bool (&kv)[2],
                                               uint64_t (&m)[2], uint64_t keep_pol, int keep_table) {
  uint64_t k[2], h[2];
  bool go[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    k[j] = sizeof(KT) == 4 ? static_cast<uint64_t>(static_cast<uint32_t>(key[j])) : static_cast<uint64_t>(key[j]);
    h[j] = single_key_hash(k[j]);
    go[j] = kv[j];
  }
  if (BLOOM) {
    uint64_t fw[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) fw[j] = go[j] ? ld_keep_l2(T.bloom + (h[j] >> T.bshift), keep_pol) : 0;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const uint64_t bm = bloom_mask(h[j]);
      go[j] = go[j] && (fw[j] & bm) == bm;
    }
  }
  const ulonglong2* base = reinterpret_cast<const ulonglong2*>(T.keys);
  ulonglong2 a[2], b[2];
  uint64_t home[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    home[j] = h[j] >> T.shift;
    a[j] = make_ulonglong2(0, 0);
    b[j] = make_ulonglong2(0, 0);
    if (go[j] && k[j] != 0) {
      const uint64_t g = home[j] & ~3ull;
      if (keep_table) {
        a[j] = ld_keep_l2x2(base + (g >> 1), keep_pol);
        b[j] = ld_keep_l2x2(base + (g >> 1) + 1, keep_pol);
      } else {
        a[j] = __ldg(base + (g >> 1));
        b[j] = __ldg(base + (g >> 1) + 1);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (!go[j]) m[j] = 0;
    else if (k[j] == 0) m[j] = __ldg(T.cnt + T.cap);
    else m[j] = hashed_resolve<UNIQUE>(T, k[j], home[j], a[j], b[j]);
  }
}

struct SinkK {
  const void* key;
  const uint64_t* kvalid;  // nullptr: no NULL keys
  const void* val;
  const uint64_t* vvalid;  // nullptr: no NULL payloads
  uint64_t n;
  JTable T;
  unsigned long long* acc;  // [0] count, [1] sum, [2] any non-null payload matched
  int keep_table;           // hashed table reads also evict-last in L2 (QEG_JOIN_TABLE_KEEP_L2=1)
};

template <typename T>
__device__ __forceinline__ void load4(const T* p, T (&o)[4]) {
  if (sizeof(T) == 8) {
    const longlong2 a = __ldcs(reinterpret_cast<const longlong2*>(p));
    const longlong2 b = __ldcs(reinterpret_cast<const longlong2*>(p) + 1);
    o[0] = static_cast<T>(a.x);
    o[1] = static_cast<T>(a.y);
    o[2] = static_cast<T>(b.x);
    o[3] = static_cast<T>(b.y);
  } else {
    const int4 a = __ldcs(reinterpret_cast<const int4*>(p));
    o[0] = static_cast<T>(a.x);
    o[1] = static_cast<T>(a.y);
    o[2] = static_cast<T>(a.z);
    o[3] = static_cast<T>(a.w);
  }
}

// The COUNT(*) / SUM(payload) sink of an inner join fused into the probe:
// each thread takes 4 consecutive rows per step (16-byte streaming loads, one
// validity word read per 4 rows), looks the keys up with read-only loads, and
// the partial count/sum are reduced per block before one atomic per block.
template <typename KT, typename VT, int STRAT, bool UNIQUE>
__global__ void __launch_bounds__(256) probe_sink_kernel(const SinkK P) {
  unsigned long long cnt = 0, sum = 0, seen = 0;
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const uint64_t nq = P.n >> 2;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // Two quads per step (q and q + stride), all loads issued before any lookup,
  // so each thread keeps 64 bytes of the probe side in flight.
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < nq; q += 2 * stride) {
    KT k[2][4];
    VT v[2][4];
    uint32_t kb[2], vb[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const uint64_t qq = q + u * stride;
      kb[u] = vb[u] = 0;
      if (qq < nq) {
        const uint64_t r0 = qq << 2;
        load4(keys + r0, k[u]);
        load4(vals + r0, v[u]);
        kb[u] = P.kvalid ? static_cast<uint32_t>(__ldg(P.kvalid + (r0 >> 6)) >> (r0 & 63)) & 0xFu : 0xFu;
        vb[u] = P.vvalid ? static_cast<uint32_t>(__ldg(P.vvalid + (r0 >> 6)) >> (r0 & 63)) & 0xFu : 0xFu;
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      uint64_t m[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) m[j] = ((kb[u] >> j) & 1u) ? sink_lookup<KT, STRAT, UNIQUE>(P.T, k[u][j]) : 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        cnt += m[j];
        if (m[j] && ((vb[u] >> j) & 1u)) {
          sum += static_cast<unsigned long long>(static_cast<int64_t>(v[u][j])) * m[j];
          seen = 1;
        }
      }
    }
  }
  // Tail rows (n not a multiple of 4).
  const uint64_t tail0 = nq << 2;
  const uint64_t gt = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (gt < P.n - tail0) {
    const uint64_t r = tail0 + gt;
    const bool kv = !P.kvalid || ((P.kvalid[r >> 6] >> (r & 63)) & 1ull);
    const uint64_t m = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, keys[r]) : 0;
    cnt += m;
    if (m && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * m;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], cnt);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], seen);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

// Two consecutive values with one load: 16 bytes for 8-byte types, 8 bytes
// for 4-byte types (the caller guarantees 16-byte-aligned columns and an even
// row index).
template <typename T>
__device__ __forceinline__ void load2(const T* p, T (&o)[2]) {
  if (sizeof(T) == 8) {
    const longlong2 a = __ldcs(reinterpret_cast<const longlong2*>(p));
    o[0] = static_cast<T>(a.x);
    o[1] = static_cast<T>(a.y);
  } else {
    const int2 a = __ldcs(reinterpret_cast<const int2*>(p));
    o[0] = static_cast<T>(a.x);
    o[1] = static_cast<T>(a.y);
  }
}

// Probe sides the 32-bit tile counters of the lean and swept sinks cover.
inline bool lean_sizes_ok(uint64_t n) { return n / 64 < (uint64_t{1} << 31); }

// Hashed single-key COUNT/SUM sink in sweeps: launch `sweep` of `nsweeps`
// handles only the probe rows whose key hash falls in the sweep's 1/nsweeps
// of the hash range. The table's home slot is the top bits of the hash, so a
// sweep's lookups stay in one contiguous window of the table, small enough to
// stay in L2 while the probe stream passes through evict-first: every sweep
// re-reads the probe keys, but a lookup is an L2 hit instead of a random DRAM
// read (on GB300 a random 32-byte read from DRAM moves a whole 128-byte line).
// A warp takes 128 rows per step (two 64-row chunks, lane i: rows 2i, 2i + 1
// of each, all key loads issued first), hashes each key once, and queues the
// rows of its sweep in shared memory, so the lookups then run with every lane
// busy. Payloads and their validity are read only for rows that matched.
constexpr int kSweepThreads = 256;
template <typename KT, typename VT, bool UNIQUE>
__global__ void __launch_bounds__(kSweepThreads, 6) probe_sink_sweep_kernel(const SinkK P, uint32_t sweep,
                                                                            uint32_t nsweeps) {
  constexpr int kRows = 128;  // rows per warp step
  __shared__ uint64_t q_key[kSweepThreads / 32][kRows];
  __shared__ uint64_t q_hash[kSweepThreads / 32][kRows];
  __shared__ uint8_t q_row[kSweepThreads / 32][kRows];
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const unsigned lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint32_t ntiles = static_cast<uint32_t>(P.n / kRows);
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const ulonglong2* tab = reinterpret_cast<const ulonglong2*>(P.T.keys);
  const uint64_t mask = P.T.cap - 1;
  using Cnt = typename std::conditional<UNIQUE, uint32_t, unsigned long long>::type;
  Cnt cnt = 0;
  uint32_t seen = 0;
  unsigned long long sum = 0;
  // Match multiplicity of key word k (hash h) in the table.
  auto lookup = [&](uint64_t k, uint64_t h) -> uint64_t {
    if (k == 0) return __ldg(P.T.cnt + P.T.cap);
    const uint64_t home = h >> P.T.shift;
    uint64_t g = home & ~3ull;
    int skip = static_cast<int>(home & 3);
    for (uint64_t t = 0; t <= mask; t += 4) {
      const ulonglong2 a = __ldg(tab + (g >> 1));
      const ulonglong2 b = __ldg(tab + (g >> 1) + 1);
      const uint64_t c[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (i < skip) continue;
        if (c[i] == k) return UNIQUE ? 1 : __ldg(P.T.cnt + g + i);
        if (c[i] == 0) return 0;
      }
      skip = 0;
      g = (g + 4) & mask;
    }
    return 0;
  };
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nwarps) {
    const uint64_t base = static_cast<uint64_t>(t) * kRows;
    KT k[2][2];
    uint64_t kw[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      load2(keys + base + c * 64 + 2 * lane, k[c]);
      kw[c] = P.kvalid ? __ldg(P.kvalid + (base >> 6) + c) : ~0ull;
    }
    // Queue the rows of this sweep.
    uint32_t nq = 0;
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const uint64_t kk = sizeof(KT) == 4 ? static_cast<uint64_t>(static_cast<uint32_t>(k[c][j]))
                                            : static_cast<uint64_t>(k[c][j]);
        const uint64_t h = single_key_hash(kk);
        const bool go = ((kw[c] >> (2 * lane + j)) & 1ull) &&
                        static_cast<uint32_t>(__umul64hi(h, nsweeps)) == sweep;
        const unsigned bal = __ballot_sync(0xffffffffu, go);
        if (go) {
          const uint32_t at = nq + __popc(bal & ((1u << lane) - 1u));
          q_key[wib][at] = kk;
          q_hash[wib][at] = h;
          q_row[wib][at] = static_cast<uint8_t>(c * 64 + 2 * lane + j);
        }
        nq += __popc(bal);
      }
    __syncwarp();
    for (uint32_t i = lane; i < nq; i += 32) {
      const uint64_t m = lookup(q_key[wib][i], q_hash[wib][i]);
      if (!m) continue;
      cnt += static_cast<Cnt>(m);
      const uint64_t r = base + q_row[wib][i];
      if (!P.vvalid || ((__ldg(P.vvalid + (r >> 6)) >> (r & 63)) & 1ull)) {
        sum += static_cast<unsigned long long>(static_cast<int64_t>(__ldcs(vals + r))) * m;
        seen = 1;
      }
    }
    __syncwarp();
  }
  // Rows after the last full step, one per thread.
  for (uint64_t r = static_cast<uint64_t>(ntiles) * kRows + static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       r < P.n; r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    if (P.kvalid && !((P.kvalid[r >> 6] >> (r & 63)) & 1ull)) continue;
    const uint64_t kk = sizeof(KT) == 4 ? static_cast<uint64_t>(static_cast<uint32_t>(keys[r]))
                                        : static_cast<uint64_t>(keys[r]);
    const uint64_t h = single_key_hash(kk);
    if (static_cast<uint32_t>(__umul64hi(h, nsweeps)) != sweep) continue;
    const uint64_t mm = lookup(kk, h);
    cnt += static_cast<Cnt>(mm);
    if (mm && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * mm;
      seen = 1;
    }
  }
  unsigned long long c64 = cnt;
  for (int o = 16; o > 0; o >>= 1) {
    c64 += __shfl_down_sync(0xffffffffu, c64, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  if (lane == 0) {
    if (c64) atomicAdd(P.acc + 0, c64);
    if (sum) atomicAdd(P.acc + 1, sum);
    if (seen) atomicMax(P.acc + 2, 1ull);
  }
}

// Software-pipelined sink. A warp owns tiles of U x 64 rows; in a tile, lane i
// takes rows 2i and 2i+1 of every 64-row chunk, so each warp load instruction
// reads one contiguous 256- or 512-byte span, and the chunk's validity is one
// 64-bit word. The loads of the warp's next tile are issued before the
// lookups of the current one, so the probe stream stays in flight while the
// table lookups (L2-resident for the dense table) complete.
template <typename KT, typename VT, int STRAT, bool UNIQUE, int U>
__global__ void __launch_bounds__(256, 4) probe_sink_pipe_kernel(const SinkK P) {
  unsigned long long cnt = 0, sum = 0, seen = 0;
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const unsigned lane = threadIdx.x & 31u;
  constexpr uint64_t kTile = 64ull * U;
  const uint64_t ntiles = P.n / kTile;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  uint64_t t = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  KT k[U][2];
  VT v[U][2];
  uint64_t kw[U], vw[U];
  auto load_tile = [&](uint64_t tile) {
    const uint64_t base = tile * kTile;
#pragma unroll
    for (int c = 0; c < U; ++c) {
      const uint64_t r = base + c * 64 + 2 * lane;
      load2(keys + r, k[c]);
      load2(vals + r, v[c]);
      kw[c] = P.kvalid ? __ldg(P.kvalid + (base >> 6) + c) : ~0ull;
      vw[c] = P.vvalid ? __ldg(P.vvalid + (base >> 6) + c) : ~0ull;
    }
  };
  if (t < ntiles) load_tile(t);
  for (; t < ntiles; t += nwarps) {
    KT ck[U][2];
    VT cv[U][2];
    uint32_t kb[U], vb[U];
#pragma unroll
    for (int c = 0; c < U; ++c) {
      ck[c][0] = k[c][0];
      ck[c][1] = k[c][1];
      cv[c][0] = v[c][0];
      cv[c][1] = v[c][1];
      kb[c] = static_cast<uint32_t>(kw[c] >> (2 * lane)) & 3u;
      vb[c] = static_cast<uint32_t>(vw[c] >> (2 * lane)) & 3u;
    }
    if (t + nwarps < ntiles) load_tile(t + nwarps);
    uint64_t m[U][2];
#pragma unroll
    for (int c = 0; c < U; ++c)
#pragma unroll
      for (int j = 0; j < 2; ++j) m[c][j] = ((kb[c] >> j) & 1u) ? sink_lookup<KT, STRAT, UNIQUE>(P.T, ck[c][j]) : 0;
#pragma unroll
    for (int c = 0; c < U; ++c)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        cnt += m[c][j];
        if (m[c][j] && ((vb[c] >> j) & 1u)) {
          sum += static_cast<unsigned long long>(static_cast<int64_t>(cv[c][j])) * m[c][j];
          seen = 1;
        }
      }
  }
  // Rows after the last full tile, one per thread.
  const uint64_t tail0 = ntiles * kTile;
  for (uint64_t r = tail0 + static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < P.n;
       r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const bool kv = !P.kvalid || ((P.kvalid[r >> 6] >> (r & 63)) & 1ull);
    const uint64_t mm = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, keys[r]) : 0;
    cnt += mm;
    if (mm && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * mm;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], cnt);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], seen);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

// Sink with a small register footprint, so that more warps per SM keep the
// probe stream (and, for hashed tables, the random table reads) in flight. A
// warp owns tiles of U x 64 rows (lane i takes rows 2i and 2i+1 of each
// 64-row chunk: one contiguous span per load instruction, one validity word
// per chunk); with PRE the next tile's loads are issued before the current
// tile's lookups. Tile indexes are 32-bit (the host launches it for fewer
// than 2^31 tiles).
template <typename KT, typename VT, int STRAT, bool UNIQUE, int U, bool PRE, int MINB, bool BLOOM = false>
__global__ void __launch_bounds__(256, MINB) probe_sink_lean_kernel(const SinkK P) {
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t keep_pol = STRAT == QEG_JOIN_HASH ? evict_last_policy() : 0;
  constexpr uint32_t kTile = 64u * U;
  const uint32_t ntiles = static_cast<uint32_t>(P.n / kTile);
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // Matches per thread fit 32 bits for unique build keys (one per row).
  using Cnt = typename std::conditional<UNIQUE, uint32_t, unsigned long long>::type;
  Cnt cnt = 0;
  uint32_t seen = 0;
  unsigned long long sum = 0;
  KT k[U][2];
  VT v[U][2];
  uint64_t kw[U], vw[U];
  auto load_tile = [&](uint32_t tile) {
    const uint64_t base = static_cast<uint64_t>(tile) * kTile;
#pragma unroll
    for (int c = 0; c < U; ++c) {
      load2(keys + base + c * 64 + 2 * lane, k[c]);
      load2(vals + base + c * 64 + 2 * lane, v[c]);
      kw[c] = P.kvalid ? __ldg(P.kvalid + (base >> 6) + c) : ~0ull;
      vw[c] = P.vvalid ? __ldg(P.vvalid + (base >> 6) + c) : ~0ull;
    }
  };
  auto consume = [&](const KT (&ck)[U][2], const VT (&cv)[U][2], const uint64_t (&ckw)[U], const uint64_t (&cvw)[U]) {
    if constexpr (STRAT == QEG_JOIN_HASH) {
      // Hashed table: the lane's two rows of a chunk are looked up together.
#pragma unroll
      for (int c = 0; c < U; ++c) {
        const bool kv[2] = {((ckw[c] >> (2 * lane)) & 1ull) != 0, ((ckw[c] >> (2 * lane + 1)) & 1ull) != 0};
        uint64_t m[2];
        hashed_lookup2<KT, UNIQUE, BLOOM>(P.T, ck[c], kv, m, keep_pol, P.keep_table);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          cnt += static_cast<Cnt>(m[j]);
          if (m[j] && ((cvw[c] >> (2 * lane + j)) & 1ull)) {
            sum += static_cast<unsigned long long>(static_cast<int64_t>(cv[c][j])) * m[j];
            seen = 1;
          }
        }
      }
    } else {
#pragma unroll
      for (int c = 0; c < U; ++c)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const bool kv = (ckw[c] >> (2 * lane + j)) & 1ull;
          if (STRAT == QEG_JOIN_DENSE && UNIQUE) {
            // Branch-free bitmap probe (a select, not a divergent call).
            const uint64_t s =
                static_cast<uint64_t>(static_cast<int64_t>(ck[c][j])) - static_cast<uint64_t>(P.T.dmin);
            const uint32_t hit =
                (kv && s < P.T.cap) ? static_cast<uint32_t>((__ldg(P.T.bitmap + (s >> 6)) >> (s & 63)) & 1ull) : 0u;
            cnt += hit;
            if (hit && ((cvw[c] >> (2 * lane + j)) & 1ull)) {
              sum += static_cast<unsigned long long>(static_cast<int64_t>(cv[c][j]));
              seen = 1;
            }
          } else {
            const uint64_t m = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, ck[c][j]) : 0;
            cnt += static_cast<Cnt>(m);
            if (m && ((cvw[c] >> (2 * lane + j)) & 1ull)) {
              sum += static_cast<unsigned long long>(static_cast<int64_t>(cv[c][j])) * m;
              seen = 1;
            }
          }
        }
    }
  };
  if (PRE) {
    if (t < ntiles) load_tile(t);
    for (; t < ntiles; t += nwarps) {
      KT ck[U][2];
      VT cv[U][2];
      uint64_t ckw[U], cvw[U];
#pragma unroll
      for (int c = 0; c < U; ++c) {
        ck[c][0] = k[c][0];
        ck[c][1] = k[c][1];
        cv[c][0] = v[c][0];
        cv[c][1] = v[c][1];
        ckw[c] = kw[c];
        cvw[c] = vw[c];
      }
      if (t + nwarps < ntiles) load_tile(t + nwarps);
      consume(ck, cv, ckw, cvw);
    }
  } else {
    for (; t < ntiles; t += nwarps) {
      load_tile(t);
      consume(k, v, kw, vw);
    }
  }
  // Rows after the last full tile, one per thread.
  for (uint64_t r = static_cast<uint64_t>(ntiles) * kTile + static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       r < P.n; r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const bool kv = !P.kvalid || ((P.kvalid[r >> 6] >> (r & 63)) & 1ull);
    const uint64_t mm = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, keys[r]) : 0;
    cnt += static_cast<Cnt>(mm);
    if (mm && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * mm;
      seen = 1;
    }
  }
  unsigned long long c64 = cnt;
  for (int o = 16; o > 0; o >>= 1) {
    c64 += __shfl_down_sync(0xffffffffu, c64, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], c64);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], static_cast<unsigned long long>(seen));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

// cp.async-staged sink. Each warp streams its tiles of 128 rows through a
// private ring of kAsyncStages shared-memory stages filled with 16-byte
// cp.async copies (keys, payloads, and the two validity words per column), so
// kAsyncStages - 1 tiles per warp are in flight without holding registers;
// lane i then takes rows i, i+32, i+64, i+96 of the landed tile.
constexpr int kAsyncStages = 4;
constexpr int kAsyncTile = 128;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <typename KT, typename VT>
constexpr size_t async_stage_bytes() {
  return kAsyncTile * sizeof(KT) + kAsyncTile * sizeof(VT) + 32;
}

template <typename KT, typename VT, int STRAT, bool UNIQUE>
__global__ void __launch_bounds__(256) probe_sink_async_kernel(const SinkK P) {
  extern __shared__ __align__(16) uint8_t async_smem[];
  constexpr size_t KB = kAsyncTile * sizeof(KT), VB = kAsyncTile * sizeof(VT);
  constexpr size_t SB = async_stage_bytes<KT, VT>();
  unsigned long long cnt = 0, sum = 0, seen = 0;
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned warp = threadIdx.x >> 5;
  uint8_t* ring = async_smem + static_cast<size_t>(warp) * kAsyncStages * SB;
  const uint64_t ntiles = P.n / kAsyncTile;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  const uint64_t first = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  auto issue = [&](uint64_t t, int st) {
    uint8_t* sp = ring + st * SB;
    const uint8_t* kg = reinterpret_cast<const uint8_t*>(keys + t * kAsyncTile);
    const uint8_t* vg = reinterpret_cast<const uint8_t*>(vals + t * kAsyncTile);
    for (unsigned c = lane; c < KB / 16; c += 32) cp_async16(sp + c * 16, kg + c * 16);
    for (unsigned c = lane; c < VB / 16; c += 32) cp_async16(sp + KB + c * 16, vg + c * 16);
    uint64_t* w = reinterpret_cast<uint64_t*>(sp + KB + VB);
    if (lane < 2) {
      if (P.kvalid) cp_async8(w + lane, P.kvalid + t * 2 + lane);
      else w[lane] = ~0ull;
    } else if (lane < 4) {
      if (P.vvalid) cp_async8(w + lane, P.vvalid + t * 2 + (lane - 2));
      else w[lane] = ~0ull;
    }
  };
  // Prologue: the first kAsyncStages - 1 tiles of this warp.
#pragma unroll
  for (int st = 0; st < kAsyncStages - 1; ++st) {
    const uint64_t t = first + st * nwarps;
    if (t < ntiles) issue(t, st);
    cp_async_commit();
  }
  int st = 0;
  for (uint64_t t = first; t < ntiles; t += nwarps) {
    const uint64_t tn = t + (kAsyncStages - 1) * nwarps;
    if (tn < ntiles) issue(tn, (st + kAsyncStages - 1) % kAsyncStages);
    cp_async_commit();
    cp_async_wait<kAsyncStages - 1>();  // this thread's copies of tile t have landed
    __syncwarp();                        // and every lane's
    const uint8_t* sp = ring + st * SB;
    const KT* sk = reinterpret_cast<const KT*>(sp);
    const VT* sv = reinterpret_cast<const VT*>(sp + KB);
    const uint64_t* w = reinterpret_cast<const uint64_t*>(sp + KB + VB);
    uint64_t m[4];
    VT v[4];
    bool vok[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const unsigned r = lane + 32 * j;
      const bool kok = (w[r >> 6] >> (r & 63)) & 1ull;
      vok[j] = (w[2 + (r >> 6)] >> (r & 63)) & 1ull;
      v[j] = sv[r];
      m[j] = kok ? sink_lookup<KT, STRAT, UNIQUE>(P.T, sk[r]) : 0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cnt += m[j];
      if (m[j] && vok[j]) {
        sum += static_cast<unsigned long long>(static_cast<int64_t>(v[j])) * m[j];
        seen = 1;
      }
    }
    __syncwarp();  // every lane is done with this stage before it is refilled
    st = (st + 1) % kAsyncStages;
  }
  cp_async_wait<0>();
  // Rows after the last full tile, one per thread.
  const uint64_t tail0 = ntiles * kAsyncTile;
  for (uint64_t r = tail0 + static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < P.n;
       r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const bool kv = !P.kvalid || ((P.kvalid[r >> 6] >> (r & 63)) & 1ull);
    const uint64_t mm = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, keys[r]) : 0;
    cnt += mm;
    if (mm && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * mm;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], cnt);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], seen);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

// ---------------------------------------------------------------------------
// Radix-partitioned COUNT/SUM join (QEG_JOIN_PARTITIONED). A single-key hash
// table puts a key's home slot at the top bits of its hash, so the keys of
// one hash partition (top `bits` bits) occupy one contiguous window of the
// table. The probe side is split into those partitions in one pass (per CTA
// tile: a shared-memory counting sort, one global reservation per partition,
// then coalesced writes of each partition's run), and the ordinary sink then
// streams the partitioned probe rows in order: at any moment the warps probe
// a window of one or two partitions, whose slice of the table stays in L2
// instead of every probe missing to HBM.
// ---------------------------------------------------------------------------
constexpr int kPartTile = 4096;  // probe rows per CTA tile of the scatter

__device__ __forceinline__ uint32_t key_part(uint64_t k, int bits) {
  return static_cast<uint32_t>(single_key_hash(k) >> (64 - bits));
}

template <typename KT>
__device__ __forceinline__ uint64_t sink_word(KT k) {
  return sizeof(KT) == 4 ? static_cast<uint64_t>(static_cast<uint32_t>(k)) : static_cast<uint64_t>(k);
}

struct PartK {
  const void* key;
  const uint64_t* kvalid;  // nullptr: no NULL keys
  const void* val;         // payloads (no NULLs on this path)
  uint64_t n;
  int bits;
  unsigned long long* hist;    // [P] partition sizes (pass 1)
  unsigned long long* cursor;  // [P] next free row of each partition (pass 2)
  uint64_t* okey;              // key words, partition order
  int64_t* oval;               // payloads, partition order
  const uint64_t* bloom;       // the table's Bloom filter: rows that miss it are dropped (nullptr: none)
  int bshift;
};

// Partition of probe key word k, or -1 when the build side's Bloom filter
// rules the key out.
__device__ __forceinline__ int probe_part(const PartK& P, uint64_t k, uint64_t pol) {
  const uint64_t h = single_key_hash(k);
  if (P.bloom) {
    const uint64_t bm = bloom_mask(h);
    if ((ld_keep_l2(P.bloom + (h >> P.bshift), pol) & bm) != bm) return -1;
  }
  return static_cast<int>(h >> (64 - P.bits));
}

// Pass 1: partition sizes (shared-memory histogram per CTA, then reductions).
template <typename KT>
__global__ void __launch_bounds__(512) ppart_hist_kernel(const PartK P) {
  extern __shared__ unsigned int phist[];
  const uint32_t np = 1u << P.bits;
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) phist[i] = 0;
  __syncthreads();
  const KT* keys = static_cast<const KT*>(P.key);
  const uint64_t pol = evict_last_policy();
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n; r += (uint64_t)gridDim.x * blockDim.x) {
    if (P.kvalid && !((__ldg(P.kvalid + (r >> 6)) >> (r & 63)) & 1ull)) continue;
    const int part = probe_part(P, sink_word(__ldg(keys + r)), pol);
    if (part >= 0) atomicAdd(phist + part, 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
    if (phist[i]) atomicAdd(P.hist + i, static_cast<unsigned long long>(phist[i]));
}

// Pass 2: tiles of kPartTile rows are counting-sorted by partition in shared
// memory, each partition's run reserved with one global atomic and written
// contiguously. NULL keys are dropped (they never match).
template <typename KT, typename VT>
__global__ void __launch_bounds__(512) ppart_scatter_kernel(const PartK P) {
  extern __shared__ __align__(16) unsigned char pscratch[];
  const uint32_t np = 1u << P.bits;
  uint64_t* skey = reinterpret_cast<uint64_t*>(pscratch);                 // [kPartTile]
  int64_t* sval = reinterpret_cast<int64_t*>(skey + kPartTile);           // [kPartTile]
  uint16_t* spart = reinterpret_cast<uint16_t*>(sval + kPartTile);        // [kPartTile]
  unsigned int* cnt = reinterpret_cast<unsigned int*>(spart + kPartTile); // [np]
  unsigned int* loff = cnt + np;                                          // [np]
  unsigned long long* gbase = reinterpret_cast<unsigned long long*>(loff + np + (np & 1));  // [np]
  constexpr int kPer = kPartTile / 512;
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const uint64_t pol = evict_last_policy();
  const uint64_t ntiles = (P.n + kPartTile - 1) / kPartTile;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    uint64_t k[kPer];
    int64_t v[kPer];
    uint32_t part[kPer], rank[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const uint64_t r = t * kPartTile + j * 512 + threadIdx.x;
      part[j] = 0xffffffffu;
      if (r < P.n && (!P.kvalid || ((__ldg(P.kvalid + (r >> 6)) >> (r & 63)) & 1ull))) {
        k[j] = sink_word(__ldcs(keys + r));
        v[j] = static_cast<int64_t>(__ldcs(vals + r));
        const int pp = probe_part(P, k[j], pol);
        if (pp >= 0) {
          part[j] = static_cast<uint32_t>(pp);
          rank[j] = atomicAdd(cnt + part[j], 1u);
        }
      }
    }
    __syncthreads();
    // Exclusive scan of the tile's partition counts (one thread per 32 bins,
    // then a scan over the bins' totals by one warp).
    if (threadIdx.x < 32) {
      const uint32_t per = (np + 31) / 32;
      const uint32_t a = threadIdx.x * per, z = min(np, a + per);
      uint32_t sum = 0;
      for (uint32_t i = a; i < z; ++i) sum += cnt[i];
      uint32_t incl = sum;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (threadIdx.x >= static_cast<unsigned>(o)) incl += y;
      }
      uint32_t run = incl - sum;
      for (uint32_t i = a; i < z; ++i) {
        loff[i] = run;
        run += cnt[i];
      }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
      if (cnt[i]) gbase[i] = atomicAdd(P.cursor + i, static_cast<unsigned long long>(cnt[i]));
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      if (part[j] != 0xffffffffu) {
        const uint32_t pos = loff[part[j]] + rank[j];
        skey[pos] = k[j];
        sval[pos] = v[j];
        spart[pos] = static_cast<uint16_t>(part[j]);
      }
    }
    __syncthreads();
    const uint32_t kept = loff[np - 1] + cnt[np - 1];
    for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x) {
      const uint32_t p = spart[i];
      const uint64_t o = gbase[p] + (i - loff[p]);
      P.okey[o] = skey[i];
      P.oval[o] = sval[i];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// TMA-staged sink: the probe columns stream into shared memory through a ring
// of kStages tiles filled by cp.async.bulk (completion on an mbarrier, L2
// evict-first so the stream does not push the table out of L2); all threads
// then do the lookups from shared memory while the next tiles are in flight.
// Thread 0 waits on each tile's mbarrier with a bounded spin and shares the
// outcome through shared memory, so a wait that runs out turns the whole block
// to the drain path together.
// ---------------------------------------------------------------------------
constexpr int kTmaThreads = 512;
constexpr int kTileRows = 4096;
constexpr int kStages = 3;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
// Bounded wait for phase `parity` of `bar`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <typename KT, typename VT>
struct TmaTile {
  KT key[kTileRows];
  VT val[kTileRows];
  uint64_t kvalid[kTileRows / 64];
  uint64_t vvalid[kTileRows / 64];
};

template <typename KT, typename VT, int STRAT, bool UNIQUE>
__global__ void __launch_bounds__(kTmaThreads) probe_sink_tma_kernel(const SinkK P, uint32_t* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  using Tile = TmaTile<KT, VT>;
  Tile* tiles = reinterpret_cast<Tile*>(smem_raw);
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ int s_ok;
  const KT* keys = static_cast<const KT*>(P.key);
  const VT* vals = static_cast<const VT*>(P.val);
  const uint64_t ntiles = P.n / kTileRows;  // full tiles; the rest is handled below
  const uint32_t tx = kTileRows * (sizeof(KT) + sizeof(VT)) + (P.kvalid ? kTileRows / 8 : 0) +
                      (P.vvalid ? kTileRows / 8 : 0);
  uint64_t pol = 0;
  auto issue = [&](uint64_t ti, int s) {
    const uint64_t r0 = ti * kTileRows;
    mbar_arrive_expect_tx(&full[s], tx);
    bulk_g2s(tiles[s].key, keys + r0, kTileRows * sizeof(KT), &full[s], pol);
    bulk_g2s(tiles[s].val, vals + r0, kTileRows * sizeof(VT), &full[s], pol);
    if (P.kvalid) bulk_g2s(tiles[s].kvalid, P.kvalid + r0 / 64, kTileRows / 8, &full[s], pol);
    if (P.vvalid) bulk_g2s(tiles[s].vvalid, P.vvalid + r0 / 64, kTileRows / 8, &full[s], pol);
  };
  if (threadIdx.x == 0) {
    pol = evict_first_policy();
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int s = 0; s < kStages; ++s) {
      const uint64_t ti = blockIdx.x + static_cast<uint64_t>(s) * gridDim.x;
      if (ti < ntiles) issue(ti, s);
    }
  }
  __syncthreads();

  unsigned long long cnt = 0, sum = 0, seen = 0;
  uint64_t it = 0;
  bool ok = true;
  for (uint64_t ti = blockIdx.x; ti < ntiles; ti += gridDim.x, ++it) {
    const int s = static_cast<int>(it % kStages);
    const uint32_t parity = static_cast<uint32_t>((it / kStages) & 1);
    if (threadIdx.x == 0) s_ok = mbar_wait_bounded(&full[s], parity) ? 1 : 0;
    __syncthreads();
    if (!s_ok) {
      ok = false;
      break;
    }
    const Tile& T = tiles[s];
    constexpr int kPer = kTileRows / kTmaThreads;
    uint64_t m[kPer];
    if (STRAT == QEG_JOIN_DENSE) {
      // Two phases so every lookup of the tile is in flight at once.
      uint64_t w[kPer];
      uint32_t b[kPer];
#pragma unroll
      for (int j = 0; j < kPer; ++j) {
        const int r = j * kTmaThreads + threadIdx.x;
        const bool kv = !P.kvalid || ((T.kvalid[r >> 6] >> (r & 63)) & 1ull);
        const uint64_t sl = static_cast<uint64_t>(static_cast<int64_t>(T.key[r])) - static_cast<uint64_t>(P.T.dmin);
        const bool in = kv && sl < P.T.cap;
        b[j] = static_cast<uint32_t>(sl & 63);
        w[j] = in ? (UNIQUE ? __ldg(P.T.bitmap + (sl >> 6)) : __ldg(P.T.cnt + sl)) : 0;
      }
#pragma unroll
      for (int j = 0; j < kPer; ++j) m[j] = UNIQUE ? ((w[j] >> b[j]) & 1ull) : w[j];
    } else {
#pragma unroll
      for (int j = 0; j < kPer; ++j) {
        const int r = j * kTmaThreads + threadIdx.x;
        const bool kv = !P.kvalid || ((T.kvalid[r >> 6] >> (r & 63)) & 1ull);
        m[j] = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, T.key[r]) : 0;
      }
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int r = j * kTmaThreads + threadIdx.x;
      if (m[j]) {
        cnt += m[j];
        if (!P.vvalid || ((T.vvalid[r >> 6] >> (r & 63)) & 1ull)) {
          sum += static_cast<unsigned long long>(static_cast<int64_t>(T.val[r])) * m[j];
          seen = 1;
        }
      }
    }
    __syncthreads();  // stage s is free again
    if (threadIdx.x == 0) {
      const uint64_t nt = ti + static_cast<uint64_t>(kStages) * gridDim.x;
      if (nt < ntiles) issue(nt, s);
    }
  }
  if (!ok) {
    // A wait ran out: report it, then let the copies this block still has in
    // flight land (bounded) before the block's shared memory is released.
    if (threadIdx.x == 0) {
      atomicOr(err, kDevSpinTimeout);
      for (uint64_t k = it; k < it + kStages; ++k) {
        const uint64_t tk = blockIdx.x + k * gridDim.x;
        if (tk >= ntiles) break;
        mbar_wait_bounded(&full[k % kStages], static_cast<uint32_t>((k / kStages) & 1));
      }
    }
    __syncthreads();
    return;
  }
  // Rows after the last full tile.
  const uint64_t rest0 = ntiles * kTileRows;
  for (uint64_t r = rest0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const bool kv = !P.kvalid || ((P.kvalid[r >> 6] >> (r & 63)) & 1ull);
    const uint64_t m = kv ? sink_lookup<KT, STRAT, UNIQUE>(P.T, keys[r]) : 0;
    cnt += m;
    if (m && (!P.vvalid || ((P.vvalid[r >> 6] >> (r & 63)) & 1ull))) {
      sum += static_cast<unsigned long long>(static_cast<int64_t>(vals[r])) * m;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], cnt);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], seen);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

// The COUNT(*) / SUM(payload) sink for any key/payload type or alignment.
template <int STRAT, bool UNIQUE>
__global__ void __launch_bounds__(512) probe_count_sum_kernel(const ProbeK P) {
  unsigned long long cnt = 0, sum = 0, seen = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P.n; p += stride) {
    if (!col_valid(P.key[0], p)) continue;
    uint64_t m = 0;
    if (STRAT == QEG_JOIN_DENSE) {
      const int64_t v = int_value(P.key[0], p);
      const uint64_t s = static_cast<uint64_t>(v) - static_cast<uint64_t>(P.T.dmin);
      if (s < P.T.cap) {
        if (UNIQUE) m = (__ldg(P.T.bitmap + (s >> 6)) >> (s & 63)) & 1ull;
        else m = __ldg(P.T.cnt + s);
      }
    } else {
      uint64_t w[1];
      w[0] = key_word(P.key[0], p);
      const int64_t s = hash_slot<false>(P.T, w, single_key_hash(w[0]), P.err);
      if (s >= 0) m = (UNIQUE && static_cast<uint64_t>(s) != P.T.cap) ? 1 : __ldg(P.T.cnt + s);
    }
    if (m == 0) continue;
    cnt += m;
    if (col_valid(P.val, p)) {
      sum += static_cast<unsigned long long>(int_value(P.val, p)) * m;
      seen = 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    seen |= __shfl_down_sync(0xffffffffu, seen, o);
  }
  __shared__ unsigned long long s_acc[3];
  if (threadIdx.x == 0) s_acc[0] = s_acc[1] = s_acc[2] = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], cnt);
    atomicAdd(&s_acc[1], sum);
    atomicOr(&s_acc[2], seen);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_acc[0]) atomicAdd(P.acc + 0, s_acc[0]);
    if (s_acc[1]) atomicAdd(P.acc + 1, s_acc[1]);
    if (s_acc[2]) atomicOr(P.acc + 2, s_acc[2]);
  }
}

__global__ void probe_count_kernel(const ProbeK P) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P.n; p += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t w[kMaxKeys], h;
    uint32_t m = 0;
    if (load_key(P.key, P.nkeys, p, w, h)) {
      const int64_t s = probe_slot(P.T, P.key, p, w, h, P.err);
      if (s >= 0) m = P.T.cnt[s];
    }
    if (m == 0 && P.left) m = 1;
    P.counts[p] = m;
  }
}

__global__ void probe_emit_kernel(const ProbeK P) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P.n; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = P.counts[p];
    if (m == 0) continue;
    uint64_t o = P.starts[p];
    uint64_t w[kMaxKeys], h;
    int64_t s = -1;
    if (load_key(P.key, P.nkeys, p, w, h)) s = probe_slot(P.T, P.key, p, w, h, P.err);
    if (s < 0 || P.T.cnt[s] == 0) {  // LEFT join, unmatched: one row, build side NULL
      P.out_probe[o] = static_cast<uint32_t>(p);
      P.out_build[o] = kNullRow;
      continue;
    }
    const uint64_t b = P.T.off[s];
    for (uint32_t t = 0; t < m; ++t) {
      P.out_probe[o + t] = static_cast<uint32_t>(p);
      P.out_build[o + t] = P.T.rows[b + t];
    }
  }
}

// ---- as-of join (tsx/asof.cpp) ---------------------------------------------
// Build: every build row becomes an item (partition slot, timestamp - tmin,
// row); rows with a NULL key or a NULL timestamp get the sentinel slot
// `nslots` and sort after every partition (they never match,
// tsx/asof.cpp:211-216). After a stable sort by (slot, timestamp) each
// partition is one timestamp-ascending run whose equal timestamps keep the
// build order, like the reference's sorted build lists (tsx/asof.cpp:158-219).
struct AsofItemsK {
  DevCol key[kMaxKeys];
  int nkeys;
  DevCol ts;
  uint64_t n;
  JTable T;
  uint32_t nslots;
  int64_t tmin;
  uint64_t* lo;
  uint32_t* hi;
  uint32_t* val;
  uint32_t* err;
};

// Partition slot of row p: 0 without keys, -1 for a NULL key or a key the
// table does not hold. A dense table needs no hash.
__device__ __forceinline__ int64_t asof_slot(const DevCol* key, int nkeys, const JTable& T, uint64_t p,
                                             uint32_t* err) {
  if (nkeys == 0) return 0;
  if (T.strategy == QEG_JOIN_DENSE) {
    if (!col_valid(key[0], p)) return -1;
    const int64_t v = dense_value(key[0], p);
    const uint64_t s = static_cast<uint64_t>(v) - static_cast<uint64_t>(T.dmin);
    return (v < T.dmin || s >= T.cap) ? -1 : static_cast<int64_t>(s);
  }
  uint64_t w[kMaxKeys], h;
  return load_key(key, nkeys, p, w, h) ? probe_slot(T, key, p, w, h, err) : -1;
}

__global__ void asof_items_kernel(const AsofItemsK P) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < P.n; r += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t slot = P.nslots;
    uint64_t rel = 0;
    if (col_valid(P.ts, r)) {
      const int64_t s = asof_slot(P.key, P.nkeys, P.T, r, P.err);
      if (s >= 0) {
        slot = static_cast<uint32_t>(s);
        rel = static_cast<uint64_t>(int_value(P.ts, r)) - static_cast<uint64_t>(P.tmin);
      }
    }
    P.lo[r] = rel;
    P.hi[r] = slot;
    P.val[r] = static_cast<uint32_t>(r);
  }
}

// Sets *unsorted when some row's time is below the previous row's (times
// without NULLs): a build side in time order only needs sorting by slot.
__global__ void time_order_kernel(DevCol ts, uint64_t n, unsigned int* unsorted) {
  bool bad = false;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < n; i += (uint64_t)gridDim.x * blockDim.x)
    bad |= int_value(ts, i) > int_value(ts, i + 1);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(unsorted, 1u);
}

// Partition runs of the sorted items: run [beg[s], end[s]) of every slot that
// has matchable rows (the arrays start zeroed: absent slots are empty), and
// the sample array (every kAsofSample-th sorted time) of the two-level search.
constexpr int kAsofSample = 32;

__global__ void asof_runs_kernel(const uint32_t* __restrict__ hi, const uint64_t* __restrict__ lo, uint64_t n,
                                 uint32_t nslots, uint2* __restrict__ runs, uint64_t* __restrict__ samp) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = hi[i];
    if (i % kAsofSample == 0) samp[i / kAsofSample] = lo[i];
    if (s >= nslots) continue;
    if (i == 0 || hi[i - 1] != s) runs[s].x = static_cast<uint32_t>(i);
    if (i + 1 == n || hi[i + 1] != s) runs[s].y = static_cast<uint32_t>(i + 1);
  }
}

// Probe: a probe row with non-NULL keys and timestamp t finds its partition,
// then the last build timestamp <= t by binary search over the partition's
// run (the reference walks a cursor over the sorted probe side to the same
// row, tsx/asof.cpp:269-296); with a tolerance the match is kept only when
// t - tb <= tolerance in uint64 arithmetic (tsx/asof.cpp:283-293). The search
// runs in two levels: over the samples inside the run (every 32nd sorted
// time, small enough to stay in L2), then over the <= 32 times between two
// samples (one or two cache lines).
struct AsofProbeK {
  DevCol key[kMaxKeys];
  int nkeys;
  DevCol ts;
  uint64_t n;
  JTable T;
  int64_t tmin;
  const uint64_t* ats;   // sorted timestamps - tmin
  const uint32_t* arow;  // build rows in the same order
  const uint2* aruns;  // partition runs: [aruns[s].x, aruns[s].y)
  const uint64_t* asamp;  // ats[i * kAsofSample]
  int hint_bits;          // log2 of the shared-memory hint table's entries
  int left, tol_set;
  uint64_t tol;
  uint32_t* match;
  uint32_t* counts;
  uint32_t* out_probe;
  uint32_t* out_build;
  uint32_t* err;
};

// First position in [b, e) whose time is > rel (e when none): a search that
// starts at a hint inside the run and gallops outward (1, 2, 4, ...
// positions) before a binary search of the bracket -- a few loads in the same
// cache lines when the hint is close, as it is for a probe side in time order.
__device__ __forceinline__ uint32_t asof_gallop(const uint64_t* __restrict__ ats, uint32_t b, uint32_t e,
                                                uint32_t h, uint64_t rel) {
  // Positions are 32-bit; the step and the sums that could pass 2^32 are not.
  uint32_t lo, hi;
  if (ats[h] <= rel) {
    lo = h + 1;
    uint64_t d = 1;
    while (lo + d - 1 < e && ats[lo + d - 1] <= rel) {
      lo += static_cast<uint32_t>(d);
      d <<= 1;
    }
    hi = static_cast<uint32_t>(lo + d - 1 < e ? lo + d - 1 : e);
  } else {
    hi = h;
    uint64_t d = 1;
    while (hi >= b + d && ats[hi - d] > rel) {
      hi -= static_cast<uint32_t>(d);
      d <<= 1;
    }
    lo = hi >= b + d ? static_cast<uint32_t>(hi - d + 1) : b;
  }
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (ats[mid] <= rel) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// First position in [b, e) whose time is > rel, from scratch: over the
// samples inside the run (every kAsofSample-th sorted time, small enough to
// stay in L2), then over the <= kAsofSample times between two samples.
__device__ __forceinline__ uint32_t asof_sampled(const AsofProbeK& P, uint32_t b, uint32_t e, uint64_t rel) {
  uint32_t lo = b, hi = e;
  const uint32_t ib = static_cast<uint32_t>((static_cast<uint64_t>(b) + kAsofSample - 1) / kAsofSample);
  const uint32_t ie = (e - 1) / kAsofSample;
  if (ib <= ie) {
    uint32_t l = ib, r = ie + 1;
    while (l < r) {
      const uint32_t mid = l + ((r - l) >> 1);
      if (P.asamp[mid] <= rel) l = mid + 1;
      else r = mid;
    }
    if (l > ib) lo = (l - 1) * kAsofSample + 1;
    if (l <= ie) hi = l * kAsofSample;
  }
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (P.ats[mid] <= rel) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Each CTA walks one contiguous range of probe rows and keeps, per slot (a
// direct-mapped table in shared memory), the position its last search ended
// at: on a probe side in time order the next search of that slot starts a few
// positions away. A hint is only a starting point (any position of the run
// gives the same answer), so races between warps on it are harmless.
// 1024 entries: measured best on 200M trades x 50M quotes over 10k symbols
// (probe 11.7 ms; 12.8 ms with 2048 entries, 20.2 ms with 4096: a bigger table
// keeps stale positions of rarely seen symbols, whose gallops cost more than
// the L2-resident sampled search a miss falls back to). QEG_ASOF_HINT_BITS
// (6..12) overrides it.
constexpr int kAsofHintBits = 10;

__global__ void __launch_bounds__(256) asof_probe_kernel(const AsofProbeK P) {
  extern __shared__ uint32_t hmem[];
  const int nh = 1 << P.hint_bits;
  uint32_t* hslot = hmem;
  uint32_t* hpos = hmem + nh;
  for (int i = threadIdx.x; i < nh; i += blockDim.x) hslot[i] = 0xffffffffu;
  __syncthreads();
  const uint64_t chunk = ((P.n + gridDim.x - 1) / gridDim.x + 255) / 256 * 256;
  const uint64_t c0 = blockIdx.x * chunk;
  const uint64_t c1 = c0 + chunk < P.n ? c0 + chunk : P.n;
  for (uint64_t p = c0 + threadIdx.x; p < c1; p += blockDim.x) {
    uint32_t m = kNullRow;
    if (col_valid(P.ts, p)) {
      const int64_t s = asof_slot(P.key, P.nkeys, P.T, p, P.err);
      if (s >= 0) {
        const int64_t t = int_value(P.ts, p);
        const uint2 run = P.aruns[s];
        const uint32_t b = run.x, e = run.y;
        if (e > b && t >= P.tmin) {
          const uint64_t rel = static_cast<uint64_t>(t) - static_cast<uint64_t>(P.tmin);
          const uint32_t hi = (static_cast<uint32_t>(s) * 2654435761u) >> (32 - P.hint_bits);
          const uint32_t hp = hpos[hi];
          const bool hit = hslot[hi] == static_cast<uint32_t>(s) && hp >= b && hp < e;
          const uint32_t j = hit ? asof_gallop(P.ats, b, e, hp, rel) : asof_sampled(P, b, e, rel);
          const uint32_t nh = static_cast<uint32_t>(j < e ? j : e - 1);
          hslot[hi] = static_cast<uint32_t>(s);
          hpos[hi] = nh;
          if (j > b && (!P.tol_set || rel - P.ats[j - 1] <= P.tol)) m = P.arow[j - 1];
        }
      }
    }
    if (P.left) {
      P.out_probe[p] = static_cast<uint32_t>(p);
      P.out_build[p] = m;
    } else {
      P.match[p] = m;
      P.counts[p] = m != kNullRow ? 1u : 0u;
    }
  }
}

__global__ void asof_emit_kernel(const AsofProbeK P, const uint64_t* __restrict__ starts) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P.n; p += (uint64_t)gridDim.x * blockDim.x) {
    if (!P.counts[p]) continue;
    const uint64_t o = starts[p];
    P.out_probe[o] = static_cast<uint32_t>(p);
    P.out_build[o] = P.match[p];
  }
}

// out[k] = src[idx[k]] (width bytes), valid[k] from the source, NULL where
// idx[k] is kNullRow. Source validity is either a bitmap (probe columns) or a
// byte per row (build store).
__global__ void gather_kernel(const void* __restrict__ src, const uint64_t* __restrict__ src_bits,
                              const uint8_t* __restrict__ src_bytes, const int32_t* __restrict__ code_map, int width,
                              const uint32_t* __restrict__ idx, uint64_t n, void* __restrict__ out,
                              uint8_t* __restrict__ valid) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = idx[k];
    if (r == kNullRow) {
      valid[k] = 0;
      if (width == 8) static_cast<uint64_t*>(out)[k] = 0;
      else if (width == 4) static_cast<uint32_t*>(out)[k] = 0;
      else static_cast<uint8_t*>(out)[k] = 0;
      continue;
    }
    uint8_t ok = 1;
    if (src_bits) ok = (src_bits[r >> 6] >> (r & 63)) & 1ull;
    else if (src_bytes) ok = src_bytes[r];
    valid[k] = ok;
    if (width == 8) static_cast<uint64_t*>(out)[k] = static_cast<const uint64_t*>(src)[r];
    else if (code_map) static_cast<int32_t*>(out)[k] = ok ? code_map[static_cast<const int32_t*>(src)[r]] : 0;
    else if (width == 4) static_cast<uint32_t*>(out)[k] = static_cast<const uint32_t*>(src)[r];
    else static_cast<uint8_t*>(out)[k] = static_cast<const uint8_t*>(src)[r];
  }
}

// Device outputs: the same gather written straight into the caller's column,
// validity packed on the fly (a warp covers 64 rows and makes one word from
// two ballots; padding bits set), so an output row is written once.
__global__ void gather_out_kernel(const void* __restrict__ src, const uint64_t* __restrict__ src_bits,
                                  const uint8_t* __restrict__ src_bytes, const int32_t* __restrict__ code_map,
                                  int width, const uint32_t* __restrict__ idx, uint64_t n, void* __restrict__ out,
                                  uint64_t* __restrict__ out_words, unsigned int* __restrict__ any_null) {
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t nw = (n + 63) / 64;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t w = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w < nw; w += nwarps) {
    unsigned half[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint64_t k = w * 64 + h * 32 + lane;
      bool ok = true;  // padding rows count as valid
      if (k < n) {
        const uint32_t r = idx[k];
        ok = r != kNullRow;
        if (ok) {
          if (src_bits) ok = (src_bits[r >> 6] >> (r & 63)) & 1ull;
          else if (src_bytes) ok = src_bytes[r];
        }
        if (width == 8) {
          static_cast<uint64_t*>(out)[k] = r == kNullRow ? 0 : static_cast<const uint64_t*>(src)[r];
        } else if (width == 4) {
          uint32_t v = 0;
          if (r != kNullRow) {
            v = static_cast<const uint32_t*>(src)[r];
            if (code_map) v = ok ? static_cast<uint32_t>(code_map[static_cast<int32_t>(v)]) : 0;
          }
          static_cast<uint32_t*>(out)[k] = v;
        } else {
          static_cast<uint8_t*>(out)[k] = r == kNullRow ? 0 : static_cast<const uint8_t*>(src)[r];
        }
      }
      half[h] = __ballot_sync(0xffffffffu, ok);
    }
    if (lane == 0) {
      const uint64_t word = static_cast<uint64_t>(half[0]) | (static_cast<uint64_t>(half[1]) << 32);
      if (out_words) out_words[w] = word;
      if (word != ~0ull) atomicOr(any_null, 1u);
    }
  }
}

// All output columns in one pass: a warp loads the probe and build row
// indices of its 64 output rows once, then writes every column's values and
// validity word for them (the per-column kernel above re-reads the indices
// once per column).
constexpr int kMaxGatherCols = 32;

struct GatherCol {
  const void* src;
  const uint64_t* bits;
  const uint8_t* bytes;
  const int32_t* code_map;
  void* out;
  uint64_t* words;
  int width;
  int side;  // 0 probe, 1 build
  int flag;  // index of the column's NULL flag
};

struct GatherK {
  GatherCol c[kMaxGatherCols];
  int ncols;
  const uint32_t* idx[2];
  uint64_t n;
  unsigned int* flags;  // per column: set when a NULL was written
};

__device__ __forceinline__ bool gather_one(const GatherCol& c, uint32_t r, uint64_t k) {
  bool ok = r != kNullRow;
  if (ok) {
    if (c.bits) ok = (c.bits[r >> 6] >> (r & 63)) & 1ull;
    else if (c.bytes) ok = c.bytes[r];
  }
  if (c.width == 8) {
    static_cast<uint64_t*>(c.out)[k] = r == kNullRow ? 0 : static_cast<const uint64_t*>(c.src)[r];
  } else if (c.width == 4) {
    uint32_t v = 0;
    if (r != kNullRow) {
      v = static_cast<const uint32_t*>(c.src)[r];
      if (c.code_map) v = ok ? static_cast<uint32_t>(c.code_map[static_cast<int32_t>(v)]) : 0;
    }
    static_cast<uint32_t*>(c.out)[k] = v;
  } else {
    static_cast<uint8_t*>(c.out)[k] = r == kNullRow ? 0 : static_cast<const uint8_t*>(c.src)[r];
  }
  return ok;
}

__global__ void __launch_bounds__(256) gather_cols_kernel(const GatherK P) {
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t nw = (P.n + 63) / 64;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t w = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w < nw; w += nwarps) {
    const uint64_t k0 = w * 64 + lane, k1 = k0 + 32;
    const bool in0 = k0 < P.n, in1 = k1 < P.n;
    uint32_t r[2][2];
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      r[sd][0] = in0 ? P.idx[sd][k0] : kNullRow;
      r[sd][1] = in1 ? P.idx[sd][k1] : kNullRow;
    }
    for (int c = 0; c < P.ncols; ++c) {
      const GatherCol& col = P.c[c];
      const int sd = col.side;
      const bool ok0 = in0 ? gather_one(col, r[sd][0], k0) : true;
      const bool ok1 = in1 ? gather_one(col, r[sd][1], k1) : true;
      const unsigned b0 = __ballot_sync(0xffffffffu, ok0), b1 = __ballot_sync(0xffffffffu, ok1);
      if (lane == 0) {
        const uint64_t word = static_cast<uint64_t>(b0) | (static_cast<uint64_t>(b1) << 32);
        if (col.words) col.words[w] = word;
        if (word != ~0ull) atomicOr(P.flags + col.flag, 1u);
      }
    }
  }
}

// Validity words copied from an aligned source range: padding bits of the
// last word set, and the column's NULL flag raised when any bit is clear.
__global__ void words_finish_kernel(uint64_t* __restrict__ words, uint64_t nw, uint64_t count,
                                    unsigned int* __restrict__ flag) {
  bool null_seen = false;
  const uint64_t step = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nw; i += step) {
    uint64_t w = words[i];
    if (i + 1 == nw && (count & 63)) {
      w |= ~0ull << (count & 63);
      words[i] = w;
    }
    null_seen |= w != ~0ull;
  }
  if (__any_sync(0xffffffffu, null_seen) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// Appends a batch column into the build store: values are copied, validity is
// expanded to a byte per row; STR codes are translated to value ids.
// RANGE (the single integer key of a build): the same pass also folds the
// key's smallest and largest value and its non-NULL count into range[0..2]
// (order-preserving encodings; one set of atomics per CTA), so the dense /
// hash decision needs no separate pass over the key.
template <bool RANGE>
__global__ void store_append_kernel(DevCol c, uint64_t n, int width, void* __restrict__ dst,
                                    uint8_t* __restrict__ dvalid, unsigned long long* __restrict__ range) {
  unsigned long long mn = ~0ull, mx = 0, cnt = 0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    const bool ok = col_valid(c, r);
    dvalid[r] = ok ? 1 : 0;
    if (c.type == kSTR) {
      static_cast<int32_t*>(dst)[r] = ok ? static_cast<int32_t>(int_value(c, r)) : 0;
    } else if (width == 8) {
      static_cast<uint64_t*>(dst)[r] = __ldg(static_cast<const unsigned long long*>(c.data) + r);
    } else if (width == 4) {
      static_cast<uint32_t*>(dst)[r] = __ldg(static_cast<const unsigned int*>(c.data) + r);
    } else {
      static_cast<uint8_t*>(dst)[r] = __ldg(static_cast<const uint8_t*>(c.data) + r);
    }
    if (RANGE && ok) {
      const unsigned long long e = enc_i64(int_value(c, r));
      mn = e < mn ? e : mn;
      mx = e > mx ? e : mx;
      ++cnt;
    }
  }
  if (!RANGE) return;
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  }
  __shared__ unsigned long long smn[32], smx[32], scn[32];
  const unsigned warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    smn[warp] = mn;
    smx[warp] = mx;
    scn[warp] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned w = 1; w < nwarps; ++w) {
      mn = min(mn, smn[w]);
      mx = max(mx, smx[w]);
      cnt += scn[w];
    }
    if (cnt) {
      atomicMin(range + 0, mn);
      atomicMax(range + 1, mx);
      atomicAdd(range + 2, cnt);
    }
  }
}

uint64_t next_pow2(uint64_t v) {
  uint64_t c = 1;
  while (c < v) c <<= 1;
  return c;
}

bool dense_capable(int32_t t) { return t == QEG_I32 || t == QEG_I64 || t == QEG_TS || t == QEG_BOOL || t == QEG_STR; }

}  // namespace

struct JoinState {
  qeg_ctx* ctx = nullptr;
  std::vector<int32_t> ptypes, btypes;
  std::vector<uint32_t> pkeys, bkeys;
  int32_t join_type = QEG_INNER;
  qeg_join_config cfg{};
  double est_distinct = 0;  // distinct build keys the hash table was sized from (0: row count)
  int32_t rebuilds = 0;     // estimate-sized tables that overflowed and were rebuilt

  // build store
  std::vector<DevBuf> bvals, bvalid;
  uint64_t nbuild = 0, bcap = 0;
  bool built = false;

  // table
  int strategy = QEG_JOIN_HASH;
  DevBuf keys, cnt, off, rows, bitmap;
  DevBuf bloom;  // hashed single-key tables larger than kBloomMinTableBytes
  int bloom_shift = 64;
  uint64_t cap = 0, distinct = 0, nonnull = 0;
  int64_t dmin = 0;
  int unique = 1;

  // radix-partitioned probe (QEG_JOIN_PARTITIONED)
  int part_bits = 0;

  // last probe batch
  std::vector<StagedCol> probe_staged;
  DevBuf counts, starts, out_probe, out_build;
  uint64_t nout = 0;

  // count/sum sink totals
  DevBuf acc;
  bool acc_init = false;

  // as-of join (qeg_asof_create): time columns, tolerance, and the build side
  // sorted by (partition slot, timestamp)
  bool asof = false;
  bool probe_identity = false;  // output row k of the last probe is probe row k (LEFT as-of)
  uint32_t ptime = 0, btime = 0;
  int32_t tol_set = 0;
  int64_t tol = 0;
  int64_t tmin = 0;
  uint32_t aslots = 0;
  DevBuf ats, arow, aruns, asamp, tbits, amatch;
  DevBuf krange;  // single integer key: [min enc, max enc, non-NULL count] over the appended batches
  void asof_build();
  void asof_probe(uint64_t n);

  JTable table() const {
    JTable T{};
    // A partitioned join probes the same global hash table.
    T.strategy = strategy == QEG_JOIN_PARTITIONED ? QEG_JOIN_HASH : strategy;
    int lg = 0;
    while ((1ull << lg) < cap && lg < 63) ++lg;
    T.shift = 64 - lg;
    T.nkeys = static_cast<int>(bkeys.size());
    T.kw = bkeys.size() == 1 ? 1 : 1 + static_cast<int>(bkeys.size());
    T.keys = keys.get<uint64_t>();
    T.cap = cap;
    T.dmin = dmin;
    T.cnt = cnt.get<uint32_t>();
    T.off = off.get<uint64_t>();
    T.rows = rows.get<uint32_t>();
    T.bitmap = bitmap.get<uint64_t>();
    T.unique = unique;
    T.bloom = bloom.get<uint64_t>();
    T.bshift = bloom_shift;
    return T;
  }

  void append(const qeg_column* cols, int ncols) {
    require(!built, "build() after build_finish()");
    require(ncols == static_cast<int>(btypes.size()), "build batch column count does not match the schema");
    const uint64_t n = cols[0].len;
    for (int c = 0; c < ncols; ++c) {
      require(cols[c].type == btypes[c], "build batch column type does not match the schema");
      require(cols[c].len == n, "build batch columns differ in length");
    }
    require(nbuild + n < 0xffffffffull, "the build side holds at most 2^32-2 rows");
    if (n == 0) return;
    if (nbuild + n > bcap) {
      const uint64_t ncap = std::max<uint64_t>(nbuild + n, std::max<uint64_t>(bcap * 2, 4096));
      for (int c = 0; c < ncols; ++c) {
        DevBuf v(ncap * type_width(btypes[c]), ctx->stream), ok(ncap, ctx->stream);
        if (nbuild) {
          QEG_CUDA(cudaMemcpyAsync(v.get(), bvals[c].get(), nbuild * type_width(btypes[c]), cudaMemcpyDeviceToDevice,
                                   ctx->stream));
          QEG_CUDA(cudaMemcpyAsync(ok.get(), bvalid[c].get(), nbuild, cudaMemcpyDeviceToDevice, ctx->stream));
        }
        bvals[c] = std::move(v);
        bvalid[c] = std::move(ok);
      }
      bcap = ncap;
    }
    bool host_input = false;
    const int range_col = (bkeys.size() == 1 && dense_capable(btypes[bkeys[0]])) ? static_cast<int>(bkeys[0]) : -1;
    if (range_col >= 0 && !krange.get()) {
      krange.alloc(24, ctx->stream);  // {min = ~0, max = 0, count = 0}
      QEG_CUDA(cudaMemsetAsync(krange.get(), 0xff, 8, ctx->stream));
      QEG_CUDA(cudaMemsetAsync(krange.get<uint8_t>() + 8, 0, 16, ctx->stream));
    }
    for (int c = 0; c < ncols; ++c) {
      StagedCol s;
      stage_column(ctx, cols[c], s);
      host_input = host_input || s.data.get() || s.validity.get() || s.code_map.get();
      const int w = static_cast<int>(type_width(btypes[c]));
      if (c == range_col)
        store_append_kernel<true><<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(
            s.dev, n, w, bvals[c].get<uint8_t>() + nbuild * w, bvalid[c].get<uint8_t>() + nbuild,
            krange.get<unsigned long long>());
      else
        store_append_kernel<false><<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(
            s.dev, n, w, bvals[c].get<uint8_t>() + nbuild * w, bvalid[c].get<uint8_t>() + nbuild, nullptr);
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
    }
    // Host inputs: their copies must finish before the call returns (the
    // caller may reuse its buffers). Staged device copies are freed in stream
    // order, after the kernels that read them.
    if (host_input) QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    nbuild += n;
  }

  // Key columns of the build store as kernel columns (validity as a byte array
  // is exposed through a bitmap-free path: keys are re-read with col_valid, so
  // the store keeps a packed bitmap per key column).
  std::vector<DevBuf> key_bits;
  DevCol store_key(int j) {
    DevCol c{};
    c.type = btypes[bkeys[j]] == QEG_STR ? QEG_I32 : btypes[bkeys[j]];  // STR stored as value ids
    c.data = bvals[bkeys[j]].get();
    c.validity = key_bits[j].get<uint64_t>();
    c.all_valid = 0;
    c.code_map = nullptr;
    return c;
  }

  void finish_build();
  void build_hash(BuildK& P, uint64_t want_cap = 0);
  uint64_t slots() const {
    return strategy == QEG_JOIN_DENSE ? cap : (bkeys.size() == 1 ? cap + 1 : cap);
  }
  void alloc_counts() {
    cnt.alloc(slots() * 4, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(cnt.get(), 0, slots() * 4, ctx->stream));
  }
  BuildK build_params(DevBuf& scratch);
  void count_rows();
  void ensure_csr();
  bool csr_built = false;
  bool counts_ready = false;  // cnt holds every slot's build row count
};

namespace {

// Validity bytes -> 64-bit LSB-first words: a warp turns 64 bytes into one
// word with two ballots.
__global__ void bytes_to_bits_kernel(const uint8_t* __restrict__ b, uint64_t n, uint64_t* __restrict__ w) {
  const uint64_t nw = (n + 63) / 64;
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t i = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; i < nw; i += nwarps) {
    const uint64_t r = i * 64 + lane;
    const unsigned lo = __ballot_sync(0xffffffffu, r < n && b[r]);
    const unsigned hi = __ballot_sync(0xffffffffu, r + 32 < n && b[r + 32]);
    if (lane == 0) w[i] = static_cast<uint64_t>(lo) | (static_cast<uint64_t>(hi) << 32);
  }
}

}  // namespace

void JoinState::finish_build() {
  require(!built, "build_finish() called twice");
  built = true;
  const int nk = static_cast<int>(bkeys.size());
  if (asof && nk == 0) {  // one global partition: no table
    asof_build();
    return;
  }
  key_bits.clear();
  for (int j = 0; j < nk; ++j) {
    key_bits.emplace_back(((nbuild + 63) / 64 + 1) * 8, ctx->stream);
    if (nbuild) {
      bytes_to_bits_kernel<<<grid_for(ctx, (nbuild / 64 + 1) * 32, 256, 8), 256, 0, ctx->stream>>>(
          bvalid[bkeys[j]].get<uint8_t>(), nbuild, key_bits[j].get<uint64_t>());
      ctx->launches++;
    }
  }
  BuildK P{};
  P.nkeys = nk;
  for (int j = 0; j < nk; ++j) P.key[j] = store_key(j);
  P.n = nbuild;
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());

  // Strategy: dense when one integer key spans a small range; otherwise one
  // global hash table, or the radix-partitioned join when asked for.
  strategy = QEG_JOIN_HASH;
  nonnull = nbuild;
  if (nk == 1 && dense_capable(btypes[bkeys[0]]) && nbuild > 0 &&
      (cfg.strategy == QEG_JOIN_AUTO || cfg.strategy == QEG_JOIN_DENSE)) {
    // The key's range was folded in while the batches were appended.
    unsigned long long r[3];
    QEG_CUDA(cudaMemcpyAsync(r, krange.get(), 24, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    nonnull = r[2];
    if (r[2] > 0) {
      const uint64_t range = (r[1] - r[0]) + 1;  // encodings preserve order; difference = value range
      if (range != 0 && range <= 4 * r[2] + 64 && range < (1ull << 32)) {
        strategy = QEG_JOIN_DENSE;
        dmin = dec_i64(r[0]);
        cap = range;
      }
    }
    if (strategy != QEG_JOIN_DENSE && cfg.strategy == QEG_JOIN_DENSE) strategy = QEG_JOIN_HASH;
  }
  DevBuf dup(16, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(dup.get(), 0, 16, ctx->stream));
  P.dup = dup.get<uint32_t>();
  P.distinct = reinterpret_cast<unsigned long long*>(dup.get<uint8_t>() + 8);
  const unsigned g = grid_for(ctx, nbuild, 256, 8);
  if (strategy == QEG_JOIN_DENSE) {
    // One bit per key value; atomicOr's old word reveals duplicates.
    bitmap.alloc(((cap + 63) / 64) * 8, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(bitmap.get(), 0, ((cap + 63) / 64) * 8, ctx->stream));
    P.T = table();
    if (nbuild && !asof) {  // the as-of join maps keys to slots only
      dense_mark_kernel<<<g, 256, 0, ctx->stream>>>(P, bitmap.get<unsigned long long>());
      const uint64_t nw = (cap + 63) / 64;
      popc_kernel<<<grid_for(ctx, nw, 256, 8), 256, 0, ctx->stream>>>(bitmap.get<unsigned long long>(), nw,
                                                                       P.distinct);
      ctx->launches += 2;
      QEG_CUDA(cudaGetLastError());
    }
  } else {
    P.no_count = asof ? 1 : 0;
    uint64_t want_cap = 0;
    est_distinct = 0;
    if (cfg.sizing == QEG_SIZE_LEARNED && nk == 1 && !asof && nbuild >= kJoinSketchMinRows) {
      // Table size from the estimated distinct build keys (the learned
      // estimator, or the classic one without weights).
      SketchResult sk;
      sketch_key_column(ctx, store_key(0), nullptr, nbuild, nbuild, 1u << 20, 0, sk);
      double g = 0, share = 0;
      if (!learned_estimate(ctx, sk, &g, &share)) g = classic_estimate(sk);
      if (const char* e = getenv("QEG_JOIN_EST_SCALE")) g *= atof(e);  // (tests: force a misestimate)
      est_distinct = std::max(g, 1.0);
      want_cap = std::max<uint64_t>(1024, next_pow2(static_cast<uint64_t>(std::ceil(kJoinSlotsPerEstimatedKey * est_distinct))));
    }
    P.ovf = dup.get<uint32_t>() + 1;
    build_hash(P, want_cap);
  }
  // The radix-partitioned join probes the same table (single key only).
  if (strategy == QEG_JOIN_HASH && nk == 1 && cfg.strategy == QEG_JOIN_PARTITIONED) {
    strategy = QEG_JOIN_PARTITIONED;
    part_bits = cfg.partition_bits > 0 ? std::min(cfg.partition_bits, 12) : 8;
  }
  uint64_t d[2] = {0, 0};
  QEG_CUDA(cudaMemcpyAsync(d, dup.get(), 16, cudaMemcpyDeviceToHost, ctx->stream));
  check_device_error(ctx);  // its synchronisation also lands d
  if (strategy != QEG_JOIN_DENSE && (d[0] >> 32) != 0) {
    // The estimate-sized table overflowed: build again at full size.
    ++rebuilds;
    est_distinct = 0;
    QEG_CUDA(cudaMemsetAsync(dup.get(), 0, 16, ctx->stream));
    P.ovf = nullptr;
    build_hash(P, 0);
    QEG_CUDA(cudaMemcpyAsync(d, dup.get(), 16, cudaMemcpyDeviceToHost, ctx->stream));
    check_device_error(ctx);
  }
  distinct = d[1];
  // Dense: the keys are unique when every non-NULL key set its own bit.
  unique = strategy == QEG_JOIN_DENSE ? (distinct == nonnull ? 1 : 0) : ((d[0] & 0xffffffffull) ? 0 : 1);
  csr_built = false;
  counts_ready = strategy != QEG_JOIN_DENSE && asof;  // (the as-of join reads no counts)
  // Repeated keys: the sinks read per-slot row counts.
  if (!unique && !asof) count_rows();
  acc.alloc(24, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(acc.get(), 0, 24, ctx->stream));
  if (asof) asof_build();
}

// As-of build: items per build row, a stable radix sort by (slot, timestamp),
// partition runs from the per-slot counts.
void JoinState::asof_build() {
  const int nk = static_cast<int>(bkeys.size());
  const uint64_t ns = nk == 0 ? 1 : slots();
  require(ns < 0xffffffffull, "as-of join: too many partitions");
  aslots = static_cast<uint32_t>(ns);
  tbits.alloc(((nbuild + 63) / 64 + 1) * 8, ctx->stream);
  if (nbuild) {
    bytes_to_bits_kernel<<<grid_for(ctx, (nbuild / 64 + 1) * 32, 256, 8), 256, 0, ctx->stream>>>(
        bvalid[btime].get<uint8_t>(), nbuild, tbits.get<uint64_t>());
    ctx->launches++;
  }
  DevCol ts{};
  ts.type = btypes[btime];
  ts.data = bvals[btime].get();
  ts.validity = tbits.get<uint64_t>();
  // Timestamp range of the build side (relative timestamps need its low end).
  DevBuf mm(24, ctx->stream);
  unsigned long long init[3] = {~0ull, 0ull, 0ull};
  QEG_CUDA(cudaMemcpyAsync(mm.get(), init, 24, cudaMemcpyHostToDevice, ctx->stream));
  if (nbuild) {
    minmax_kernel<<<grid_for(ctx, nbuild, 256, 8), 256, 0, ctx->stream>>>(ts, nbuild, mm.get<unsigned long long>());
    ctx->launches++;
  }
  unsigned long long r[3];
  QEG_CUDA(cudaMemcpyAsync(r, mm.get(), 24, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  tmin = r[2] ? dec_i64(r[0]) : 0;
  const uint64_t range = r[2] ? r[1] - r[0] : 0;
  int lo_bits = 0, hi_bits = 0;
  while (lo_bits < 64 && (range >> lo_bits) != 0) ++lo_bits;
  while (hi_bits < 32 && (static_cast<uint64_t>(aslots) >> hi_bits) != 0) ++hi_bits;

  const uint64_t n = nbuild;
  // A build side already in time order (no NULL times) only needs its stable
  // sort by slot: time order within every slot is kept.
  if (n > 1 && r[2] == n) {
    DevBuf flag(4, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(flag.get(), 0, 4, ctx->stream));
    time_order_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(ts, n, flag.get<unsigned int>());
    ctx->launches++;
    uint32_t unsorted = 1;
    QEG_CUDA(cudaMemcpyAsync(&unsorted, flag.get(), 4, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!unsorted) lo_bits = 0;
  }
  DevBuf a_lo(std::max<uint64_t>(n, 1) * 8, ctx->stream), b_lo(std::max<uint64_t>(n, 1) * 8, ctx->stream);
  DevBuf a_hi(std::max<uint64_t>(n, 1) * 4, ctx->stream), b_hi(std::max<uint64_t>(n, 1) * 4, ctx->stream);
  DevBuf a_val(std::max<uint64_t>(n, 1) * 4, ctx->stream), b_val(std::max<uint64_t>(n, 1) * 4, ctx->stream);
  if (n) {
    AsofItemsK P{};
    P.nkeys = nk;
    for (int j = 0; j < nk; ++j) P.key[j] = store_key(j);
    P.ts = ts;
    P.n = n;
    if (nk) P.T = table();
    P.nslots = aslots;
    P.tmin = tmin;
    P.lo = a_lo.get<uint64_t>();
    P.hi = a_hi.get<uint32_t>();
    P.val = a_val.get<uint32_t>();
    P.err = static_cast<uint32_t*>(ctx->dev_err.get());
    asof_items_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  SortItems A{a_lo.get<uint64_t>(), a_hi.get<uint32_t>(), a_val.get<uint32_t>()};
  SortItems B{b_lo.get<uint64_t>(), b_hi.get<uint32_t>(), b_val.get<uint32_t>()};
  const SortItems R = radix_sort_items(ctx, A, B, n, lo_bits, hi_bits);
  aruns.alloc(ns * 8, ctx->stream);
  asamp.alloc((n / kAsofSample + 1) * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(aruns.get(), 0, ns * 8, ctx->stream));
  if (n) {
    asof_runs_kernel<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(
        R.hi, R.lo, n, aslots, aruns.get<uint2>(), asamp.get<uint64_t>());
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  // Keep the sorted timestamps and rows; the slot words are no longer needed.
  const bool in_a = R.lo == A.lo;
  ats = in_a ? std::move(a_lo) : std::move(b_lo);
  arow = in_a ? std::move(a_val) : std::move(b_val);
  check_device_error(ctx);  // synchronises the stream
}

// One global hash table of the build keys (+ per-slot row counts).
void JoinState::build_hash(BuildK& P, uint64_t want_cap) {
  const int nk = static_cast<int>(bkeys.size());
  const uint64_t full = std::max<uint64_t>(1024, next_pow2(2 * std::max<uint64_t>(nbuild, 1)));
  cap = (want_cap > 0 && want_cap < full) ? want_cap : full;
  // An estimate-sized single-key table bounds its inserts' probes; a full-size
  // one (two slots per build row) cannot overflow.
  P.probe_limit = kEstimatedTableProbeLimit;
  if (cap == full || nk != 1) P.ovf = nullptr;
  const int kw = nk == 1 ? 1 : 1 + nk;
  const uint64_t krows = nk == 1 ? cap + 1 : cap;
  keys.alloc(krows * kw * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(keys.get(), 0, krows * kw * 8, ctx->stream));
  // Row counts are deferred (P.presence): only key word 0's side slot of a
  // single-key table is counted here.
  cnt.alloc(slots() * 4, ctx->stream);
  if (nk == 1) QEG_CUDA(cudaMemsetAsync(cnt.get<uint32_t>() + cap, 0, 4, ctx->stream));
  P.presence = asof ? 0 : 1;
  // A single-key table too large to stay in L2 gets a Bloom filter of
  // kBloomBitsPerKey bits per build row (an L2-resident word per probe row):
  // probe keys that miss it skip the table. QEG_JOIN_BLOOM=0 turns it off,
  // =1 gives every single-key table one (for tests and measurement).
  bloom.release();
  bloom_shift = 64;
  const char* bloom_env = getenv("QEG_JOIN_BLOOM");
  const int bloom_mode = bloom_env ? atoi(bloom_env) : -1;
  const bool want_bloom = bloom_mode == 1 || (bloom_mode != 0 && krows * 8 >= kBloomMinTableBytes);
  if (nk == 1 && !asof && want_bloom) {
    // Bits per distinct key: the estimate's (with a two-fold margin) when the
    // table was sized from it, else the build rows'.
    const uint64_t bkeys_n = (cap < full && est_distinct > 0)
                                 ? std::min<uint64_t>(nbuild, static_cast<uint64_t>(2.0 * est_distinct) + 1)
                                 : nbuild;
    const uint64_t words = next_pow2(std::max<uint64_t>(64, (bkeys_n * kBloomBitsPerKey + 63) / 64));
    int lg = 0;
    while ((1ull << lg) < words) ++lg;
    bloom.alloc(words * 8, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(bloom.get(), 0, words * 8, ctx->stream));
    bloom_shift = 64 - lg;
    P.bloom = bloom.get<unsigned long long>();
  }
  P.T = table();
  if (nbuild) {
    build_count_kernel<<<grid_for(ctx, nbuild, 256, 8), 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
}

// COUNT/SUM sink of a partitioned join: the probe side split by partition
// (histogram, scan, tile-sorted scatter), then the ordinary hashed sink over
// the partitioned rows in order.
template <typename KT, typename VT>
void partitioned_sink(JoinState& st, const DevCol& key, const DevCol& val, uint64_t n, SinkK S,
                      void (*sink)(SinkK)) {
  qeg_ctx* ctx = st.ctx;
  const uint32_t np = 1u << st.part_bits;
  PartK K{};
  K.key = key.data;
  K.kvalid = key.all_valid ? nullptr : key.validity;
  K.val = val.data;
  K.n = n;
  K.bits = st.part_bits;
  K.bloom = st.bloom.get<uint64_t>();
  K.bshift = st.bloom_shift;
  DevBuf hist(static_cast<size_t>(np) * 8, ctx->stream), cursor((static_cast<size_t>(np) + 1) * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(hist.get(), 0, hist.bytes(), ctx->stream));
  K.hist = hist.get<unsigned long long>();
  const size_t hb = static_cast<size_t>(np) * 4;
  ppart_hist_kernel<KT><<<grid_for(ctx, n, 512, 4), 512, hb, ctx->stream>>>(K);
  // Partition starts: an exclusive scan of the sizes (tiny, on the host).
  std::vector<unsigned long long> h(np), c(np + 1);
  QEG_CUDA(cudaMemcpyAsync(h.data(), hist.get(), np * 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  c[0] = 0;
  for (uint32_t i = 0; i < np; ++i) c[i + 1] = c[i] + h[i];
  const uint64_t total = c[np];
  QEG_CUDA(cudaMemcpyAsync(cursor.get(), c.data(), (np + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
  K.cursor = cursor.get<unsigned long long>();
  DevBuf okey(std::max<uint64_t>(total, 1) * 8, ctx->stream), oval(std::max<uint64_t>(total, 1) * 8, ctx->stream);
  K.okey = okey.get<uint64_t>();
  K.oval = oval.get<int64_t>();
  const size_t sb = static_cast<size_t>(kPartTile) * 18 + static_cast<size_t>(np) * 16 + 16;
  const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(ppart_scatter_kernel<KT, VT>), 512, sb);
  const uint64_t ntiles = (n + kPartTile - 1) / kPartTile;
  const unsigned g = static_cast<unsigned>(
      std::max<uint64_t>(1, std::min<uint64_t>(ntiles, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
  ppart_scatter_kernel<KT, VT><<<g, 512, sb, ctx->stream>>>(K);
  // The partitioned rows: 64-bit key words and payloads, no NULL keys.
  S.key = K.okey;
  S.kvalid = nullptr;
  S.val = K.oval;
  S.vvalid = nullptr;
  S.n = total;
  if (total) {
    int sink_per_sm = 0;
    QEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sink_per_sm, sink, 256, 0));
    const uint64_t want = (total / 8 + 255) / 256;
    const unsigned gs = static_cast<unsigned>(std::max<uint64_t>(
        1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(sink_per_sm, 1))));
    sink<<<gs, 256, 0, ctx->stream>>>(S);
  }
  ctx->launches += 3;
  QEG_CUDA(cudaGetLastError());
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));  // the partition buffers die with this scope
}

void probe_count_sum_partitioned(JoinState& st, const DevCol& key, const DevCol& val, uint64_t n, const SinkK& S) {
  const bool k8 = type_width(key.type) == 8, v8 = type_width(val.type) == 8;
  // The partitioned rows are 64-bit key words and payloads.
  void (*sink)(SinkK) = st.unique ? probe_sink_pipe_kernel<long long, long long, QEG_JOIN_HASH, true, 2>
                                  : probe_sink_pipe_kernel<long long, long long, QEG_JOIN_HASH, false, 2>;
  if (k8 && v8) partitioned_sink<long long, long long>(st, key, val, n, S, sink);
  else if (k8) partitioned_sink<long long, int>(st, key, val, n, S, sink);
  else if (v8) partitioned_sink<int, long long>(st, key, val, n, S, sink);
  else partitioned_sink<int, int>(st, key, val, n, S, sink);
}

BuildK JoinState::build_params(DevBuf& scratch) {
  BuildK P{};
  P.nkeys = static_cast<int>(bkeys.size());
  for (int j = 0; j < P.nkeys; ++j) P.key[j] = store_key(j);
  P.n = nbuild;
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());
  scratch.alloc(16, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(scratch.get(), 0, 16, ctx->stream));
  P.dup = scratch.get<uint32_t>();
  P.distinct = reinterpret_cast<unsigned long long*>(scratch.get<uint8_t>() + 8);
  P.T = table();
  return P;
}

// Per-slot build row counts (needed when keys repeat, and by the
// pair-materialising probe): a second pass over the build keys, which finds
// every key's slot (a hash table is complete) and counts its rows.
void JoinState::count_rows() {
  alloc_counts();
  counts_ready = true;
  DevBuf scratch;
  BuildK P = build_params(scratch);
  if (nbuild) {
    build_count_kernel<<<grid_for(ctx, nbuild, 256, 8), 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
}

// Builds the CSR row lists (off, rows) on the first probe that materialises
// pairs; the COUNT/SUM sink never needs them.
void JoinState::ensure_csr() {
  if (csr_built) return;
  if (!counts_ready) count_rows();
  const uint64_t n = slots();
  off.alloc((n + 1) * 8, ctx->stream);
  const uint64_t total = exclusive_scan(ctx, cnt.get<uint32_t>(), n, off.get<uint64_t>());
  rows.alloc(std::max<uint64_t>(total, 1) * 4, ctx->stream);
  DevBuf fill(n * 4, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(fill.get(), 0, n * 4, ctx->stream));
  DevBuf scratch;
  BuildK P = build_params(scratch);
  P.fill = fill.get<uint32_t>();
  P.rows_out = rows.get<uint32_t>();
  if (nbuild) {
    build_scatter_kernel<<<grid_for(ctx, nbuild, 256, 8), 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  check_device_error(ctx);  // synchronises the stream
  csr_built = true;
}

}  // namespace qeg

struct qeg_join {
  qeg::JoinState st;
};

using namespace qeg;

namespace {

void validate_probe(const JoinState& st, const qeg_column* cols, int ncols) {
  require(cols != nullptr, "cols is NULL");
  require(ncols == static_cast<int>(st.ptypes.size()), "probe batch column count does not match the schema");
  for (int c = 0; c < ncols; ++c) {
    require(cols[c].type == st.ptypes[c], "probe batch column type does not match the schema");
    require(cols[c].len == cols[0].len, "probe batch columns differ in length");
  }
}

}  // namespace

void JoinState::asof_probe(uint64_t n) {
  AsofProbeK P{};
  P.nkeys = static_cast<int>(pkeys.size());
  for (int j = 0; j < P.nkeys; ++j) P.key[j] = probe_staged[pkeys[j]].dev;
  P.ts = probe_staged[ptime].dev;
  P.n = n;
  if (P.nkeys) P.T = table();
  P.tmin = tmin;
  P.ats = ats.get<uint64_t>();
  P.arow = arow.get<uint32_t>();
  P.aruns = aruns.get<uint2>();
  P.asamp = asamp.get<uint64_t>();
  P.left = join_type == QEG_LEFT;
  P.tol_set = tol_set;
  P.tol = static_cast<uint64_t>(tol);
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());
  {
    const char* e = std::getenv("QEG_ASOF_HINT_BITS");
    P.hint_bits = e ? std::max(6, std::min(12, std::atoi(e))) : kAsofHintBits;
  }
  const size_t hsb = static_cast<size_t>(8) << P.hint_bits;  // slot + position per entry
  const unsigned g = grid_for(ctx, n, 256, 8);
  if (P.left) {
    out_probe.alloc(n * 4, ctx->stream);
    out_build.alloc(n * 4, ctx->stream);
    P.out_probe = out_probe.get<uint32_t>();
    P.out_build = out_build.get<uint32_t>();
    asof_probe_kernel<<<g, 256, hsb, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    check_device_error(ctx);
    nout = n;
    probe_identity = true;
    return;
  }
  amatch.alloc(n * 4, ctx->stream);
  counts.alloc(n * 4, ctx->stream);
  starts.alloc((n + 1) * 8, ctx->stream);
  P.match = amatch.get<uint32_t>();
  P.counts = counts.get<uint32_t>();
  asof_probe_kernel<<<g, 256, hsb, ctx->stream>>>(P);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  const uint64_t total = exclusive_scan(ctx, counts.get<uint32_t>(), n, starts.get<uint64_t>());
  out_probe.alloc(std::max<uint64_t>(total, 1) * 4, ctx->stream);
  out_build.alloc(std::max<uint64_t>(total, 1) * 4, ctx->stream);
  P.out_probe = out_probe.get<uint32_t>();
  P.out_build = out_build.get<uint32_t>();
  if (total) {
    asof_emit_kernel<<<g, 256, 0, ctx->stream>>>(P, starts.get<uint64_t>());
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  check_device_error(ctx);
  nout = total;
}

namespace {

ProbeK probe_params(JoinState& st, uint64_t n) {
  ProbeK P{};
  P.nkeys = static_cast<int>(st.pkeys.size());
  for (int j = 0; j < P.nkeys; ++j) P.key[j] = st.probe_staged[st.pkeys[j]].dev;
  P.n = n;
  P.T = st.table();
  P.left = st.join_type == QEG_LEFT;
  P.err = static_cast<uint32_t*>(st.ctx->dev_err.get());
  return P;
}

}  // namespace

extern "C" {

qeg_status qeg_join_create(qeg_ctx* ctx, const int32_t* probe_types, int nprobe, const int32_t* build_types,
                           int nbuild, const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
                           int32_t join_type, const qeg_join_config* cfg, qeg_join** out) {
  return guarded(ctx, [&] {
    require(ctx != nullptr && out != nullptr, "ctx/out is NULL");
    require(nkeys >= 1, "equi-join needs >=1 key");
    require(nkeys <= kMaxKeys, "GPU join supports at most 8 key columns");
    require(join_type == QEG_INNER || join_type == QEG_LEFT, "unknown join type");
    require(nprobe >= 1 && nbuild >= 1, "join sides need >=1 column");
    QEG_CUDA(cudaSetDevice(ctx->device));
    auto j = std::make_unique<qeg_join>();
    JoinState& st = j->st;
    st.ctx = ctx;
    st.ptypes.assign(probe_types, probe_types + nprobe);
    st.btypes.assign(build_types, build_types + nbuild);
    st.pkeys.assign(probe_keys, probe_keys + nkeys);
    st.bkeys.assign(build_keys, build_keys + nkeys);
    for (int k = 0; k < nkeys; ++k) {
      require(st.pkeys[k] < static_cast<uint32_t>(nprobe) && st.bkeys[k] < static_cast<uint32_t>(nbuild),
              "join key column index out of range");
      require(st.ptypes[st.pkeys[k]] == st.btypes[st.bkeys[k]],
              "HashJoin: join key column types must match positionally");
    }
    st.join_type = join_type;
    if (cfg) st.cfg = *cfg;
    st.bvals.resize(nbuild);
    st.bvalid.resize(nbuild);
    *out = j.release();
  });
}

qeg_status qeg_asof_create(qeg_ctx* ctx, const int32_t* probe_types, int nprobe, const int32_t* build_types,
                           int nbuild, const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
                           uint32_t probe_time, uint32_t build_time, int32_t asof_type, int32_t has_tolerance,
                           int64_t tolerance, qeg_join** out) {
  return guarded(ctx, [&] {
    require(ctx != nullptr && out != nullptr, "ctx/out is NULL");
    require(nkeys >= 0 && (nkeys == 0 || (probe_keys != nullptr && build_keys != nullptr)), "key lists are NULL");
    require(nkeys <= kMaxKeys, "GPU as-of join supports at most 8 key columns");
    require(asof_type == QEG_INNER || asof_type == QEG_LEFT, "unknown as-of join type");
    require(nprobe >= 1 && nbuild >= 1 && probe_types != nullptr && build_types != nullptr,
            "join sides need >=1 column");
    require(probe_time < static_cast<uint32_t>(nprobe) && build_time < static_cast<uint32_t>(nbuild),
            "as-of time column index out of range");
    auto ts_ok = [](int32_t t) { return t == QEG_I32 || t == QEG_I64 || t == QEG_TS; };
    require(ts_ok(probe_types[probe_time]) && ts_ok(build_types[build_time]),
            "AsofJoin: time columns must be I32/I64/TS");
    for (int k = 0; k < nkeys; ++k) {
      require(probe_keys[k] < static_cast<uint32_t>(nprobe) && build_keys[k] < static_cast<uint32_t>(nbuild),
              "as-of key column index out of range");
      require(probe_types[probe_keys[k]] == build_types[build_keys[k]],
              "AsofJoin: key column types must match positionally");
    }
    QEG_CUDA(cudaSetDevice(ctx->device));
    auto j = std::make_unique<qeg_join>();
    JoinState& st = j->st;
    st.ctx = ctx;
    st.ptypes.assign(probe_types, probe_types + nprobe);
    st.btypes.assign(build_types, build_types + nbuild);
    st.pkeys.assign(probe_keys, probe_keys + nkeys);
    st.bkeys.assign(build_keys, build_keys + nkeys);
    st.join_type = asof_type;
    st.asof = true;
    st.ptime = probe_time;
    st.btime = build_time;
    st.tol_set = has_tolerance ? 1 : 0;
    st.tol = tolerance;
    st.bvals.resize(nbuild);
    st.bvalid.resize(nbuild);
    *out = j.release();
  });
}

qeg_status qeg_join_build(qeg_join* j, const qeg_column* cols, int ncols) {
  qeg::NvtxRange nvtx_range("qeg_join_build");
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr && cols != nullptr, "join/cols is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    j->st.append(cols, ncols);
  });
}

qeg_status qeg_join_build_finish(qeg_join* j) {
  qeg::NvtxRange nvtx_range("qeg_join_build_finish");
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr, "join is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    j->st.finish_build();
  });
}

qeg_status qeg_join_probe(qeg_join* j, const qeg_column* cols, int ncols, uint64_t* out_rows) {
  qeg::NvtxRange nvtx_range("qeg_join_probe");
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr && out_rows != nullptr, "join/out_rows is NULL");
    JoinState& st = j->st;
    require(st.built, "probe() before build_finish()");
    validate_probe(st, cols, ncols);
    QEG_CUDA(cudaSetDevice(ctx->device));
    const uint64_t n = cols[0].len;
    require(n < 0xffffffffull, "a probe batch holds at most 2^32-2 rows");
    st.probe_staged.clear();
    st.probe_staged.resize(ncols);
    st.probe_identity = false;
    for (int c = 0; c < ncols; ++c) stage_column(ctx, cols[c], st.probe_staged[c]);
    st.nout = 0;
    if (n == 0) {
      *out_rows = 0;
      return;
    }
    if (st.asof) {
      st.asof_probe(n);
      *out_rows = st.nout;
      return;
    }
    st.ensure_csr();
    st.counts.alloc(n * 4, ctx->stream);
    st.starts.alloc((n + 1) * 8, ctx->stream);
    ProbeK P = probe_params(st, n);
    P.counts = st.counts.get<uint32_t>();
    const unsigned g = grid_for(ctx, n, 256, 8);
    probe_count_kernel<<<g, 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    const uint64_t total = exclusive_scan(ctx, st.counts.get<uint32_t>(), n, st.starts.get<uint64_t>());
    st.out_probe.alloc(std::max<uint64_t>(total, 1) * 4, ctx->stream);
    st.out_build.alloc(std::max<uint64_t>(total, 1) * 4, ctx->stream);
    P.starts = st.starts.get<uint64_t>();
    P.out_probe = st.out_probe.get<uint32_t>();
    P.out_build = st.out_build.get<uint32_t>();
    probe_emit_kernel<<<g, 256, 0, ctx->stream>>>(P);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    check_device_error(ctx);
    st.nout = total;
    *out_rows = total;
  });
}

qeg_status qeg_join_fetch(qeg_join* j, uint64_t first, uint64_t count, const qeg_out_column* outs) {
  qeg::NvtxRange nvtx_range("qeg_join_fetch");
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr && outs != nullptr, "join/outs is NULL");
    JoinState& st = j->st;
    require(first <= st.nout && count <= st.nout - first, "fetch range outside the probed batch's output");
    QEG_CUDA(cudaSetDevice(ctx->device));
    if (count == 0) {
      for (size_t c = 0; c < st.ptypes.size() + st.btypes.size(); ++c)
        if (outs[c].all_valid) *outs[c].all_valid = 1;
      return;
    }
    const size_t ncol = st.ptypes.size() + st.btypes.size();
    bool dev_out = true;
    for (size_t c = 0; c < ncol; ++c)
      dev_out = dev_out && outs[c].data && is_device_ptr(outs[c].data) &&
                (!outs[c].validity || is_device_ptr(outs[c].validity));
    // Column c of the output as a gather-kernel column writing into out/words.
    auto gather_col = [&](GatherCol& g, size_t c, void* out, uint64_t* words) {
      const bool pc = c < st.ptypes.size();
      const size_t bc = pc ? 0 : c - st.ptypes.size();
      g.flag = static_cast<int>(c);
      g.width = static_cast<int>(type_width(pc ? st.ptypes[c] : st.btypes[bc]));
      g.side = pc ? 0 : 1;
      g.out = out;
      g.words = words;
      if (pc) {
        const StagedCol& sc = st.probe_staged[c];
        g.src = sc.dev.data;
        g.bits = sc.dev.all_valid ? nullptr : sc.dev.validity;
        g.code_map = st.ptypes[c] == QEG_STR ? sc.dev.code_map : nullptr;
      } else {
        g.src = st.bvals[bc].get();
        g.bytes = st.bvalid[bc].get<uint8_t>();
      }
    };
    if (dev_out) {
      // One pass per column into the caller's device buffers, one sync.
      DevBuf flags(ncol * 4, ctx->stream);
      QEG_CUDA(cudaMemsetAsync(flags.get(), 0, ncol * 4, ctx->stream));
      const unsigned gw = grid_for(ctx, (count + 63) / 64 * 32, 256, 8);
      // Output row k = probe row first + k (LEFT as-of) with a word-aligned
      // start: probe columns are plain copies, made by the copy engines on a
      // side stream while the gather kernel fills the build columns.
      std::vector<char> copied(ncol, 0);
      bool forked = false;
      DevBuf tmp_words;
      if (st.probe_identity && first % 64 == 0) {
        const uint64_t nw = (count + 63) / 64;
        auto copyable = [&](size_t c) { return !(st.ptypes[c] == QEG_STR && st.probe_staged[c].dev.code_map); };
        size_t ntmp = 0;  // copied columns with NULLs but no validity output: words still needed for the flag
        for (size_t c = 0; c < st.ptypes.size(); ++c)
          ntmp += copyable(c) && !st.probe_staged[c].dev.all_valid && !outs[c].validity;
        if (ntmp) tmp_words.alloc(ntmp * nw * 8, ctx->stream);  // before ev_in: ordered ahead of the side stream
        if (!ctx->side) {
          QEG_CUDA(cudaEventCreateWithFlags(&ctx->side_in, cudaEventDisableTiming));
          QEG_CUDA(cudaEventCreateWithFlags(&ctx->side_out, cudaEventDisableTiming));
          QEG_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        }
        QEG_CUDA(cudaEventRecord(ctx->side_in, ctx->stream));
        QEG_CUDA(cudaStreamWaitEvent(ctx->side, ctx->side_in, 0));
        forked = true;
        size_t itmp = 0;
        for (size_t c = 0; c < st.ptypes.size(); ++c) {
          if (!copyable(c)) continue;  // dictionary codes need translating: gathered below
          const StagedCol& sc = st.probe_staged[c];
          const size_t w = type_width(st.ptypes[c]);
          QEG_CUDA(cudaMemcpyAsync(outs[c].data, static_cast<const uint8_t*>(sc.dev.data) + first * w, count * w,
                                   cudaMemcpyDeviceToDevice, ctx->side));
          if (sc.dev.all_valid) {
            if (outs[c].validity) QEG_CUDA(cudaMemsetAsync(outs[c].validity, 0xff, nw * 8, ctx->side));
          } else {
            uint64_t* words = outs[c].validity ? outs[c].validity : tmp_words.get<uint64_t>() + nw * itmp++;
            QEG_CUDA(cudaMemcpyAsync(words, sc.dev.validity + first / 64, nw * 8, cudaMemcpyDeviceToDevice,
                                     ctx->side));
            words_finish_kernel<<<grid_for(ctx, nw, 256, 4), 256, 0, ctx->side>>>(words, nw, count,
                                                                                 flags.get<unsigned int>() + c);
            ctx->launches++;
            QEG_CUDA(cudaGetLastError());
          }
          copied[c] = 1;
        }
        QEG_CUDA(cudaEventRecord(ctx->side_out, ctx->side));
      }
      if (ncol <= static_cast<size_t>(kMaxGatherCols)) {
        GatherK G{};
        G.idx[0] = st.out_probe.get<uint32_t>() + first;
        G.idx[1] = st.out_build.get<uint32_t>() + first;
        G.n = count;
        G.flags = flags.get<unsigned int>();
        for (size_t c = 0; c < ncol; ++c)
          if (!copied[c]) gather_col(G.c[G.ncols++], c, outs[c].data, outs[c].validity);
        if (G.ncols > 0) {
          gather_cols_kernel<<<gw, 256, 0, ctx->stream>>>(G);
          ctx->launches++;
          QEG_CUDA(cudaGetLastError());
        }
      }
      if (forked) QEG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->side_out, 0));
      for (size_t c = 0; c < ncol && ncol > static_cast<size_t>(kMaxGatherCols); ++c) {
        const bool pc = c < st.ptypes.size();
        const size_t bc = pc ? 0 : c - st.ptypes.size();
        const int w = static_cast<int>(type_width(pc ? st.ptypes[c] : st.btypes[bc]));
        const void* src = pc ? st.probe_staged[c].dev.data : st.bvals[bc].get();
        const uint64_t* bits = nullptr;
        const uint8_t* bytes = nullptr;
        const int32_t* cm = nullptr;
        const uint32_t* idx = (pc ? st.out_probe.get<uint32_t>() : st.out_build.get<uint32_t>()) + first;
        if (pc) {
          const StagedCol& sc = st.probe_staged[c];
          bits = sc.dev.all_valid ? nullptr : sc.dev.validity;
          cm = st.ptypes[c] == QEG_STR ? sc.dev.code_map : nullptr;
        } else {
          bytes = st.bvalid[bc].get<uint8_t>();
        }
        gather_out_kernel<<<gw, 256, 0, ctx->stream>>>(src, bits, bytes, cm, w, idx, count, outs[c].data,
                                                      outs[c].validity, flags.get<unsigned int>() + c);
        ctx->launches++;
        QEG_CUDA(cudaGetLastError());
      }
      std::vector<uint32_t> f(ncol);
      QEG_CUDA(cudaMemcpyAsync(f.data(), flags.get(), ncol * 4, cudaMemcpyDeviceToHost, ctx->stream));
      QEG_CUDA(cudaStreamSynchronize(ctx->stream));
      for (size_t c = 0; c < ncol; ++c)
        if (outs[c].all_valid) *outs[c].all_valid = f[c] ? 0 : 1;
      return;
    }
    if (ncol <= static_cast<size_t>(kMaxGatherCols)) {
      // Host (or mixed) outputs: chunks of rows gathered in one pass into
      // device staging buffers, each column then copied out; one sync.
      const uint64_t chunk = std::min<uint64_t>((count + 63) / 64 * 64, uint64_t{1} << 24);
      const uint64_t cw = chunk / 64;
      size_t row_bytes = 0;
      std::vector<size_t> vofs(ncol);
      for (size_t c = 0; c < ncol; ++c) {
        vofs[c] = row_bytes * chunk;
        row_bytes += type_width(c < st.ptypes.size() ? st.ptypes[c] : st.btypes[c - st.ptypes.size()]);
      }
      DevBuf vals(row_bytes * chunk, ctx->stream), words(ncol * cw * 8, ctx->stream), flags(ncol * 4, ctx->stream);
      QEG_CUDA(cudaMemsetAsync(flags.get(), 0, ncol * 4, ctx->stream));
      for (uint64_t off = 0; off < count; off += chunk) {
        const uint64_t n = std::min(chunk, count - off);
        GatherK G{};
        G.ncols = static_cast<int>(ncol);
        G.idx[0] = st.out_probe.get<uint32_t>() + first + off;
        G.idx[1] = st.out_build.get<uint32_t>() + first + off;
        G.n = n;
        G.flags = flags.get<unsigned int>();
        for (size_t c = 0; c < ncol; ++c)
          gather_col(G.c[c], c, vals.get<uint8_t>() + vofs[c], words.get<uint64_t>() + c * cw);
        gather_cols_kernel<<<grid_for(ctx, (n + 63) / 64 * 32, 256, 8), 256, 0, ctx->stream>>>(G);
        ctx->launches++;
        QEG_CUDA(cudaGetLastError());
        for (size_t c = 0; c < ncol; ++c) {
          const size_t w = static_cast<size_t>(G.c[c].width);
          if (outs[c].data)
            QEG_CUDA(cudaMemcpyAsync(static_cast<uint8_t*>(outs[c].data) + off * w, vals.get<uint8_t>() + vofs[c],
                                     n * w, cudaMemcpyDefault, ctx->stream));
          if (outs[c].validity)  // off is a multiple of 64: whole words
            QEG_CUDA(cudaMemcpyAsync(outs[c].validity + off / 64, words.get<uint64_t>() + c * cw, (n + 63) / 64 * 8,
                                     cudaMemcpyDefault, ctx->stream));
        }
      }
      std::vector<uint32_t> f(ncol);
      QEG_CUDA(cudaMemcpyAsync(f.data(), flags.get(), ncol * 4, cudaMemcpyDeviceToHost, ctx->stream));
      QEG_CUDA(cudaStreamSynchronize(ctx->stream));
      for (size_t c = 0; c < ncol; ++c)
        if (outs[c].all_valid) *outs[c].all_valid = f[c] ? 0 : 1;
      return;
    }
    DevBuf vals(count * 8, ctx->stream), valid(count, ctx->stream);
    const unsigned g = grid_for(ctx, count, 256, 8);
    for (size_t c = 0; c < st.ptypes.size(); ++c) {
      const StagedCol& s = st.probe_staged[c];
      const int w = static_cast<int>(type_width(st.ptypes[c]));
      gather_kernel<<<g, 256, 0, ctx->stream>>>(s.dev.data, s.dev.all_valid ? nullptr : s.dev.validity, nullptr,
                                               st.ptypes[c] == QEG_STR ? s.dev.code_map : nullptr, w,
                                               st.out_probe.get<uint32_t>() + first, count, vals.get(),
                                               valid.get<uint8_t>());
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
      fetch_column(ctx, vals.get(), valid.get<uint8_t>(), w, 0, count, outs[c]);
    }
    for (size_t c = 0; c < st.btypes.size(); ++c) {
      const int w = static_cast<int>(type_width(st.btypes[c]));
      gather_kernel<<<g, 256, 0, ctx->stream>>>(st.bvals[c].get(), nullptr, st.bvalid[c].get<uint8_t>(), nullptr, w,
                                               st.out_build.get<uint32_t>() + first, count, vals.get(),
                                               valid.get<uint8_t>());
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
      fetch_column(ctx, vals.get(), valid.get<uint8_t>(), w, 0, count, outs[st.ptypes.size() + c]);
    }
  });
}

qeg_status qeg_join_probe_count_sum(qeg_join* j, const qeg_column* probe_key, const qeg_column* probe_val) {
  qeg::NvtxRange nvtx_range("qeg_join_probe_count_sum");
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr && probe_key != nullptr && probe_val != nullptr, "join/columns are NULL");
    JoinState& st = j->st;
    require(st.built, "probe before build_finish()");
    require(!st.asof, "the count/sum sink is not an as-of join");
    require(st.bkeys.size() == 1, "the count/sum sink takes a single key column");
    require(st.join_type == QEG_INNER, "the count/sum sink is an inner join");
    require(probe_key->type == st.btypes[st.bkeys[0]], "probe key type does not match the build key type");
    require(probe_val->type != QEG_F64 && probe_val->type != QEG_STR, "the count/sum sink sums an integer column");
    require(probe_key->len == probe_val->len, "probe columns differ in length");
    QEG_CUDA(cudaSetDevice(ctx->device));
    const uint64_t n = probe_key->len;
    if (n == 0 || st.distinct == 0) return;
    StagedCol k, v;
    stage_column(ctx, *probe_key, k);
    stage_column(ctx, *probe_val, v);
    ProbeK P{};
    P.nkeys = 1;
    P.key[0] = k.dev;
    P.val = v.dev;
    P.n = n;
    P.T = st.table();
    P.acc = st.acc.get<unsigned long long>();
    P.err = static_cast<uint32_t*>(ctx->dev_err.get());
    const int kt = probe_key->type, vt = probe_val->type;
    const bool kfast = kt == QEG_I32 || kt == QEG_I64 || kt == QEG_TS;
    const bool vfast = vt == QEG_I32 || vt == QEG_I64 || vt == QEG_TS;
    const bool aligned = (reinterpret_cast<uintptr_t>(k.dev.data) % 16 == 0) &&
                         (reinterpret_cast<uintptr_t>(v.dev.data) % 16 == 0);
    if (kfast && vfast && aligned) {
      SinkK S{};
      S.key = k.dev.data;
      S.kvalid = k.dev.all_valid ? nullptr : k.dev.validity;
      S.val = v.dev.data;
      S.vvalid = v.dev.all_valid ? nullptr : v.dev.validity;
      S.n = n;
      S.T = st.table();
      S.acc = st.acc.get<unsigned long long>();
      if (const char* e = getenv("QEG_JOIN_TABLE_KEEP_L2")) S.keep_table = atoi(e) != 0;
      if (st.strategy == QEG_JOIN_PARTITIONED && v.dev.all_valid) {
        // (Payload NULLs would need a partitioned validity column: the direct
        // hashed sink below handles them.)
        probe_count_sum_partitioned(st, k.dev, v.dev, n, S);
        return;
      }
      const bool k8 = type_width(kt) == 8, v8 = type_width(vt) == 8, dense = st.strategy == QEG_JOIN_DENSE;
      // Hashed tables: QEG_JOIN_SWEEPS=n > 1 probes in n sweeps over windows of
      // the table (opt-in: on GB300 the 16M-key table's 64 MB windows reach a
      // 73% L2 hit rate and each sweep re-reads the 2 GB key column, so 256M
      // probes take 5.8 ms in 2 sweeps and 6.8 ms in 4, against 3.8 ms for
      // the direct probe below).
      if (st.strategy == QEG_JOIN_HASH && lean_sizes_ok(n)) {
        uint64_t sweeps = 1;
        if (const char* e = getenv("QEG_JOIN_SWEEPS")) sweeps = std::max(1, atoi(e));
        if (sweeps > 1) {
          auto sweep_all = [&](void (*kern)(SinkK, uint32_t, uint32_t)) {
            int per_sm = 0;
            QEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSweepThreads, 0));
            const uint64_t want = (n / 128 + 7) / 8;
            const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(
                1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
            for (uint32_t w = 0; w < sweeps; ++w) {
              kern<<<grid, kSweepThreads, 0, ctx->stream>>>(S, w, static_cast<uint32_t>(sweeps));
              ctx->launches++;
            }
          };
          if (k8 && v8) sweep_all(st.unique ? probe_sink_sweep_kernel<long long, long long, true>
                                            : probe_sink_sweep_kernel<long long, long long, false>);
          else if (k8) sweep_all(st.unique ? probe_sink_sweep_kernel<long long, int, true>
                                           : probe_sink_sweep_kernel<long long, int, false>);
          else if (v8) sweep_all(st.unique ? probe_sink_sweep_kernel<int, long long, true>
                                           : probe_sink_sweep_kernel<int, long long, false>);
          else sweep_all(st.unique ? probe_sink_sweep_kernel<int, int, true> : probe_sink_sweep_kernel<int, int, false>);
          QEG_CUDA(cudaGetLastError());
          if (k.data.get() || v.data.get() || k.validity.get() || v.validity.get())
            QEG_CUDA(cudaStreamSynchronize(ctx->stream));  // staged inputs die with this scope
          return;
        }
      }
      // One wave of resident blocks; each thread strides over the probe side.
      auto launch = [&](void (*kern)(SinkK)) {
        const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), 256, 0);
        const uint64_t want = (n / 8 + 255) / 256;
        const unsigned grid = static_cast<unsigned>(
            std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
        kern<<<grid, 256, 0, ctx->stream>>>(S);
      };
      // The TMA-staged kernel (one block of kTmaThreads per SM, a kStages ring
      // of shared-memory tiles) is opt-in (QEG_SINK_TMA=1): on GB300 the
      // register-pipelined kernel reads the probe side faster (1.05 ms against
      // 1.38 ms for 256M dense-table probes; 5.9 against 10.4 ms hashed).
      auto al16 = [](const void* p) { return p == nullptr || reinterpret_cast<uintptr_t>(p) % 16 == 0; };
      const char* tma_env = getenv("QEG_SINK_TMA");
      // The lean kernel is the default. Dense table with unique build keys: 32
      // registers at 8 CTAs of 256 per SM (full occupancy) stream the 256M-row
      // probe side at 96% of the measured HBM copy bandwidth on GB300. The
      // same kernel with the next tile's loads issued early, or at 6 CTAs per
      // SM, measured 88-96%; the 64-register pipelined kernel with 128-row
      // warp tiles (4 CTAs per SM) 73%, and 81% at 6 CTAs per SM (40
      // registers, spilling). Hashed tables: 40 registers at 6 CTAs per SM
      // (the probe loop spills 76 B at 32 registers) probe 256M rows against
      // 16M unique keys in 4.4 ms, against 5.5 ms at 8 CTAs and 5.6 ms for the
      // pipelined kernel. QEG_SINK_PIPE=0|1|2|4|8 picks one for measurement.
      const bool lean_ok = n / 64 < (uint64_t{1} << 31);
      const bool bloomed = st.bloom.get() != nullptr;
      // CTAs per SM of the hashed sink (QEG_SINK_HASH_MINB=4|6|8, for measurement).
      const char* minb_env = getenv("QEG_SINK_HASH_MINB");
      const int hash_minb = minb_env ? atoi(minb_env) : 6;
      const char* pipe_env = getenv("QEG_SINK_PIPE");
      const int pipe = pipe_env ? atoi(pipe_env) : (lean_ok ? 1 : 2);
      const bool use_tma = n >= static_cast<uint64_t>(kTileRows) * ctx->sms * 2 && al16(S.kvalid) && al16(S.vvalid) &&
                           tma_env != nullptr && tma_env[0] == '1';
      auto launch_async = [&](void (*kern)(SinkK), size_t sb) {
        const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), 256, sb);
        const uint64_t want = (n / kAsyncTile + 7) / 8;
        const unsigned grid = static_cast<unsigned>(
            std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
        kern<<<grid, 256, sb, ctx->stream>>>(S);
      };
      auto launch_tma = [&](void (*kern)(SinkK, uint32_t*), size_t tile_bytes) {
        const size_t sb = tile_bytes * kStages;
        raise_dynamic_smem(reinterpret_cast<const void*>(kern), sb);
        kern<<<ctx->sms, kTmaThreads, sb, ctx->stream>>>(S, static_cast<uint32_t*>(ctx->dev_err.get()));
      };
#define QEG_SINK(KT, VT)                                                                                           \
  do {                                                                                                             \
    const size_t tb = sizeof(TmaTile<KT, VT>);                                                                     \
    if (use_tma) {                                                                                                 \
      if (dense && st.unique) launch_tma(probe_sink_tma_kernel<KT, VT, QEG_JOIN_DENSE, true>, tb);                \
      else if (dense) launch_tma(probe_sink_tma_kernel<KT, VT, QEG_JOIN_DENSE, false>, tb);                       \
      else if (st.unique) launch_tma(probe_sink_tma_kernel<KT, VT, QEG_JOIN_HASH, true>, tb);                     \
      else launch_tma(probe_sink_tma_kernel<KT, VT, QEG_JOIN_HASH, false>, tb);                                   \
    } else if (pipe == 8) {                                                                                        \
      const size_t sb = async_stage_bytes<KT, VT>() * kAsyncStages * 8;                                            \
      if (dense && st.unique) launch_async(probe_sink_async_kernel<KT, VT, QEG_JOIN_DENSE, true>, sb);            \
      else if (dense) launch_async(probe_sink_async_kernel<KT, VT, QEG_JOIN_DENSE, false>, sb);                   \
      else if (st.unique) launch_async(probe_sink_async_kernel<KT, VT, QEG_JOIN_HASH, true>, sb);                 \
      else launch_async(probe_sink_async_kernel<KT, VT, QEG_JOIN_HASH, false>, sb);                               \
    } else if (pipe == 2) {                                                                                        \
      if (dense && st.unique) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_DENSE, true, 2>);                    \
      else if (dense) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_DENSE, false, 2>);                           \
      else if (st.unique) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_HASH, true, 2>);                         \
      else launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_HASH, false, 2>);                                       \
    } else if (pipe == 1 && lean_ok) {                                                                             \
      if (dense && st.unique) launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_DENSE, true, 1, false, 8>);          \
      else if (dense) launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_DENSE, false, 1, false, 8>);                 \
      else if (bloomed && st.unique && hash_minb == 4)                                                            \
        launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, true, 1, false, 4, true>);                            \
      else if (bloomed && st.unique && hash_minb == 8)                                                            \
        launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, true, 1, false, 8, true>);                            \
      else if (bloomed && st.unique) launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, true, 1, false, 6, true>); \
      else if (bloomed) launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, false, 1, false, 6, true>);          \
      else if (st.unique) launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, true, 1, false, 6>);               \
      else launch(probe_sink_lean_kernel<KT, VT, QEG_JOIN_HASH, false, 1, false, 6>);                             \
    } else if (pipe == 4) {                                                                                        \
      if (dense && st.unique) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_DENSE, true, 4>);                    \
      else if (dense) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_DENSE, false, 4>);                           \
      else if (st.unique) launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_HASH, true, 4>);                         \
      else launch(probe_sink_pipe_kernel<KT, VT, QEG_JOIN_HASH, false, 4>);                                       \
    } else if (dense && st.unique) launch(probe_sink_kernel<KT, VT, QEG_JOIN_DENSE, true>);                       \
    else if (dense) launch(probe_sink_kernel<KT, VT, QEG_JOIN_DENSE, false>);                                    \
    else if (st.unique) launch(probe_sink_kernel<KT, VT, QEG_JOIN_HASH, true>);                                  \
    else launch(probe_sink_kernel<KT, VT, QEG_JOIN_HASH, false>);                                                \
  } while (0)
      if (k8 && v8) QEG_SINK(long long, long long);
      else if (k8) QEG_SINK(long long, int);
      else if (v8) QEG_SINK(int, long long);
      else QEG_SINK(int, int);
#undef QEG_SINK
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
      if (k.data.get() || v.data.get() || k.validity.get() || v.validity.get())
        QEG_CUDA(cudaStreamSynchronize(ctx->stream));  // staged inputs die with this scope
      return;
    }
    int per_sm = 0;
    const int block = 512;
    const unsigned g0 = static_cast<unsigned>(std::min<uint64_t>((n + block - 1) / block, ctx->sms * 4ull));
    if (st.strategy == QEG_JOIN_DENSE) {
      if (st.unique) probe_count_sum_kernel<QEG_JOIN_DENSE, true><<<g0, block, 0, ctx->stream>>>(P);
      else probe_count_sum_kernel<QEG_JOIN_DENSE, false><<<g0, block, 0, ctx->stream>>>(P);
    } else {
      if (st.unique) probe_count_sum_kernel<QEG_JOIN_HASH, true><<<g0, block, 0, ctx->stream>>>(P);
      else probe_count_sum_kernel<QEG_JOIN_HASH, false><<<g0, block, 0, ctx->stream>>>(P);
    }
    (void)per_sm;
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));  // staged inputs die with this scope
  });
}

qeg_status qeg_join_count_sum_result(qeg_join* j, int64_t* count, int64_t* sum, int32_t* sum_valid) {
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr && count && sum && sum_valid, "NULL argument");
    QEG_CUDA(cudaSetDevice(ctx->device));
    unsigned long long a[3] = {0, 0, 0};
    if (j->st.acc.get()) {
      QEG_CUDA(cudaMemcpyAsync(a, j->st.acc.get(), 24, cudaMemcpyDeviceToHost, ctx->stream));
    }
    check_device_error(ctx);
    *count = static_cast<int64_t>(a[0]);
    *sum = static_cast<int64_t>(a[1]);
    *sum_valid = a[2] ? 1 : 0;
  });
}

qeg_status qeg_join_stats(const qeg_join* j, int32_t* strategy, int32_t* partition_bits, uint64_t* distinct_keys) {
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr, "join is NULL");
    if (strategy) *strategy = j->st.strategy;
    if (partition_bits) *partition_bits = j->st.strategy == QEG_JOIN_PARTITIONED ? j->st.part_bits : 0;
    if (distinct_keys) *distinct_keys = j->st.distinct;
  });
}

qeg_status qeg_join_sizing_stats(const qeg_join* j, uint64_t* slots, double* est_distinct, int32_t* rebuilds) {
  qeg_ctx* ctx = j ? j->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(j != nullptr, "join is NULL");
    if (slots) *slots = j->st.cap;
    if (est_distinct) *est_distinct = j->st.est_distinct;
    if (rebuilds) *rebuilds = j->st.rebuilds;
  });
}

void qeg_join_destroy(qeg_join* j) {
  if (!j) return;
  cudaSetDevice(j->st.ctx->device);
  delete j;
}

}  // extern "C"
