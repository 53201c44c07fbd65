// qeg_agg.cu -- hash GROUP BY on sm_103a: replaces qe::Aggregate
// (ops/aggregate.h:102-144, ops/aggregate.cpp).
//
// Table layout (HBM). One row of 64-bit words per group:
//   single key : [key word][fields...]            + 2 side rows at index cap
//                (key word 0, which doubles as the empty marker) and cap+1
//                (the NULL key group)
//   multi key  : [state][null mask][key words...][fields...]; state 0 = empty,
//                1 = being published, >= 2 = the row's hash tag
//   global     : one row [unused][fields...]
// Fields hold the reference's AggCell state (ops/agg_internal.h:47-51) in a
// form where all-zero bits are the identity of every aggregate, so tables are
// initialised by memset: row count, per-column NULL count (non-null count =
// rows - nulls), integer / F64 sums, and MIN/MAX as order-preserving unsigned
// encodings updated with atomicMax (qeg_device.cuh).
//
// Kernel: each CTA keeps a private shared-memory table (first-come insertion,
// or preloaded with heavy hitters) and falls back to the global table, whose
// key words are claimed with one CAS. Rows whose key cannot be placed within
// the probe limit are spilled (row index) and re-run after the host grows the
// table (rehash) -- the GPU form of HashTable::grow (ops/hashtable.cpp:75-91).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "qeg_agg.h"
#include "qeg_warpagg.cuh"

namespace qeg {

namespace {

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Acquire load: a state word published after the key words (a fence, then
// the atomic exchange of the tag) makes those key words visible to the loads
// that follow it.
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Probe length for new keys once the global table is nearly full.
constexpr int kFullProbe = 16;
// The partitioned strategy is chosen (QEG_AGG_AUTO) for inputs of at least
// kPartMinRows rows whose estimated global table would take kPartMinTableBytes
// or more (half of L2: its random rows would mostly come from DRAM).
constexpr uint64_t kPartMinRows = 1ull << 22;
constexpr uint64_t kPartMinTableBytes = 64ull << 20;
// At most 2^kPartMaxBits partitions (the sizing pass keeps a 32-bit counter
// per partition in shared memory), and QEG_AGG_AUTO partitions only while the
// estimate averages at most kPartMaxFill of a second-pass table per partition.
constexpr int kPartMaxBits = 15;
constexpr double kPartMaxFill = 0.6;
// ... and only while the sketch's heavy hitters cover less than this share of
// the rows (a heavy head is better served by the CTA-private tables).
constexpr double kPartMaxHotShare = 0.3;

__device__ __forceinline__ uint64_t ld_volatile_shared(const uint64_t* p) {
  return *reinterpret_cast<const volatile uint64_t*>(p);
}

// Loads the values of one row for every referenced value column.
template <int NV>
__device__ __forceinline__ void load_values(const AggK& P, uint64_t p, bool (&vv)[kMaxVals],
                                            uint64_t (&vb)[kMaxVals]) {
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    vv[c] = false;
    vb[c] = 0;
    if (c < P.nvals) {
      const DevCol& col = P.val[c];
      vv[c] = col_valid(col, p);
      if (vv[c]) {
        if (col.type == kF64)
          vb[c] = static_cast<uint64_t>(__ldg(static_cast<const long long*>(col.data) + p));
        else
          vb[c] = static_cast<uint64_t>(int_value(col, p));
      }
    }
  }
}

__device__ __forceinline__ uint64_t key_hash1(uint64_t k) { return hash_fold(kHashSeed, k); }

// Single-key global lookup/insert. Returns the row, or nullptr when the key
// could not be placed within the probe limit.
__device__ __forceinline__ uint64_t* global_row1(const AggK& P, bool kv, uint64_t k, uint64_t h,
                                                 unsigned long long& inserted, int limit) {
  const int W = P.row_words;
  if (!kv) return P.table + (P.cap + 1) * W;
  if (k == 0) return P.table + P.cap * W;
  // Linear probing. The home slot alone first (one sector, and the answer for
  // most keys at the target load), then four slots per step: their key words
  // are loaded together (independent loads) and examined in slot order, so a
  // long probe costs a quarter of the dependent memory round trips. A key
  // word never changes once set, so a stale non-empty value stays correct.
  uint64_t s = __umul64hi(h, P.cap);
  {
    uint64_t* r = P.table + s * W;
    const uint64_t cur = ld_relaxed(r);
    if (cur == k) return r;
    if (cur == 0) {
      const unsigned long long old =
          atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, static_cast<unsigned long long>(k));
      if (old == 0) {
        ++inserted;
        return r;
      }
      if (old == k) return r;
    }
    if (++s == P.cap) s = 0;
  }
  for (int t = 1; t < limit; t += 4) {
    uint64_t idx[4], cur[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint64_t x = s + j;
      if (x >= P.cap) x -= P.cap;
      idx[j] = x;
      cur[j] = ld_relaxed(P.table + x * W);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint64_t* r = P.table + idx[j] * W;
      if (cur[j] == k) return r;
      if (cur[j] == 0) {
        const unsigned long long old =
            atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, static_cast<unsigned long long>(k));
        if (old == 0) {
          ++inserted;
          return r;
        }
        if (old == k) return r;
      }
    }
    s += 4;
    if (s >= P.cap) s -= P.cap;
  }
  return nullptr;
}

// Multi-key global lookup/insert with a publish protocol: claim (0 -> 1), write
// null mask and key words, fence, publish the tag. Readers wait (bounded) on a
// row being published.
__device__ __forceinline__ uint64_t* global_rowN(const AggK& P, const uint64_t* words, uint64_t nullmask,
                                                 uint64_t h, unsigned long long& inserted) {
  const int W = P.row_words;
  const uint64_t tag = (h >> 32) | 2ull;
  uint64_t s = __umul64hi(h, P.cap);
  for (int t = 0; t < P.probe_limit; ++t) {
    uint64_t* r = P.table + s * W;
    uint64_t st = ld_acquire(r);
    if (st == 0) {
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, 1ull);
      if (old == 0) {
        r[1] = nullmask;
        for (int j = 0; j < P.nkeys; ++j) r[2 + j] = words[j];
        __threadfence();
        atomicExch(reinterpret_cast<unsigned long long*>(r), static_cast<unsigned long long>(tag));
        ++inserted;
        return r;
      }
      st = old;
    }
    st = wait_published(r, st, kSpinLimit, P.err);
    if (st == kRowClaimed) return nullptr;
    if (st == tag) {
      bool eq = ld_relaxed(r + 1) == nullmask;
      for (int j = 0; eq && j < P.nkeys; ++j) eq = ld_relaxed(r + 2 + j) == words[j];
      if (eq) return r;
    }
    s = (s + 1 == P.cap) ? 0 : s + 1;
  }
  return nullptr;
}

__device__ __forceinline__ void spill_row(const AggK& P, uint64_t p) {
  const unsigned long long i = atomicAdd(P.counters + 0, 1ull);
  if (i < P.spill_cap)
    P.spill_rows[i] = static_cast<uint32_t>(p);
  else
    atomicOr(P.err, kDevSpillOverflow);
}

// Row of key word k (nonzero) in a finished single-key table, or nullptr.
__device__ __forceinline__ uint64_t* find_row1(uint64_t* table, uint64_t cap, int W, uint64_t k) {
  uint64_t s = __umul64hi(key_hash1(k), cap);
  for (uint64_t t = 0; t < cap; ++t) {
    uint64_t* r = table + s * W;
    const uint64_t cur = r[0];
    if (cur == k) return r;
    if (cur == 0) return nullptr;
    if (++s == cap) s = 0;
  }
  return nullptr;
}

// Merges one field block `src` (a partial aggregate) into `dst`.
__device__ __forceinline__ void merge_fields(uint64_t* dst, const uint64_t* src, const AggK& P) {
  for (int f = 0; f < P.nfields; ++f) {
    const uint64_t v = src[f];
    if (v == 0) continue;  // zero is the identity of every field
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst + f);
    switch (P.fkind[f]) {
      case F_ROWS:
      case F_NULLS:
      case F_SUMI: atomicAdd(d, static_cast<unsigned long long>(v)); break;
      case F_SUMF: atomicAdd(reinterpret_cast<double*>(d), __longlong_as_double(static_cast<long long>(v))); break;
      default: atomicMax(d, static_cast<unsigned long long>(v)); break;
    }
  }
}

// Combines the rows of every peer group and lets each group's leader apply the
// result to `f` (its field block; ignored on other lanes). `space` says where
// `f` lives (RowSpace): a warp-private row is updated without atomics (one
// leader per group and one group per row within a warp), shared and global
// rows with reductions of their state space. One loop over the fields keeps
// the code small.
template <int NV>
__device__ __forceinline__ void warp_apply(uint64_t* f, bool leader, int space, unsigned peers, const PeerPlan& pp,
                                           const AggK& P, const bool (&vv)[kMaxVals],
                                           const uint64_t (&vb)[kMaxVals]) {
  if (leader) field_red_at(space, f, F_ROWS, static_cast<uint64_t>(__popc(peers)));
#pragma unroll 1
  for (int fi = 1; fi < P.nfields; ++fi) {
    const uint8_t kind = P.fkind[fi];
    const int c = P.fcol[fi];
    bool v = false;
    uint64_t b = 0;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      if (j == c) {
        v = vv[j];
        b = vb[j];
      }
    }
    const uint64_t x = peer_reduce(field_contrib(kind, v, b), kind, pp);
    if (leader) field_red_at(space, f + fi, kind, x);
  }
}

// ---------------------------------------------------------------------------
// The aggregation kernel. MODE 0: global (no key), 1: single key, 2: multi key.
// Warps walk the rows 32 at a time (blockDim.x is a multiple of 32), so every
// lane reaches the warp-wide intrinsics.
// ---------------------------------------------------------------------------
// The CTA-private table row of a single key (side rows for key word 0 and the
// NULL key), or -1: the key is not there (read-only table) or did not fit
// within smem_probe slots.
__device__ __forceinline__ int smem_row(uint64_t* sm, int S, int W, const AggK& P, bool kv, uint64_t k, uint64_t h) {
  if (!kv) return S + 1;
  if (k == 0) return S;
  uint64_t s = h & (S - 1);
  for (int t = 0; t < P.smem_probe; ++t) {
    const uint64_t cur = ld_volatile_shared(&sm[s * W]);
    if (cur == k) return static_cast<int>(s);
    if (cur == 0) {
      if (!P.smem_insert) return -1;
      const unsigned long long old =
          atomicCAS(reinterpret_cast<unsigned long long*>(&sm[s * W]), 0ull, static_cast<unsigned long long>(k));
      if (old == 0 || old == k) return static_cast<int>(s);
    }
    s = (s + 1) & (S - 1);
  }
  return -1;
}

// Table-full signal (all lanes of the warp call it): inserts are counted per
// warp and published every 64; once the count passes P.full_at, lookups of new
// keys give up after a short probe and spill instead of walking probe_limit
// slots of a full table.
__device__ __forceinline__ void track_full(const AggK& P, unsigned lane, uint32_t iter, bool inserted_now,
                                           unsigned& pending, bool& full) {
  pending += __popc(__ballot_sync(0xffffffffu, inserted_now));
  if (pending >= 64 || (iter & 15) == 15) {
    if (lane == 0) {
      if (pending) {
        const unsigned long long before = atomicAdd(P.counters + 3, static_cast<unsigned long long>(pending));
        if (before + pending >= P.full_at) atomicExch(P.full_flag, 1u);
      }
      full = full || ld_relaxed_u32(P.full_flag) != 0;
    }
    pending = 0;
    full = __shfl_sync(0xffffffffu, full, 0);
  }
}

// Field sets with kernels of their own (qeg_warpagg.cuh): COUNT/SUM/MIN/MAX
// over an integer column plus SUM over an F64 column, and COUNT/SUM/AVG/MIN/
// MAX over one F64 column, each without and with NULL counts, and COUNT(*).
constexpr uint32_t kSpecIntF64 = 6u | spec_field(1, 0, 0) | spec_field(2, F_SUMI, 0) | spec_field(3, F_MINI, 0) |
                                 spec_field(4, F_MAXI, 0) | spec_field(5, 0, 1) | spec_field(6, F_SUMF, 1);
constexpr uint32_t kSpecIntF64Nulls = 6u | spec_field(1, F_NULLS, 0) | spec_field(2, F_SUMI, 0) |
                                      spec_field(3, F_MINI, 0) | spec_field(4, F_MAXI, 0) |
                                      spec_field(5, F_NULLS, 1) | spec_field(6, F_SUMF, 1);
constexpr uint32_t kSpecF64 = 4u | spec_field(1, 0, 0) | spec_field(2, F_SUMF, 0) | spec_field(3, F_MINF, 0) |
                              spec_field(4, F_MAXF, 0);
constexpr uint32_t kSpecF64Nulls = 4u | spec_field(1, F_NULLS, 0) | spec_field(2, F_SUMF, 0) |
                                   spec_field(3, F_MINF, 0) | spec_field(4, F_MAXF, 0);
constexpr uint32_t kSpecCount = 0u;
// SUM over an integer column plus SUM/MIN/MAX over an F64 column (bar-style
// aggregates: volume, then mean/low/high price), without NULL counts.
constexpr uint32_t kSpecIntSumF64Stats = 6u | spec_field(1, 0, 0) | spec_field(2, F_SUMI, 0) | spec_field(3, 0, 1) |
                                         spec_field(4, F_SUMF, 1) | spec_field(5, F_MINF, 1) |
                                         spec_field(6, F_MAXF, 1);

// The global (MODE 0) and single-key (MODE 1) kernels combine the rows of a
// warp that share a group before applying them (warp peer aggregation, with
// warp-private rows for the hottest keys); measured on GB300 over 64M rows
// this runs 1.3x faster than every lane applying its own row with atomics,
// for a 1024-group column as for a Zipf(1.1) column with preloaded heavy
// hitters. The composite-key kernel (MODE 2) combines peers the same way.
template <int MODE, int NV, uint32_t SPEC>
__global__ void __launch_bounds__(1024) agg_kernel(const AggK P) {
  extern __shared__ uint64_t sm[];
  const int W = P.row_words;
  // Shared-memory rows use an odd stride in 8-byte words, so the same field of
  // different rows falls in different banks.
  const int SW = W | 1;
  const int S = (MODE == 0) ? 1 : P.smem_slots;  // power of two, or 0 = off
  const int srows = (MODE == 0) ? 1 : (S > 0 ? S + 2 : 0);
  const int fo = (MODE == 2) ? 2 + P.nkeys : 1;  // field offset within a global row
  const unsigned lane = threadIdx.x & 31u;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  // Warp-private rows after the table: MODE 0 one per warp; MODE 1 (preloaded
  // table) one per warp for each of the WH hottest keys, with a rank byte per
  // table slot (0 = not one of them) and the table slot of every rank.
  const int WH = (MODE == 0) ? 1 : ((MODE == 1 && S > 0 && P.nhot > 0) ? P.warp_hot : 0);
  uint64_t* wrows = sm + srows * SW;
  uint8_t* srank = reinterpret_cast<uint8_t*>(wrows + nwarps * WH * SW);
  uint16_t* hslot = reinterpret_cast<uint16_t*>(srank + ((srows + 7) & ~7));
  const bool ranked = MODE == 1 && WH > 0;

  for (int i = threadIdx.x; i < (srows + nwarps * WH) * SW; i += blockDim.x) sm[i] = 0;
  if (ranked)
    for (int i = threadIdx.x; i < srows; i += blockDim.x) srank[i] = 0;
  __syncthreads();
  if (MODE == 1 && S > 0 && P.nhot > 0) {
    for (int i = threadIdx.x; i < P.nhot; i += blockDim.x) {
      const uint64_t k = P.hot[i];
      if (k == 0) continue;
      uint64_t s = key_hash1(k) & (S - 1);
      for (int t = 0; t < S; ++t) {
        const unsigned long long old =
            atomicCAS(reinterpret_cast<unsigned long long*>(&sm[s * SW]), 0ull, static_cast<unsigned long long>(k));
        if (old == 0 || old == k) {
          if (old == 0 && i < WH) {
            srank[s] = static_cast<uint8_t>(i + 1);
            hslot[i] = static_cast<uint16_t>(s);
          }
          break;
        }
        s = (s + 1) & (S - 1);
      }
    }
    __syncthreads();
  }

  unsigned long long inserted = 0;
  unsigned pending = 0;  // table-full signal state (track_full)
  bool full = MODE == 1 && P.full_flag && ld_relaxed_u32(P.full_flag) != 0;
  uint32_t iter = 0;
  const uint64_t step = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = static_cast<uint64_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); base < P.nrows;
       base += step, ++iter) {
    const uint64_t i = base + lane;
    bool live = i < P.nrows;
    uint64_t p = i;
    if (live && P.sel) {
      p = P.sel[i];
      if (p >= P.len) {
        atomicOr(P.err, kDevBadInput);
        live = false;
      }
    }
    bool vv[kMaxVals];
    uint64_t vb[kMaxVals];
#pragma unroll
    for (int c = 0; c < kMaxVals; ++c) {
      vv[c] = false;
      vb[c] = 0;
    }
    if (live) load_values<NV>(P, p, vv, vb);
    const unsigned livemask = __ballot_sync(0xffffffffu, live);

    if (MODE == 0) {
      const unsigned peers = live ? livemask : (1u << lane);
      const PeerPlan pp = plan_peers(peers, lane);
      if constexpr (SPEC != kGenericSpec)
        spec_apply<SPEC, NV>(&wrows[warp * SW + 1], live && __ffs(peers) - 1 == static_cast<int>(lane), kRowPrivate,
                             peers, pp, vv, vb);
      else
        warp_apply<NV>(&wrows[warp * SW + 1], live && __ffs(peers) - 1 == static_cast<int>(lane), kRowPrivate, peers,
                       pp, P, vv, vb);
      continue;
    }
    if (MODE == 1) {
      const DevCol& kc = P.key[0];
      const bool kv = live && col_valid(kc, p);
      const uint64_t k = kv ? key_word(kc, p) : 0;
      const bool key32 = kc.type == kI32 || kc.type == kSTR || kc.type == kBOOL;  // key words fit 32 bits
      // Peers: live lanes with the same key word and the same validity.
      const unsigned same = match_word64(k, lane, key32);
      const unsigned vmask = __ballot_sync(0xffffffffu, kv);
      unsigned peers = live ? (same & livemask & (kv ? vmask : ~vmask)) : (1u << lane);
      const bool leader = live && __ffs(peers) - 1 == static_cast<int>(lane);
      // The leader finds (or places) the group's row.
      uint64_t* f = nullptr;
      int space = kRowGlobal;
      const unsigned long long ins0 = inserted;
      if (leader) {
        const uint64_t h = key_hash1(k);
        const int srow = S > 0 ? smem_row(sm, S, SW, P, kv, k, h) : -1;
        if (srow >= 0) {
          const int rk = (ranked && srow < S) ? srank[srow] : 0;
          if (rk) {
            f = &wrows[(warp * WH + rk - 1) * SW + 1];
            space = kRowPrivate;
          } else {
            f = &sm[srow * SW + 1];
            space = kRowShared;
          }
        } else {
          uint64_t* r = global_row1(P, kv, k, h, inserted, full ? kFullProbe : P.probe_limit);
          if (r) f = r + 1;
        }
      }
      // A group whose row could not be placed spills each of its rows.
      const unsigned placed = __ballot_sync(0xffffffffu, f != nullptr);
      const bool ok = live && ((placed >> (__ffs(peers) - 1)) & 1u);
      if (live && !ok) {
        spill_row(P, p);
        peers = 1u << lane;
      }
      const PeerPlan pp = plan_peers(ok ? peers : (1u << lane), lane);
      if constexpr (SPEC != kGenericSpec) spec_apply<SPEC, NV>(f, leader && ok, space, peers, pp, vv, vb);
      else warp_apply<NV>(f, leader && ok, space, peers, pp, P, vv, vb);
      if (P.full_flag) track_full(P, lane, iter, inserted != ins0, pending, full);
      continue;
    }
    // MODE 2: composite key, global table only. Lanes with the same key tuple
    // combine like MODE 1: they match on the tuple hash, then every lane
    // checks its words against the match group's first lane (a lane that
    // differs -- a hash collision inside the warp -- goes alone), and the
    // group's leader finds the row and applies the combined fields.
    uint64_t words[kMaxKeys];
    uint64_t nullmask = live ? 0 : ~0ull, h = kHashSeed;
#pragma unroll
    for (int j = 0; j < kMaxKeys; ++j) {
      words[j] = 0;
      if (live && j < P.nkeys) {
        const bool kv = col_valid(P.key[j], p);
        words[j] = kv ? key_word(P.key[j], p) : 0;
        if (!kv) nullmask |= 1ull << j;
        h = hash_fold(h, kv ? words[j] : 0x9E3779B97F4A7C15ull);
      }
    }
    // (Matched on a 32-bit fold of the tuple hash; the word check below
    // drops any lane that collides.)
    const uint64_t hm = live ? h : ~static_cast<uint64_t>(lane);
    const unsigned same = __match_any_sync(0xffffffffu, static_cast<uint32_t>(hm ^ (hm >> 32)));
    const int ref = __ffs(same) - 1;
    const uint64_t ref_h = __shfl_sync(0xffffffffu, hm, ref);
    const uint64_t ref_nm = __shfl_sync(0xffffffffu, nullmask, ref);
    bool eq = ref_h == hm && ref_nm == nullmask;
#pragma unroll
    for (int j = 0; j < kMaxKeys; ++j)
      if (j < P.nkeys) eq &= __shfl_sync(0xffffffffu, words[j], ref) == words[j];
    const unsigned eqmask = __ballot_sync(0xffffffffu, eq);
    unsigned peers = (live && eq) ? (same & eqmask & livemask) : (1u << lane);
    const bool leader = live && __ffs(peers) - 1 == static_cast<int>(lane);
    uint64_t* f = nullptr;
    if (leader) {
      uint64_t* r = global_rowN(P, words, nullmask, h, inserted);
      if (r) f = r + fo;
    }
    const unsigned placed = __ballot_sync(0xffffffffu, f != nullptr);
    const bool ok = live && ((placed >> (__ffs(peers) - 1)) & 1u);
    if (live && !ok) {
      spill_row(P, p);
      peers = 1u << lane;
    }
    const PeerPlan pp = plan_peers(ok ? peers : (1u << lane), lane);
    if constexpr (SPEC != kGenericSpec) spec_apply<SPEC, NV>(f, leader && ok, kRowGlobal, peers, pp, vv, vb);
    else warp_apply<NV>(f, leader && ok, kRowGlobal, peers, pp, P, vv, vb);
  }

  // Fold the warp-private rows into the CTA table.
  if (WH > 0) {
    __syncthreads();
    for (int i = threadIdx.x; i < nwarps * WH; i += blockDim.x) {
      const uint64_t* src = &wrows[i * SW];
      if (src[1] == 0) continue;
      const int slot = (MODE == 0) ? 0 : hslot[i % WH];
      merge_fields(&sm[slot * SW + 1], src + 1, P);
    }
  }
  // Flush the CTA-private table into the global table.
  if (MODE != 2 && srows > 0) {
    __syncthreads();
    for (int sr = threadIdx.x; sr < srows; sr += blockDim.x) {
      const uint64_t* src = &sm[sr * SW];
      if (src[1] == 0) continue;  // no row landed here
      uint64_t* dst;
      if (MODE == 0) {
        dst = P.table;
      } else if (sr == S + 1) {
        dst = P.table + (P.cap + 1) * W;
      } else if (sr == S) {
        dst = P.table + P.cap * W;
      } else {
        const uint64_t k = src[0];
        dst = global_row1(P, true, k, key_hash1(k), inserted, P.probe_limit);
      }
      if (dst) {
        merge_fields(dst + 1, src + 1, P);
      } else {
        const unsigned long long i = atomicAdd(P.counters + 1, 1ull);
        if (i < P.part_cap) {
          for (int w = 0; w < W; ++w) P.spill_parts[i * W + w] = src[w];
        } else {
          atomicOr(P.err, kDevSpillOverflow);
        }
      }
    }
  }
  // Occupancy accounting: one atomic per warp.
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}

// ---------------------------------------------------------------------------
// Composite keys with a CTA-private table (QEG_AGG_SMEM in mode 2, opt-in).
// Each CTA walks one contiguous range of rows and keeps the groups it meets
// in a shared-memory table of composite rows ([state][null mask][key
// words][fields], the global row format), which it flushes into the global
// table whenever half of it is in use, and at the end. It pays off when the
// groups live at one time in a CTA's range fit its table (input with
// locality); most rows then cost shared-memory reductions, and the global
// table sees one merge per (CTA, group, flush) instead of one per row. Groups
// that miss the private table (probe limit, or no free slot while the global
// table is full) take the global path and spill as usual; partial rows that
// cannot be merged at the final flush go to the partial-row list, merged
// after the host grows the table.
// ---------------------------------------------------------------------------
constexpr int kPrivProbe = 16;

// Composite-row hash of a row's key words and NULL mask (the kernels' rule).
__device__ __forceinline__ uint64_t row_hashN(const AggK& P, const uint64_t* words, uint64_t nullmask) {
  uint64_t h = kHashSeed;
  for (int j = 0; j < P.nkeys; ++j) h = hash_fold(h, ((nullmask >> j) & 1ull) ? 0x9E3779B97F4A7C15ull : words[j]);
  return h;
}

// The private-table slot of a key tuple (found, or claimed when `may_insert`),
// or -1. A claim publishes the key words before the row's tag (fence within
// the CTA); a lookup that sees a claim in progress waits for it, bounded.
__device__ __forceinline__ int priv_row(uint64_t* sm, int S, int SW, const AggK& P, const uint64_t* words,
                                        uint64_t nullmask, uint64_t h, unsigned* used, bool may_insert) {
  const uint64_t tag = (h >> 32) | 2ull;
  int s = static_cast<int>(h & static_cast<uint64_t>(S - 1));
  for (int t = 0; t < kPrivProbe; ++t) {
    uint64_t* r = &sm[s * SW];
    uint64_t st = ld_volatile_shared(r);
    if (st == 0) {
      if (!may_insert) return -1;
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, 1ull);
      if (old == 0) {
        r[1] = nullmask;
        for (int j = 0; j < P.nkeys; ++j) r[2 + j] = words[j];
        __threadfence_block();
        atomicExch(reinterpret_cast<unsigned long long*>(r), static_cast<unsigned long long>(tag));
        atomicAdd(used, 1u);
        return s;
      }
      st = old;
    }
    int spins = 0;
    while (st == 1) {
      if (++spins > kSpinLimit) {
        atomicOr(P.err, kDevSpinTimeout);
        return -1;
      }
      st = ld_volatile_shared(r);
    }
    if (st == tag) {
      __threadfence_block();
      bool eq = ld_volatile_shared(r + 1) == nullmask;
      for (int j = 0; eq && j < P.nkeys; ++j) eq = ld_volatile_shared(r + 2 + j) == words[j];
      if (eq) return s;
    }
    s = (s + 1) & (S - 1);
  }
  return -1;
}

// Merges the private table into the global table (every thread of the CTA
// calls it). Rows that merge are cleared; the rest stay (global table full)
// or, at the final flush, go to the partial-row list.
__device__ __forceinline__ void priv_flush(uint64_t* sm, int S, int SW, const AggK& P, unsigned* used,
                                           unsigned* left, int* gfull, bool final, unsigned long long& inserted) {
  const int W = P.row_words;
  const int fo = 2 + P.nkeys;
  if (threadIdx.x == 0) *left = 0;
  __syncthreads();
  for (int slot = threadIdx.x; slot < S; slot += blockDim.x) {
    uint64_t* src = &sm[slot * SW];
    if (src[0] < 2) continue;
    uint64_t words[kMaxKeys];
    for (int j = 0; j < P.nkeys; ++j) words[j] = src[2 + j];
    uint64_t* dst = global_rowN(P, words, src[1], row_hashN(P, words, src[1]), inserted);
    if (dst) {
      merge_fields(dst + fo, src + fo, P);
    } else if (final) {
      const unsigned long long i = atomicAdd(P.counters + 1, 1ull);
      if (i < P.part_cap) {
        for (int w = 0; w < W; ++w) P.spill_parts[i * W + w] = src[w];
      } else {
        atomicOr(P.err, kDevSpillOverflow);
      }
    } else {
      atomicAdd(left, 1u);
      continue;
    }
    for (int w = 0; w < W; ++w) src[w] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *used = *left;
    if (*left >= static_cast<unsigned>(S / 2)) *gfull = 1;
  }
  __syncthreads();
}

template <int NV, uint32_t SPEC>
__global__ void __launch_bounds__(512, 2) agg2_private_kernel(const AggK P) {
  extern __shared__ uint64_t sm[];
  const int W = P.row_words;
  const int SW = W | 1;
  const int S = P.smem_slots;
  const int fo = 2 + P.nkeys;
  const unsigned lane = threadIdx.x & 31u;
  __shared__ unsigned s_used, s_left;
  __shared__ int s_gfull;
  for (int i = threadIdx.x; i < S * SW; i += blockDim.x) sm[i] = 0;
  if (threadIdx.x == 0) {
    s_used = 0;
    s_gfull = 0;
  }
  __syncthreads();
  unsigned long long inserted = 0;
  const uint64_t per = (P.nrows + gridDim.x - 1) / gridDim.x;
  const uint64_t chunk = (per + blockDim.x - 1) / blockDim.x * blockDim.x;
  const uint64_t r0 = static_cast<uint64_t>(blockIdx.x) * chunk;
  const uint64_t r1 = r0 + chunk < P.nrows ? r0 + chunk : P.nrows;
  // Block-uniform loop: every thread makes the same passes (the flush check
  // synchronises the CTA after each one).
  for (uint64_t base = r0; base < r1; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    bool live = i < r1;
    uint64_t p = i;
    if (live && P.sel) {
      p = P.sel[i];
      if (p >= P.len) {
        atomicOr(P.err, kDevBadInput);
        live = false;
      }
    }
    bool vv[kMaxVals];
    uint64_t vb[kMaxVals];
#pragma unroll
    for (int c = 0; c < kMaxVals; ++c) {
      vv[c] = false;
      vb[c] = 0;
    }
    if (live) load_values<NV>(P, p, vv, vb);
    const unsigned livemask = __ballot_sync(0xffffffffu, live);
    uint64_t words[kMaxKeys];
    uint64_t nullmask = live ? 0 : ~0ull, h = kHashSeed;
#pragma unroll
    for (int j = 0; j < kMaxKeys; ++j) {
      words[j] = 0;
      if (live && j < P.nkeys) {
        const bool kv = col_valid(P.key[j], p);
        words[j] = kv ? key_word(P.key[j], p) : 0;
        if (!kv) nullmask |= 1ull << j;
        h = hash_fold(h, kv ? words[j] : 0x9E3779B97F4A7C15ull);
      }
    }
    // Peers: lanes with the same key tuple (hash match, then an exact check
    // against the match group's first lane), as in agg_kernel's mode 2.
    // (Matched on a 32-bit fold of the tuple hash; the word check below
    // drops any lane that collides.)
    const uint64_t hm = live ? h : ~static_cast<uint64_t>(lane);
    const unsigned same = __match_any_sync(0xffffffffu, static_cast<uint32_t>(hm ^ (hm >> 32)));
    const int ref = __ffs(same) - 1;
    const uint64_t ref_h = __shfl_sync(0xffffffffu, hm, ref);
    const uint64_t ref_nm = __shfl_sync(0xffffffffu, nullmask, ref);
    bool eq = ref_h == hm && ref_nm == nullmask;
#pragma unroll
    for (int j = 0; j < kMaxKeys; ++j)
      if (j < P.nkeys) eq &= __shfl_sync(0xffffffffu, words[j], ref) == words[j];
    const unsigned eqmask = __ballot_sync(0xffffffffu, eq);
    unsigned peers = (live && eq) ? (same & eqmask & livemask) : (1u << lane);
    const bool leader = live && __ffs(peers) - 1 == static_cast<int>(lane);
    uint64_t* f = nullptr;
    int space = kRowGlobal;
    if (leader) {
      const int slot = priv_row(sm, S, SW, P, words, nullmask, h, &s_used, s_gfull == 0);
      if (slot >= 0) {
        f = &sm[slot * SW + fo];
        space = kRowShared;
      } else {
        uint64_t* r = global_rowN(P, words, nullmask, h, inserted);
        if (r) f = r + fo;
      }
    }
    const unsigned placed = __ballot_sync(0xffffffffu, f != nullptr);
    const bool ok = live && ((placed >> (__ffs(peers) - 1)) & 1u);
    if (live && !ok) {
      spill_row(P, p);
      peers = 1u << lane;
    }
    const PeerPlan pp = plan_peers(ok ? peers : (1u << lane), lane);
    if constexpr (SPEC != kGenericSpec) spec_apply<SPEC, NV>(f, leader && ok, space, peers, pp, vv, vb);
    else warp_apply<NV>(f, leader && ok, space, peers, pp, P, vv, vb);
    // One CTA-wide decision (a barrier that also ORs the predicate), so every
    // thread enters the flush, or none does.
    if (__syncthreads_or(threadIdx.x == 0 && s_used >= static_cast<unsigned>(S / 2) && s_gfull == 0))
      priv_flush(sm, S, SW, P, &s_used, &s_left, &s_gfull, false, inserted);
  }
  __syncthreads();
  priv_flush(sm, S, SW, P, &s_used, &s_left, &s_gfull, true, inserted);
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}

// Re-inserts every occupied row of `old` into the (zeroed) table of P.
template <int MODE>
__global__ void rehash_kernel(const AggK P, const uint64_t* __restrict__ old, uint64_t old_cap) {
  const int W = P.row_words;
  unsigned long long inserted = 0;
  const uint64_t total = (MODE == 1) ? old_cap + 2 : old_cap;
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < total;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t* src = old + s * W;
    uint64_t* dst = nullptr;
    if (MODE == 1) {
      if (s == old_cap) {
        dst = P.table + P.cap * W;
      } else if (s == old_cap + 1) {
        dst = P.table + (P.cap + 1) * W;
      } else {
        const uint64_t k = src[0];
        if (k == 0) continue;
        // The new table has room for every row: probe as far as it takes.
        dst = global_row1(P, true, k, key_hash1(k), inserted, static_cast<int>(P.cap < (1ull << 30) ? P.cap : (1ull << 30)));
      }
      if (!dst) {
        atomicOr(P.err, kDevSpillOverflow);
        continue;
      }
      for (int f = 1; f < W; ++f) dst[f] = src[f];
    } else {
      const uint64_t st = src[0];
      if (st < 2) continue;
      uint64_t words[kMaxKeys];
      for (int j = 0; j < P.nkeys; ++j) words[j] = src[2 + j];
      uint64_t h = kHashSeed;
      for (int j = 0; j < P.nkeys; ++j) h = hash_fold(h, ((src[1] >> j) & 1) ? 0x9E3779B97F4A7C15ull : words[j]);
      dst = global_rowN(P, words, src[1], h, inserted);
      if (!dst) {
        atomicOr(P.err, kDevSpillOverflow);
        continue;
      }
      for (int f = 2 + P.nkeys; f < W; ++f) dst[f] = src[f];
    }
  }
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}

// Merges spilled partial rows (single-key rows, or composite rows of the
// composite private tables) into the table.
// ---------------------------------------------------------------------------
// Partitioned strategy (QEG_AGG_PARTITIONED, single key). Three passes over
// the batch: a sizing pass counts, per key-hash partition, the rows that are
// not heavy hitters; the first pass aggregates the heavy hitters in read-only
// per-CTA tables and appends every other row to its partition's region of the
// pool; the second pass aggregates one partition per CTA in shared memory and
// appends the groups to the tail rows. Heavy-hitter membership and partitions
// use cheap multiplicative hashes (one 64-bit multiply); the global table and
// the tail rows keep the table's own key hash.
// ---------------------------------------------------------------------------
constexpr uint64_t kPartMul = 0xD1B54A32D192ED03ull;

// Partition hash of key word k: the partition is its top bits, a second-pass
// table slot the bits below them.
__device__ __forceinline__ uint64_t part_mix(uint64_t k) { return (k ^ (k >> 31)) * kPartMul; }

// Hash of a hot-key lookup (its top bits pick the bucket) and the slot of a
// key given its bucket's displacement d: the displacement is mixed in before
// the final multiply, so each d places a bucket's keys independently.
__host__ __device__ __forceinline__ uint64_t hot_phf_hash(uint64_t k) {
  return (k ^ (k >> 29)) * 0x9E3779B97F4A7C15ull;
}
__host__ __device__ __forceinline__ uint32_t hot_phf_slot(uint64_t h, uint32_t d, int lgT) {
  return static_cast<uint32_t>(((h ^ (static_cast<uint64_t>(d) * 0xC2B2AE3D27D4EB4Full)) * 0x94D049BB133111EBull) >>
                               (64 - lgT));
}

// Heavy-hitter lookup: a perfect hash of the hot key words built on the host
// (hot_phf_build; hash-and-displace), so a lookup is a fixed sequence of two
// multiplies and three shared-memory loads with no probe loop. Layout (words
// of 8 bytes): [2^lgT slot keys (0 = empty)][2^lgT u16 slot ranks][2^lgB u16
// bucket displacements].
__device__ __forceinline__ int phf_rank(const uint64_t* skey, const uint16_t* srank, const uint16_t* disp, int lgT,
                                        int lgB, uint64_t k) {
  const uint64_t h = hot_phf_hash(k);
  const uint32_t b = static_cast<uint32_t>(h >> (64 - lgB));
  const uint32_t s = hot_phf_slot(h, disp[b], lgT);
  return skey[s] == k ? static_cast<int>(srank[s]) : -1;
}

// Parameters of the partitioned passes beyond AggK.
struct PartA {
  int nhot;                  // heavy hitters (ranks 0..nhot-1); rank nhot: NULL key, nhot + 1: key word 0
  int rw;                    // field words per heavy-hitter row (odd)
  int lgT, lgB;              // heavy-hitter perfect hash: 2^lgT slots, 2^lgB buckets
  const uint64_t* phf;       // its words (phf_words of them)
  int phf_words;
  unsigned long long* hist;  // sizing pass: rows per partition
};

// Copies the heavy-hitter perfect hash into shared memory. All threads call
// it; ends with a barrier.
__device__ __forceinline__ void load_phf(const PartA& A, uint64_t* sm) {
  for (int i = threadIdx.x; i < A.phf_words; i += blockDim.x) sm[i] = __ldg(A.phf + i);
  __syncthreads();
}

// Rows each thread keeps in flight in the partitioned passes: fewer when
// more value columns travel with each row (registers).
template <int NV>
constexpr int part_rows() {
  return NV <= 2 ? 4 : (NV <= 4 ? 2 : 1);
}

// Sizing pass: rows per partition of every row that will reach the pool (a
// non-NULL key other than key word 0 and not a heavy hitter). 32-bit counters
// per CTA in shared memory, added to A.hist at the end. Each thread has R
// rows in flight per iteration (coalesced: row j of a tile is j * blockDim.x
// + threadIdx.x), their key loads issued before any is used.
template <int R>
__global__ void __launch_bounds__(1024) part_hist_kernel(const AggK P, const PartA A) {
  extern __shared__ uint64_t hsm[];
  const int T = 1 << A.lgT;
  const uint64_t* skey = hsm;
  const uint16_t* srank = reinterpret_cast<const uint16_t*>(hsm + T);
  const uint16_t* disp = srank + T;
  uint32_t* cnt = reinterpret_cast<uint32_t*>(hsm + A.phf_words);
  const uint32_t np = 1u << (64 - P.part_shift);
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) cnt[i] = 0;
  load_phf(A, hsm);
  const DevCol& kc = P.key[0];
  const uint64_t tile = static_cast<uint64_t>(blockDim.x) * R;
  for (uint64_t base = blockIdx.x * tile; base < P.nrows; base += static_cast<uint64_t>(gridDim.x) * tile) {
    uint64_t kw[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint64_t i = base + static_cast<uint64_t>(j) * blockDim.x + threadIdx.x;
      bool ok = i < P.nrows;
      uint64_t p = i;
      if (ok && P.sel) {
        p = P.sel[i];
        ok = p < P.len;  // (the first pass reports it)
      }
      ok = ok && col_valid(kc, p);
      kw[j] = ok ? key_word(kc, p) : 0;
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint64_t k = kw[j];
      if (k != 0 && phf_rank(skey, srank, disp, A.lgT, A.lgB, k) < 0)
        atomicAdd(&cnt[part_mix(k) >> P.part_shift], 1u);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
    if (cnt[i]) atomicAdd(A.hist + i, static_cast<unsigned long long>(cnt[i]));
}

// First pass. Heavy hitters (and the NULL key and key word 0, which always
// have rows) aggregate into the CTA's rows by rank with warp peer aggregation
// (matched on the 32-bit rank); every other row is appended to its
// partition's region. R rows per thread are loaded before any is applied.
// At the end each CTA merges its rows into the global table.
template <int NV, uint32_t SPEC, int R>
__global__ void __launch_bounds__(512) part_pass1_kernel(const AggK P, const PartA A) {
  extern __shared__ uint64_t psm[];
  const int T = 1 << A.lgT;
  const uint64_t* skey = psm;
  const uint16_t* srank = reinterpret_cast<const uint16_t*>(psm + T);
  const uint16_t* disp = srank + T;
  uint64_t* rows = psm + A.phf_words;  // (nhot + 2) rows of A.rw words
  const unsigned lane = threadIdx.x & 31u;
  const int RW = A.rw;
  const int nrow = A.nhot + 2;
  for (int i = threadIdx.x; i < nrow * RW; i += blockDim.x) rows[i] = 0;
  load_phf(A, psm);
  const DevCol& kc = P.key[0];
  const uint64_t tile = static_cast<uint64_t>(blockDim.x) * R;
  for (uint64_t base = blockIdx.x * tile; base < P.nrows; base += static_cast<uint64_t>(gridDim.x) * tile) {
    uint64_t pr[R], kw[R];
    bool live[R], kv[R];
    bool vv[R][kMaxVals];
    uint64_t vb[R][kMaxVals];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint64_t i = base + static_cast<uint64_t>(j) * blockDim.x + threadIdx.x;
      live[j] = i < P.nrows;
      uint64_t p = i;
      if (live[j] && P.sel) {
        p = P.sel[i];
        if (p >= P.len) {
          atomicOr(P.err, kDevBadInput);
          live[j] = false;
        }
      }
      pr[j] = p;
#pragma unroll
      for (int c = 0; c < kMaxVals; ++c) {
        vv[j][c] = false;
        vb[j][c] = 0;
      }
      if (live[j]) load_values<NV>(P, p, vv[j], vb[j]);
      kv[j] = live[j] && col_valid(kc, p);
      kw[j] = kv[j] ? key_word(kc, p) : 0;
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint64_t k = kw[j];
      int rank = -1;
      if (live[j]) rank = !kv[j] ? A.nhot : (k == 0 ? A.nhot + 1 : phf_rank(skey, srank, disp, A.lgT, A.lgB, k));
      const bool hot = rank >= 0;
      if (__ballot_sync(0xffffffffu, hot)) {
        // Lanes of one rank combine their rows; the lowest applies them.
        const unsigned peers = __match_any_sync(0xffffffffu, hot ? static_cast<unsigned>(rank) : (0x80000000u | lane));
        const bool leader = hot && __ffs(peers) - 1 == static_cast<int>(lane);
        const PeerPlan pp = plan_peers(peers, lane);
        uint64_t* f = rows + static_cast<size_t>(hot ? rank : 0) * RW;
        if constexpr (SPEC != kGenericSpec) spec_apply<SPEC, NV>(f, leader, kRowShared, peers, pp, vv[j], vb[j]);
        else warp_apply<NV>(f, leader, kRowShared, peers, pp, P, vv[j], vb[j]);
      }
      if (live[j] && !hot) {
        // Partitions are many: lanes rarely share one, so each reserves alone.
        const uint32_t part = static_cast<uint32_t>(part_mix(k) >> P.part_shift);
        const uint64_t at = P.part_off[part] + atomicAdd(P.part_fill + part, 1ull);
        if (at < P.part_off[part + 1]) {
          P.pool_key[at] = k;
#pragma unroll
          for (int c = 0; c < NV; ++c)
            if (c < P.nvals) P.pool_val[c][at] = vb[j][c];
        } else {
          spill_row(P, pr[j]);  // (the sizing pass counted every such row: not reached)
        }
      }
    }
  }
  __syncthreads();
  // Merge the CTA's rows into the global table.
  unsigned long long inserted = 0;
  const int W = P.row_words;
  for (int r = threadIdx.x; r < nrow; r += blockDim.x) {
    const uint64_t* src = rows + static_cast<size_t>(r) * RW;
    if (src[0] == 0) continue;  // no row counted here
    uint64_t* dst;
    if (r == A.nhot) {
      dst = P.table + (P.cap + 1) * W;
    } else if (r == A.nhot + 1) {
      dst = P.table + P.cap * W;
    } else {
      const uint64_t k = P.hot[r];
      dst = global_row1(P, true, k, key_hash1(k), inserted, P.probe_limit);
      if (!dst) {
        const unsigned long long j = atomicAdd(P.counters + 1, 1ull);
        if (j < P.part_cap) {
          P.spill_parts[j * W] = k;
          for (int w = 1; w < W; ++w) P.spill_parts[j * W + w] = src[w - 1];
        } else {
          atomicOr(P.err, kDevSpillOverflow);
        }
        continue;
      }
    }
    merge_fields(dst + 1, src, P);
  }
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}

// Slot of key word k (nonzero, partition hash m) in a second-pass table of
// S = 2^lgS slots with row stride SW, inserting it when absent; -1 when S / 2
// slots were probed (the table is too full).
__device__ __forceinline__ int part_smem_slot(uint64_t* sm, int lgS, int shift, int SW, uint64_t k, uint64_t m) {
  const uint32_t mask = (1u << lgS) - 1u;
  uint32_t s = static_cast<uint32_t>(m >> (shift - lgS)) & mask;
  for (uint32_t t = 0; t <= (mask >> 1); ++t) {
    const uint64_t cur = ld_volatile_shared(&sm[static_cast<size_t>(s) * SW]);
    if (cur == k) return static_cast<int>(s);
    if (cur == 0) {
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(&sm[static_cast<size_t>(s) * SW]),
                                               0ull, static_cast<unsigned long long>(k));
      if (old == 0 || old == k) return static_cast<int>(s);
    }
    s = (s + 1) & mask;
  }
  return -1;
}

// Second pass: each CTA takes partitions in turn and aggregates the
// partition's pool rows (every key nonzero and non-NULL, every value present)
// in a shared-memory table, with R rows per thread loaded before any is
// applied; lanes whose rows share a slot (a key) combine them first (warp peer
// aggregation, matched on the 32-bit slot); then it appends the table's groups to
// the tail rows with one reservation per CTA and clears the rows it used. A
// partition with more groups than the table holds is listed as failed and
// appends nothing (the host aggregates it into the global table instead), so
// the pass can be re-run with a larger tail buffer.
template <int NV, uint32_t SPEC, int R>
__global__ void __launch_bounds__(1024) part_agg_kernel(const AggK P, const PartB B) {
  extern __shared__ uint64_t sm[];
  __shared__ int s_fail;
  __shared__ unsigned long long s_wbase[32];
  const int W = P.row_words, SW = W | 1, S = B.slots;
  int lgS = 0;
  while ((1 << lgS) < S) ++lgS;
  const unsigned lane = threadIdx.x & 31u;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int i = threadIdx.x; i < S * SW; i += blockDim.x) sm[i] = 0;
  for (uint32_t part = blockIdx.x; part < B.nparts; part += gridDim.x) {
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    const uint64_t begin = B.part_off[part];
    const uint64_t n = B.part_off[part + 1] - begin;
    const uint64_t tile = static_cast<uint64_t>(blockDim.x) * R;
    for (uint64_t b0 = 0; b0 < n; b0 += tile) {
      uint64_t kw[R];
      bool vv[R][kMaxVals];
      uint64_t vb[R][kMaxVals];
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const uint64_t at = b0 + static_cast<uint64_t>(j) * blockDim.x + threadIdx.x;
        const bool ok = at < n;
        kw[j] = ok ? static_cast<uint64_t>(__ldcs(reinterpret_cast<const unsigned long long*>(B.pool_key + begin + at)))
                   : 0;
#pragma unroll
        for (int c = 0; c < kMaxVals; ++c) {
          vv[j][c] = ok && c < NV && c < P.nvals;
          vb[j][c] = (ok && c < NV && c < P.nvals)
                         ? static_cast<uint64_t>(
                               __ldcs(reinterpret_cast<const unsigned long long*>(B.pool_val[c] + begin + at)))
                         : 0;
        }
      }
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const uint64_t k = kw[j];
        const bool live = k != 0;  // (pool keys are nonzero: zero marks a row past the partition's end)
        int slot = -1;
        if (live) {
          slot = part_smem_slot(sm, lgS, P.part_shift, SW, k, part_mix(k));
          if (slot < 0) s_fail = 1;
        }
        const bool ok = slot >= 0;
        if (__ballot_sync(0xffffffffu, ok)) {
          // A slot holds one key: lanes of one slot combine their rows.
          const unsigned peers = __match_any_sync(0xffffffffu, ok ? static_cast<unsigned>(slot) : (0x80000000u | lane));
          const bool leader = ok && __ffs(peers) - 1 == static_cast<int>(lane);
          const PeerPlan pp = plan_peers(peers, lane);
          uint64_t* f = &sm[static_cast<size_t>(ok ? slot : 0) * SW + 1];
          if constexpr (SPEC != kGenericSpec) spec_apply<SPEC, NV>(f, leader, kRowShared, peers, pp, vv[j], vb[j]);
          else warp_apply<NV>(f, leader, kRowShared, peers, pp, P, vv[j], vb[j]);
        }
      }
    }
    __syncthreads();
    const bool failed = s_fail != 0;
    // Groups out: count the occupied slots per warp, one reservation per CTA.
    unsigned cnt = 0;
    for (int s0 = warp * 32; s0 < S; s0 += nwarps * 32) {
      const int s = s0 + static_cast<int>(lane);
      cnt += __popc(__ballot_sync(0xffffffffu, s < S && sm[static_cast<size_t>(s) * SW] != 0));
    }
    if (lane == 0) s_wbase[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long run = 0;
      for (int w = 0; w < nwarps; ++w) {
        const unsigned long long c = s_wbase[w];
        s_wbase[w] = run;
        run += c;
      }
      unsigned long long base = 0;
      if (failed) {
        const unsigned long long fi = atomicAdd(B.counters + 1, 1ull);
        if (fi < B.nparts) B.failed[fi] = part;
      } else if (run) {
        base = atomicAdd(B.counters + 0, run);
      }
      for (int w = 0; w < nwarps; ++w) s_wbase[w] += base;
    }
    __syncthreads();
    unsigned long long pos = s_wbase[warp];
    for (int s0 = warp * 32; s0 < S; s0 += nwarps * 32) {
      const int s = s0 + static_cast<int>(lane);
      const bool occ = s < S && sm[static_cast<size_t>(s) * SW] != 0;
      const unsigned m = __ballot_sync(0xffffffffu, occ);
      if (occ) {
        const unsigned long long o = pos + __popc(m & ((1u << lane) - 1u));
        if (!failed && o < B.tails_cap)
          for (int w = 0; w < W; ++w) B.tails[o * W + w] = sm[static_cast<size_t>(s) * SW + w];
        for (int w = 0; w < W; ++w) sm[static_cast<size_t>(s) * SW + w] = 0;
      }
      pos += __popc(m);
    }
    __syncthreads();
  }
}

template <int MODE>
__global__ void merge_parts_kernel(const AggK P, const uint64_t* __restrict__ parts, uint64_t n) {
  const int W = P.row_words;
  unsigned long long inserted = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t* src = parts + i * W;
    uint64_t* dst;
    int fo;
    if (MODE == 2) {
      uint64_t words[kMaxKeys];
      for (int j = 0; j < P.nkeys; ++j) words[j] = src[2 + j];
      dst = global_rowN(P, words, src[1], row_hashN(P, words, src[1]), inserted);
      fo = 2 + P.nkeys;
    } else {
      const uint64_t k = src[0];
      // The caller sized the table for these rows: probe as far as it takes.
      dst = global_row1(P, true, k, key_hash1(k), inserted, static_cast<int>(P.cap < (1ull << 30) ? P.cap : (1ull << 30)));
      fo = 1;
    }
    if (!dst) {
      atomicOr(P.err, kDevSpillOverflow);
      continue;
    }
    merge_fields(dst + fo, src + fo, P);
  }
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}

// Writes one output value of result type `t` from a 64-bit word.
__device__ __forceinline__ void store_typed(void* base, uint64_t i, int32_t t, uint64_t w) {
  switch (t) {
    case kI32:
    case kSTR: static_cast<int32_t*>(base)[i] = static_cast<int32_t>(static_cast<uint32_t>(w)); break;
    case kBOOL: static_cast<uint8_t*>(base)[i] = static_cast<uint8_t>(w & 1ull); break;
    default: static_cast<uint64_t*>(base)[i] = w; break;
  }
}

// Compacts occupied rows into dense output columns (keys, then aggregates),
// applying the reference's finalisation (ops/agg_internal.h:169-229).
template <int MODE>
__global__ void __launch_bounds__(1024) finalize_kernel(const AggK P, const FinK F) {
  const int W = P.row_words;
  const int fo = (MODE == 2) ? 2 + P.nkeys : 1;
  const uint64_t total = (MODE == 0) ? 1 : (MODE == 1 ? P.cap + 2 : P.cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  // Output positions: one atomic per CTA and pass (the warps' counts are
  // prefixed in shared memory), not one per warp -- a sparse table of tens of
  // millions of slots would otherwise serialise on the counter.
  __shared__ unsigned long long wpos[32];
  // kFinPer slots per thread and pass: fewer passes, so fewer barriers.
  constexpr int kFinPer = 4;
  const uint64_t span = static_cast<uint64_t>(blockDim.x) * kFinPer;
  for (uint64_t base = blockIdx.x * span; base < total; base += gridDim.x * span) {
    bool occk[kFinPer];
    unsigned mk[kFinPer];
    unsigned cnt = 0;
#pragma unroll
    for (int k = 0; k < kFinPer; ++k) {
      const uint64_t sk = base + static_cast<uint64_t>(k) * blockDim.x + threadIdx.x;
      bool o = false;
      if (sk < total) {
        const uint64_t* rk = P.table + sk * W;
        if (MODE == 0) o = true;
        else if (MODE == 1) o = (sk < P.cap) ? (rk[0] != 0) : (rk[1] != 0);
        else o = rk[0] >= 2;
        if (MODE == 1 && o && F.merge_table && sk < P.cap) {
          // The key also has a row in the second table: merge into it there.
          uint64_t* m = find_row1(F.merge_table, F.merge_cap, W, rk[0]);
          if (m) {
            merge_fields(m + 1, rk + 1, P);
            o = false;
          }
        }
      }
      occk[k] = o;
      mk[k] = __ballot_sync(0xffffffffu, o);
      cnt += __popc(mk[k]);
    }
    if (lane == 0) wpos[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long run = 0;
      for (int w = 0; w < nwarps; ++w) {
        const unsigned long long c = wpos[w];
        wpos[w] = run;
        run += c;
      }
      const unsigned long long b = run ? atomicAdd(F.out_count, run) : 0;
      for (int w = 0; w < nwarps; ++w) wpos[w] += b;
    }
    __syncthreads();
    unsigned long long wbase = wpos[warp];
    __syncthreads();  // wpos is rewritten by the next pass
    for (int k = 0; k < kFinPer; ++k) {
      const unsigned m = mk[k];
      const unsigned long long kbase = wbase;
      wbase += __popc(m);
      if (!occk[k]) continue;
      const uint64_t s = base + static_cast<uint64_t>(k) * blockDim.x + threadIdx.x;
      const uint64_t* r = P.table + s * W;
      const uint64_t o = kbase + __popc(m & ((1u << lane) - 1u));
      if (o >= F.out_cap) {
        atomicOr(P.err, kDevSpillOverflow);
        continue;
      }
      // keys
      for (int j = 0; j < P.nkeys; ++j) {
        bool isnull;
        uint64_t w;
        if (MODE == 1) {
          isnull = (s == P.cap + 1);
          w = (s == P.cap) ? 0 : r[0];
          if (F.packed_width > 0) {  // (partition key, bucket index) packed in one word
            isnull = false;
            w = j == 0 ? static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(w >> 32))))
                       : static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(w))) *
                                               F.packed_width);
          }
        } else {
          isnull = (r[1] >> j) & 1ull;
          w = r[2 + j];
        }
        F.valid[j][o] = isnull ? 0 : 1;
        store_typed(F.vals[j], o, F.rtype[j], isnull ? 0 : w);
      }
      // aggregates
      const uint64_t* f = r + fo;
      const uint64_t rows = f[0];
      for (int a = 0; a < F.naggs; ++a) {
        const int oc = P.nkeys + a;
        const int vf = F.vfield[a];
        const uint64_t nulls = F.nfield[a] >= 0 ? f[F.nfield[a]] : 0;
        const uint64_t nn = rows - nulls;
        const int32_t rt = F.rtype[oc];
        uint8_t ok = 1;
        uint64_t w = 0;
        switch (F.func[a]) {
          case 0: w = rows; break;  // COUNT(*)
          case 1: w = nn; break;    // COUNT(col)
          case 2:                   // SUM
            if (nn == 0) ok = 0;
            else w = f[vf];
            break;
          case 5: {  // AVG = sum / non-null count, in double (ops/agg_internal.h:217-227)
            if (nn == 0) {
              ok = 0;
            } else {
              const double sum = (P.fkind[vf] == F_SUMF) ? __longlong_as_double(static_cast<long long>(f[vf]))
                                                          : static_cast<double>(static_cast<int64_t>(f[vf]));
              w = static_cast<uint64_t>(__double_as_longlong(sum / static_cast<double>(nn)));
            }
            break;
          }
          default: {  // MIN / MAX
            if (nn == 0) {
              ok = 0;
              break;
            }
            const uint8_t fk = P.fkind[vf];
            const uint64_t e = f[vf];
            if (fk == F_MINF) w = dec_f64_bits(~e);
            else if (fk == F_MAXF) w = dec_f64_bits(e);
            else if (fk == F_MINI) w = static_cast<uint64_t>(dec_i64(~e));
            else w = static_cast<uint64_t>(dec_i64(e));
            break;
          }
        }
        F.valid[oc][o] = ok;
        store_typed(F.vals[oc], o, rt, ok ? w : 0);
      }
    }
  }
}

int32_t agg_result_type(int32_t func, int32_t in) {
  switch (func) {
    case QEG_COUNT_STAR:
    case QEG_COUNT: return QEG_I64;
    case QEG_SUM: return in == QEG_F64 ? QEG_F64 : QEG_I64;
    case QEG_AVG: return QEG_F64;
    default: return in;
  }
}

uint64_t next_pow2(uint64_t v) {
  uint64_t c = 1;
  while (c < v) c <<= 1;
  return c;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

void AggState::plan(const int32_t* col_types, int ncols, const uint32_t* key_cols, int nk,
                    const qeg_agg_spec* aggs_in, int na) {
  require(ncols > 0 && col_types != nullptr, "aggregate needs an input schema");
  require(na >= 1 && aggs_in != nullptr, "Aggregate needs >=1 aggregate");
  require(nk >= 0 && nk <= kMaxKeys, "GPU aggregate supports 0..8 key columns");
  require(na <= kMaxAggs, "GPU aggregate supports at most 32 aggregates");
  types.assign(col_types, col_types + ncols);
  for (int32_t t : types) require(t >= QEG_I32 && t <= QEG_STR, "unknown column type");
  keys.assign(key_cols, key_cols + nk);
  for (uint32_t k : keys) require(k < static_cast<uint32_t>(ncols), "key column index out of range");
  aggs.assign(aggs_in, aggs_in + na);
  mode = nk == 0 ? 0 : (nk == 1 ? 1 : 2);

  // Distinct value columns and their fields, grouped by column.
  val_cols.clear();
  fkind.assign(1, F_ROWS);
  std::vector<std::vector<uint8_t>> per_col;
  vfield.assign(na, -1);
  nfield.assign(na, -1);
  rtypes.clear();
  for (uint32_t k : keys) rtypes.push_back(types[k]);
  struct Want { int col; uint8_t kind; };
  std::vector<Want> wants;
  for (int a = 0; a < na; ++a) {
    const qeg_agg_spec& s = aggs[a];
    require(s.func >= QEG_COUNT_STAR && s.func <= QEG_AVG, "unknown aggregate function");
    if (s.func == QEG_COUNT_STAR) {
      rtypes.push_back(QEG_I64);
      continue;
    }
    require(s.input_col < static_cast<uint32_t>(ncols), "aggregate input column out of range");
    const int32_t in = types[s.input_col];
    if (in == QEG_STR && (s.func == QEG_SUM || s.func == QEG_AVG))
      require(false, s.func == QEG_SUM ? "SUM is not defined on STR (VARCHAR)"
                                       : "AVG is not defined on STR (VARCHAR)");
    rtypes.push_back(agg_result_type(s.func, in));
  }
  // Assign fields per distinct column.
  std::vector<int> colslot(ncols, -1);
  for (int a = 0; a < na; ++a) {
    const qeg_agg_spec& s = aggs[a];
    if (s.func == QEG_COUNT_STAR) continue;
    if (colslot[s.input_col] < 0) {
      require(static_cast<int>(val_cols.size()) < kMaxVals, "GPU aggregate supports at most 8 input columns");
      colslot[s.input_col] = static_cast<int>(val_cols.size());
      val_cols.push_back(s.input_col);
      per_col.emplace_back();
    }
    const int vc = colslot[s.input_col];
    const bool isf = types[s.input_col] == QEG_F64;
    uint8_t kind = F_NULLS;
    if (s.func == QEG_SUM || s.func == QEG_AVG) kind = isf ? F_SUMF : F_SUMI;
    if (s.func == QEG_MIN) kind = isf ? F_MINF : F_MINI;
    if (s.func == QEG_MAX) kind = isf ? F_MAXF : F_MAXI;
    auto& v = per_col[vc];
    if (std::find(v.begin(), v.end(), F_NULLS) == v.end()) v.insert(v.begin(), F_NULLS);
    if (kind != F_NULLS && std::find(v.begin(), v.end(), kind) == v.end()) v.push_back(kind);
  }
  // Fields of a column in kind order (NULLS, sums, MINs, MAXes) whatever the
  // order of the aggregates, so equal field sets share a specialised kernel.
  for (auto& v : per_col) std::sort(v.begin(), v.end());
  cfirst.assign(val_cols.size(), 0);
  cnf.assign(val_cols.size(), 0);
  for (size_t c = 0; c < val_cols.size(); ++c) {
    cfirst[c] = static_cast<int>(fkind.size());
    cnf[c] = static_cast<int>(per_col[c].size());
    for (uint8_t k : per_col[c]) fkind.push_back(k);
  }
  require(static_cast<int>(fkind.size()) <= kMaxFields, "too many aggregate state fields for the GPU path");
  for (int a = 0; a < na; ++a) {
    const qeg_agg_spec& s = aggs[a];
    if (s.func == QEG_COUNT_STAR) continue;
    const int vc = colslot[s.input_col];
    const bool isf = types[s.input_col] == QEG_F64;
    uint8_t kind = F_NULLS;
    if (s.func == QEG_SUM || s.func == QEG_AVG) kind = isf ? F_SUMF : F_SUMI;
    if (s.func == QEG_MIN) kind = isf ? F_MINF : F_MINI;
    if (s.func == QEG_MAX) kind = isf ? F_MAXF : F_MAXI;
    for (int k = 0; k < cnf[vc]; ++k) {
      if (fkind[cfirst[vc] + k] == F_NULLS) nfield[a] = cfirst[vc] + k;
      if (fkind[cfirst[vc] + k] == kind) vfield[a] = cfirst[vc] + k;
    }
  }
  nfields = static_cast<int>(fkind.size());
  row_words = (mode == 2 ? 2 + nk : 1) + nfields;
}

DevCol AggState::key_col(const std::vector<StagedCol>& staged, size_t j) const {
  DevCol c = staged[keys[j]].dev;
  c.bucket = (bucket_width > 0 && j + 1 == keys.size()) ? bucket_width : 0;
  if (packed && j == 0) {
    c.type1 = c.type;
    c.type = kPackedKey;
    c.all_valid = 1;
    c.validity = nullptr;
    c.data2 = staged[keys[1]].dev.data;
    c.type2 = staged[keys[1]].dev.type;
    c.bucket = bucket_width;
  }
  return c;
}

namespace {
// Smallest and largest value of an integer column (valid rows), as
// order-preserving encodings: out[0] = min, out[1] = max.
__global__ void int_range_kernel(DevCol c, uint64_t n, unsigned long long* out) {
  unsigned long long mn = ~0ull, mx = 0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    if (!col_valid(c, r)) continue;
    const unsigned long long e = enc_i64(int_value(c, r));
    mn = e < mn ? e : mn;
    mx = e > mx ? e : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  __shared__ unsigned long long smn[32], smx[32];
  const unsigned warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    smn[warp] = mn;
    smx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned w = 1; w < nwarps; ++w) {
      mn = min(mn, smn[w]);
      mx = max(mx, smx[w]);
    }
    atomicMin(out + 0, mn);
    atomicMax(out + 1, mx);
  }
}

// Packed window rows -> composite rows: every occupied single-key row (and
// the key-0 side row) is decoded into (partition key, bucket start) key words
// and inserted into the new composite table with its fields.
__global__ void unpack_kernel(const AggK P, const uint64_t* __restrict__ old, uint64_t old_cap, int old_w,
                              int64_t width, int32_t key_type, int32_t time_type) {
  unsigned long long inserted = 0;
  const int fo = 2 + P.nkeys;
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < old_cap + 2;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t* src = old + s * old_w;
    uint64_t k;
    if (s < old_cap) {
      k = src[0];
      if (k == 0) continue;
    } else {
      if (src[1] == 0) continue;  // side rows: occupied when their row count is not zero
      if (s == old_cap + 1) {     // a NULL key cannot be packed
        atomicOr(P.err, kDevBadInput);
        continue;
      }
      k = 0;
    }
    uint64_t words[kMaxKeys] = {};
    const int32_t a = static_cast<int32_t>(static_cast<uint32_t>(k >> 32));
    words[0] = key_type == kI32 ? static_cast<uint64_t>(static_cast<uint32_t>(a))
                                : static_cast<uint64_t>(static_cast<int64_t>(a));
    const int64_t b = static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(k))) * width;
    words[1] = time_type == kI32 ? static_cast<uint64_t>(static_cast<uint32_t>(static_cast<int32_t>(b)))
                                 : static_cast<uint64_t>(b);
    uint64_t* dst = global_rowN(P, words, 0, row_hashN(P, words, 0), inserted);
    if (!dst) {
      atomicOr(P.err, kDevSpillOverflow);
      continue;
    }
    for (int f = 0; f < P.nfields; ++f) dst[fo + f] = src[1 + f];
  }
  for (int o = 16; o > 0; o >>= 1) inserted += __shfl_down_sync(0xffffffffu, inserted, o);
  if ((threadIdx.x & 31) == 0 && inserted) atomicAdd(P.counters + 2, inserted);
}
}  // namespace

// The batch can keep (or start) the packed key: both key columns without
// NULLs, the key's values (an I64/TS key) and every bucket index of the time
// column within int32.
bool AggState::can_pack(const std::vector<StagedCol>& staged, uint64_t len) {
  if (!packable || staged.empty()) return false;
  const DevCol& a = staged[keys[0]].dev;
  const DevCol& t = staged[keys[1]].dev;
  if (!a.all_valid || !t.all_valid) return false;
  if (len == 0) return true;
  const bool wide_key = a.type != kI32;
  DevBuf mm(32, ctx->stream);
  const unsigned long long init[4] = {~0ull, 0ull, ~0ull, 0ull};
  QEG_CUDA(cudaMemcpyAsync(mm.get(), init, 32, cudaMemcpyHostToDevice, ctx->stream));
  int_range_kernel<<<grid_for(ctx, len, 256, 4), 256, 0, ctx->stream>>>(t, len, mm.get<unsigned long long>());
  ctx->launches++;
  if (wide_key) {
    int_range_kernel<<<grid_for(ctx, len, 256, 4), 256, 0, ctx->stream>>>(a, len, mm.get<unsigned long long>() + 2);
    ctx->launches++;
  }
  QEG_CUDA(cudaGetLastError());
  unsigned long long r[4];
  QEG_CUDA(cudaMemcpyAsync(r, mm.get(), 32, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (wide_key && (dec_i64(r[2]) < INT32_MIN || dec_i64(r[3]) > INT32_MAX)) return false;
  const int64_t qmin = dec_i64(r[0]) / bucket_width, qmax = dec_i64(r[1]) / bucket_width;
  if (!table.get()) {
    pack_qmin = qmin;
    pack_qmax = qmax;
  }
  return qmin >= INT32_MIN && qmax <= INT32_MAX;
}

// Converts the packed single-key table into composite rows (same capacity),
// after which the window runs as an ordinary composite-key GROUP BY.
void AggState::unpack() {
  DevBuf old;
  old.swap(table);
  const uint64_t old_cap = cap;
  const int old_w = row_words;
  packed = false;
  mode = 2;
  row_words = 2 + static_cast<int>(keys.size()) + nfields;
  strategy = QEG_AGG_GLOBAL;
  smem_slots = 0;
  nhot = 0;
  alloc_table(old_cap);
  part_cap = static_cast<uint64_t>(ctx->sms) * 32 * 2 + 64;
  spill_parts.alloc(part_cap * row_words * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(counters.get<uint8_t>() + 16, 0, 8, ctx->stream));
  AggK P = kparams_base();
  const unsigned g = grid_for(ctx, old_cap + 2, 256, 8);
  unpack_kernel<<<g, 256, 0, ctx->stream>>>(P, old.get<uint64_t>(), old_cap, old_w, bucket_width, types[keys[0]],
                                            types[keys[1]]);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  uint64_t c[3];
  read_counters(c);
  check_device_error(ctx);
  inserted = c[2];
}

AggK AggState::kparams(const std::vector<StagedCol>& staged, const uint32_t* sel, uint64_t nrows,
                       uint64_t len) const {
  AggK P{};
  P.nkeys = static_cast<int>(keys.size());
  for (size_t j = 0; j < keys.size(); ++j) P.key[j] = key_col(staged, j);
  P.nvals = static_cast<int>(val_cols.size());
  for (size_t c = 0; c < val_cols.size(); ++c) {
    P.val[c] = staged[val_cols[c]].dev;
    P.cfirst[c] = static_cast<uint8_t>(cfirst[c]);
    P.cnf[c] = static_cast<uint8_t>(cnf[c]);
  }
  P.nfields = nfields;
  for (int f = 0; f < nfields; ++f) P.fkind[f] = fkind[f];
  set_field_columns(P);
  P.row_words = row_words;
  P.table = table.get<uint64_t>();
  P.cap = cap;
  P.sel = sel;
  P.nrows = nrows;
  P.len = len;
  P.smem_slots = smem_slots;
  P.smem_insert = smem_insert;
  // Private-table slots a lookup probes before it takes the global table
  // (QEG_AGG_SMEM_PROBE overrides).
  {
    static const int probe = [] {
      const char* e = std::getenv("QEG_AGG_SMEM_PROBE");
      return e ? std::max(1, std::min(64, std::atoi(e))) : 8;
    }();
    // The partitioned strategy's read-only private table: exact membership
    // (the sizing pass counts exactly the rows that miss it).
    P.smem_probe = (strategy == QEG_AGG_PARTITIONED && !smem_insert) ? std::max(1, smem_slots) : probe;
  }
  P.hot = hot_keys_dev.get<uint64_t>();
  P.nhot = nhot;
  P.warp_hot = warp_hot();
  P.probe_limit = probe_limit;
  P.spill_rows = spill_rows.get<uint32_t>();
  P.spill_cap = spill_cap;
  P.spill_parts = spill_parts.get<uint64_t>();
  P.part_cap = part_cap;
  P.counters = counters.get<unsigned long long>();
  if (mode == 1) {
    // Raise the table-full signal at 85% occupancy (counting the keys already in).
    const uint64_t at = static_cast<uint64_t>(0.85 * static_cast<double>(cap));
    P.full_flag = reinterpret_cast<uint32_t*>(P.counters + 4);
    P.full_at = at > inserted ? at - inserted : 1;
  }
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());
  return P;
}

uint32_t AggState::field_spec(const AggK& P) const {
  // The launch's field set, NULL counts of columns without NULLs skipped.
  const int n = nfields - 1;
  if (n > 7) return kGenericSpec;
  uint32_t spec = static_cast<uint32_t>(n);
  for (int i = 1; i <= n; ++i) {
    const int col = P.fcol[i];
    if (col > 1) return kGenericSpec;
    int kind = fkind[i];
    if (kind == F_NULLS && P.val[col].all_valid) kind = 0;
    spec |= spec_field(i, kind, col);
  }
  return spec;
}

void AggState::set_field_columns(AggK& P) const {
  for (size_t c = 0; c < cfirst.size(); ++c)
    for (int k = 0; k < cnf[c]; ++k) P.fcol[cfirst[c] + k] = static_cast<uint8_t>(c);
}

// 1024-thread CTAs for the single-key private-table strategy (one CTA per SM
// with a 2048-slot table: measured 1.28x faster than 512 threads on a 512M-row
// Zipf(1.1) GROUP BY), 512 otherwise.
int AggState::block_threads() const {
  if (cfg.block_threads > 0) return cfg.block_threads;
  return (mode == 1 && (strategy == QEG_AGG_SMEM || strategy == QEG_AGG_PARTITIONED)) ? 1024 : 512;
}

int AggState::warp_hot() const {
  if (mode != 1 || nhot <= 0 || smem_slots <= 0) return 0;
  // Up to 32 keys, within 32 KB of warp-private rows.
  const int fit = 32768 / ((block_threads() / 32) * (row_words | 1) * 8);
  return std::max(0, std::min({32, nhot, fit}));
}

void AggState::alloc_table(uint64_t new_cap) {
  cap = std::max<uint64_t>(new_cap, 1024);
  const uint64_t rows = (mode == 1) ? cap + 2 : (mode == 0 ? 1 : cap);
  table.alloc(rows * row_words * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(table.get(), 0, rows * row_words * 8, ctx->stream));
}

size_t AggState::smem_bytes(int block) const {
  const int srows = mode == 0 ? 1 : (smem_slots > 0 ? smem_slots + 2 : 0);
  const int wh = mode == 0 ? 1 : warp_hot();
  size_t b = (static_cast<size_t>(srows) + static_cast<size_t>(block / 32) * wh) * (row_words | 1) * 8;
  if (mode == 1 && wh > 0) b += ((srows + 7) & ~7) + 2 * wh;  // slot ranks + rank slots
  return b;
}

void AggState::launch_private(const AggK& P, uint64_t nrows) {
  void (*kern)(AggK) = nullptr;
  const int nv = static_cast<int>(val_cols.size());
  const uint32_t spec = field_spec(P);
  if (spec == kSpecIntF64) kern = agg2_private_kernel<2, kSpecIntF64>;
  else if (spec == kSpecIntF64Nulls) kern = agg2_private_kernel<2, kSpecIntF64Nulls>;
  else if (spec == kSpecF64) kern = agg2_private_kernel<1, kSpecF64>;
  else if (spec == kSpecF64Nulls) kern = agg2_private_kernel<1, kSpecF64Nulls>;
  else if (spec == kSpecCount) kern = agg2_private_kernel<1, kSpecCount>;
  else if (spec == kSpecIntSumF64Stats) kern = agg2_private_kernel<2, kSpecIntSumF64Stats>;
  else if (nv <= 1) kern = agg2_private_kernel<1, kGenericSpec>;
  else if (nv <= 2) kern = agg2_private_kernel<2, kGenericSpec>;
  else if (nv <= 4) kern = agg2_private_kernel<4, kGenericSpec>;
  else kern = agg2_private_kernel<8, kGenericSpec>;
  const int block = 512;
  const size_t sb = static_cast<size_t>(smem_slots) * (row_words | 1) * 8;
  const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), block, sb);
  require(per_sm > 0, "aggregate kernel does not fit on an SM with this configuration");
  // Each CTA walks one contiguous range; a few thousand rows at least.
  uint64_t grid = std::min<uint64_t>((nrows + 4095) / 4096, static_cast<uint64_t>(ctx->sms) * per_sm);
  if (grid == 0) grid = 1;
  kern<<<(unsigned)grid, block, sb, ctx->stream>>>(P);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
}

void AggState::launch(const AggK& P, uint64_t nrows) {
  if (mode == 2 && strategy == QEG_AGG_SMEM) {
    launch_private(P, nrows);
    return;
  }
  const int block = block_threads();
  const size_t sb = smem_bytes(block);
  if (mode == 1)  // running insert count and table-full flag
    QEG_CUDA(cudaMemsetAsync(counters.get<uint8_t>() + 24, 0, 16, ctx->stream));
  // Kernel variant: the mode and the number of value columns rounded up to 1,
  // 2, 4 or 8 (loops over value columns are unrolled to that count).
  void (*kern)(AggK) = nullptr;
  const int nv = static_cast<int>(val_cols.size());
#define QEG_AGG_VARIANT(M)                                       \
  (nv <= 1   ? agg_kernel<M, 1, kGenericSpec>                     \
   : nv <= 2 ? agg_kernel<M, 2, kGenericSpec>                     \
   : nv <= 4 ? agg_kernel<M, 4, kGenericSpec>                     \
             : agg_kernel<M, 8, kGenericSpec>)
#define QEG_AGG_SPEC(M)                                                       \
  (spec == kSpecIntF64        ? agg_kernel<M, 2, kSpecIntF64>                 \
   : spec == kSpecIntF64Nulls ? agg_kernel<M, 2, kSpecIntF64Nulls>            \
   : spec == kSpecF64         ? agg_kernel<M, 1, kSpecF64>                    \
   : spec == kSpecF64Nulls    ? agg_kernel<M, 1, kSpecF64Nulls>               \
   : spec == kSpecCount       ? agg_kernel<M, 1, kSpecCount>                  \
   : spec == kSpecIntSumF64Stats ? agg_kernel<M, 2, kSpecIntSumF64Stats>      \
                              : nullptr)
  const uint32_t spec = field_spec(P);
  if (mode == 0) kern = QEG_AGG_SPEC(0);
  else if (mode == 1) kern = QEG_AGG_SPEC(1);
  else kern = QEG_AGG_SPEC(2);
  if (kern == nullptr) {
    if (mode == 0) kern = QEG_AGG_VARIANT(0);
    else if (mode == 1) kern = QEG_AGG_VARIANT(1);
    else kern = QEG_AGG_VARIANT(2);
  }
#undef QEG_AGG_SPEC
#undef QEG_AGG_VARIANT
  const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), block, sb);
  require(per_sm > 0, "aggregate kernel does not fit on an SM with this configuration");
  // Each CTA should aggregate a few thousand rows at least, so clearing and
  // flushing its private table (which touches occupied rows only) stays small.
  const uint64_t min_rows_per_cta = 4096;
  uint64_t want = (nrows + min_rows_per_cta - 1) / min_rows_per_cta;
  uint64_t grid = std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * per_sm);
  if (grid == 0) grid = 1;
  kern<<<(unsigned)grid, block, sb, ctx->stream>>>(P);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
}

void AggState::read_counters(uint64_t out[3]) {
  QEG_CUDA(cudaMemcpyAsync(out, counters.get(), 24, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
}

void AggState::grow(uint64_t new_cap) {
  DevBuf old;
  old.swap(table);
  const uint64_t old_cap = cap;
  alloc_table(new_cap);
  QEG_CUDA(cudaMemsetAsync(counters.get<uint8_t>() + 16, 0, 8, ctx->stream));
  std::vector<StagedCol> none;
  AggK P = kparams_base();
  const uint64_t n = (mode == 1) ? old_cap + 2 : old_cap;
  const unsigned g = grid_for(ctx, n, 256, 8);
  if (mode == 1) rehash_kernel<1><<<g, 256, 0, ctx->stream>>>(P, old.get<uint64_t>(), old_cap);
  else rehash_kernel<2><<<g, 256, 0, ctx->stream>>>(P, old.get<uint64_t>(), old_cap);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  ++resizes;
}

AggK AggState::kparams_base() const {
  std::vector<StagedCol> dummy;
  AggK P{};
  P.nkeys = static_cast<int>(keys.size());
  P.nvals = static_cast<int>(val_cols.size());
  for (size_t c = 0; c < val_cols.size(); ++c) {
    P.cfirst[c] = static_cast<uint8_t>(cfirst[c]);
    P.cnf[c] = static_cast<uint8_t>(cnf[c]);
  }
  P.nfields = nfields;
  for (int f = 0; f < nfields; ++f) P.fkind[f] = fkind[f];
  set_field_columns(P);
  P.row_words = row_words;
  P.table = table.get<uint64_t>();
  P.cap = cap;
  P.probe_limit = probe_limit;
  P.counters = counters.get<unsigned long long>();
  P.err = static_cast<uint32_t*>(ctx->dev_err.get());
  return P;
}

void AggState::consume(const qeg_column* cols, int ncols, const uint32_t* sel, uint64_t sel_len) {
  require(!finished, "consume() after finish()");
  require(ncols == static_cast<int>(types.size()), "batch column count does not match the schema");
  require(cols != nullptr, "cols is NULL");
  const uint64_t len = cols[0].len;
  for (int c = 0; c < ncols; ++c) {
    require(cols[c].type == types[c], "batch column type does not match the schema");
    require(cols[c].len == len, "batch columns differ in length");
    require(cols[c].all_valid || cols[c].validity != nullptr,
            "column with all_valid=0 must carry a validity bitmap");
  }
  const uint64_t nrows = sel ? sel_len : len;
  require(len <= 0xffffffffull, "a batch holds at most 2^32-1 rows");
  std::vector<StagedCol> staged(ncols);
  for (uint32_t k : keys) stage_column(ctx, cols[k], staged[k]);
  for (uint32_t v : val_cols) stage_column(ctx, cols[v], staged[v]);
  DevBuf selbuf;
  const uint32_t* dsel = nullptr;
  stage_sel(ctx, sel, sel_len, selbuf, &dsel);
  if (!table.get()) first_consume(staged, nrows, len, dsel);
  else if (packed && !can_pack(staged, len)) unpack();
  if (nrows > spill_cap) {  // a later, larger batch: the spill list must hold all of it
    spill_cap = nrows;
    spill_rows.alloc(spill_cap * 4, ctx->stream);
  }
  rows_seen += nrows;
  if (nrows == 0) return;

  if (strategy == QEG_AGG_PARTITIONED) {
    if (part_eligible(staged)) {
      consume_partitioned(staged, nrows, len, dsel);
      return;
    }
    // A batch the partitioned passes cannot take (NULL values): the groups so
    // far join the global table and the rest runs the private-table path.
    merge_tails();
    strategy = QEG_AGG_SMEM;
  }
  AggK P = kparams(staged, dsel, nrows, len);
  launch(P, nrows);
  settle(staged, len);
}

// After a pass: while rows were spilled (their key found no slot within the
// probe limit) or private-table rows could not be flushed, grow the global
// table and replay them.
void AggState::settle(const std::vector<StagedCol>& staged, uint64_t len) {
  uint64_t c[3];
  read_words_and_error(ctx, counters.get(), 3, c);  // one synchronisation
  inserted = c[2];
  uint64_t nspill = c[0], nparts = c[1];
  int rounds = 0;
  while (nspill > 0 || nparts > 0) {
    require(++rounds < 64, "aggregate table failed to converge after 64 resize rounds");
    // Copy the spill lists out of the way, grow the table, then replay.
    DevBuf rows_copy(std::max<uint64_t>(nspill, 1) * 4, ctx->stream), parts_copy(std::max<uint64_t>(nparts, 1) * row_words * 8, ctx->stream);
    if (nspill) QEG_CUDA(cudaMemcpyAsync(rows_copy.get(), spill_rows.get(), nspill * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (nparts) QEG_CUDA(cudaMemcpyAsync(parts_copy.get(), spill_parts.get(), nparts * row_words * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    const uint64_t want = std::max<uint64_t>(cap * 2, next_pow2(2 * (inserted + nparts + nspill / 4)));
    grow(want);
    QEG_CUDA(cudaMemsetAsync(counters.get(), 0, 16, ctx->stream));
    if (nparts) {
      AggK Q = kparams_base();
      if (mode == 2)
        merge_parts_kernel<2><<<grid_for(ctx, nparts, 256, 8), 256, 0, ctx->stream>>>(Q, parts_copy.get<uint64_t>(),
                                                                                      nparts);
      else
        merge_parts_kernel<1><<<grid_for(ctx, nparts, 256, 8), 256, 0, ctx->stream>>>(Q, parts_copy.get<uint64_t>(),
                                                                                      nparts);
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
    }
    if (nspill) {
      AggK Q = kparams(staged, rows_copy.get<uint32_t>(), nspill, len);
      launch(Q, nspill);
    }
    read_words_and_error(ctx, counters.get(), 3, c);
    inserted = c[2];
    nspill = c[0];
    nparts = c[1];
  }
}

void AggState::first_consume(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len,
                             const uint32_t* dsel) {
  // A window with one I32 partition key starts packed when the batch allows.
  if (packable && can_pack(staged, len)) {
    packed = true;
    mode = 1;
    row_words = 1 + nfields;
  }
  // Sizing. QEG_SIZE_FIXED: the configured (or default) first capacity, grown on
  // overflow. QEG_SIZE_LEARNED: the estimator's group count (see qeg_estimate),
  // falling back to the row count bound when no estimate is available.
  uint64_t want;
  est_groups = 0;
  if (mode == 0) {
    want = 1;
  } else if (cfg.expected_groups > 0) {
    // The sketch still runs for its skew estimate (the private-table strategy
    // needs the heavy-hitter share) and, with hot_keys > 0, the heavy hitters.
    if (mode == 1 && (cfg.hot_keys > 0 || nrows >= kSketchMinRows)) estimate_groups(staged, nrows, len, dsel);
    want = static_cast<uint64_t>(static_cast<double>(cfg.expected_groups) / kTargetLoad) + 64;
    est_groups = static_cast<double>(cfg.expected_groups);
  } else if (cfg.sizing == QEG_SIZE_FIXED) {
    want = cfg.initial_capacity ? cfg.initial_capacity : (1ull << 20);
  } else if (nrows < kSketchMinRows) {
    // Too few rows for the sketch to pay for its round trip: the row count
    // bounds the group count, capped at the fixed default.
    want = std::min<uint64_t>(static_cast<uint64_t>(static_cast<double>(nrows) / kTargetLoad) + 64, 1ull << 20);
  } else {
    est_groups = estimate_groups(staged, nrows, len, dsel);
    // Head-room over the estimate keeps the probe short if it is low; an
    // estimate that is far too low is caught by overflow -> grow -> replay.
    want = static_cast<uint64_t>(std::max(kEstimateHeadroom * est_groups / kTargetLoad, 1024.0));
  }
  // Partitioned strategy: asked for, or chosen when the estimate puts the
  // global table far beyond L2 (every row would be a random DRAM round trip
  // there) and the key column has no heavy head. With a heavy head the
  // CTA-private tables absorb most rows and the rest reach the global table:
  // on GB300, 512M Zipf(1.1) rows over 64M keys take 28.0 ms that way against
  // 31.3 ms partitioned. Its global table only takes the private tables'
  // flushes, so it starts small.
  bool go_part = false;
  if (mode == 1 && part_eligible(staged)) {
    // Asked for: partitioned unless the estimate exceeds what its 2^15
    // second-pass tables hold (every partition would overflow into the global
    // table one by one: 2.6 s for 512M rows over 64M uniform keys, against
    // 131 ms through the global table, which it then takes).
    if (cfg.strategy == QEG_AGG_PARTITIONED)
      go_part = !(est_groups > kPartMaxFill * part_table_slots() * static_cast<double>(1u << kPartMaxBits));
    else if (cfg.strategy == QEG_AGG_AUTO && nrows >= kPartMinRows && est_groups > 0 &&
             hot_share < kPartMaxHotShare &&
             est_groups / kTargetLoad * row_words * 8.0 >= static_cast<double>(kPartMinTableBytes) &&
             est_groups <= kPartMaxFill * part_table_slots() * static_cast<double>(1u << kPartMaxBits))
      go_part = true;  // (more groups than 2^15 second-pass tables hold: the global table)
  }
  if (go_part) want = next_pow2(2ull * ctx->sms * (2048 + 2));
  alloc_table(want);
  counters.alloc(64, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(counters.get(), 0, 64, ctx->stream));
  // The spill list holds every row of a batch and the partial-row list every
  // private-table slot of every resident CTA, so neither can overflow.
  spill_cap = std::max<uint64_t>(1u << 16, nrows);
  spill_rows.alloc(spill_cap * 4, ctx->stream);

  // Strategy.
  strategy = go_part ? QEG_AGG_SMEM : (cfg.strategy == QEG_AGG_PARTITIONED ? QEG_AGG_AUTO : cfg.strategy);
  // Composite keys: CTA-private tables with periodic flushes when asked for,
  // the global table alone otherwise. (On the 200M-trade (sym, minute) window
  // the private tables measured slower, 39.3 vs 35.3 ms: the ~10k live groups
  // of a minute do not fit a CTA's table, while they do fit L2.)
  if (mode == 2) strategy = cfg.strategy == QEG_AGG_SMEM ? QEG_AGG_SMEM : QEG_AGG_GLOBAL;
  if (mode == 0) strategy = QEG_AGG_SMEM;
  // Leave room for the warp-private rows (<= 32 KB) and the slot ranks.
  const int max_slots =
      static_cast<int>(std::min<size_t>(8192, ((ctx->smem_optin - 32768) / ((row_words | 1) * 8 + 1)) - 2));
  int slots = 1;
  while (slots * 2 <= max_slots) slots *= 2;
  if (strategy == QEG_AGG_AUTO) {
    // Private tables pay off when a CTA sees each key many times: few groups
    // (all fit) or a heavy head of the key distribution.
    strategy = (est_groups > 0 && est_groups > 64.0 * slots && hot_share < 0.3) ? QEG_AGG_GLOBAL : QEG_AGG_SMEM;
  }
  nhot = 0;
  if (strategy == QEG_AGG_SMEM && mode == 1) {
    // First-come private tables of 2048 slots by default: on a heavy head the
    // hot keys arrive first and keep their slots. Preloading the sketch's
    // heavy hitters into a read-only table (hot_keys > 0) is kept as an
    // option; measured on GB300 it is slower than the first-come table
    // (34.1 vs 29.9 ms on 512M Zipf(1.1) rows with 1024-thread CTAs).
    // The partitioned strategy preloads the heavy hitters (when the sketch
    // found any) into a read-only 2048-slot table: which rows reach the pool
    // must not depend on the order rows arrive in, so a sizing pass can count
    // them.
    const bool preload = !heavy_candidates.empty() && (go_part || (cfg.hot_keys > 0 && est_groups > 1024));
    smem_slots = cfg.smem_slots > 0 ? static_cast<int>(next_pow2(cfg.smem_slots))
                                    : ((preload && !go_part) ? 1024 : 2048);
    smem_slots = std::min(smem_slots, slots);
    smem_insert = go_part ? 0 : 1;
    if (preload) {
      const int want_hot = cfg.hot_keys > 0 ? cfg.hot_keys : smem_slots / 2;
      nhot = static_cast<int>(std::min<size_t>(heavy_candidates.size(), std::min(want_hot, smem_slots / 2)));
      hot_keys_dev.alloc(std::max(nhot, 1) * 8, ctx->stream);
      QEG_CUDA(cudaMemcpyAsync(hot_keys_dev.get(), heavy_candidates.data(), nhot * 8, cudaMemcpyHostToDevice,
                               ctx->stream));
      QEG_CUDA(cudaStreamSynchronize(ctx->stream));
      smem_insert = 0;
    }
  } else if (strategy == QEG_AGG_SMEM && mode == 2) {
    // Two 512-thread CTAs per SM, each with its table.
    const size_t row_bytes = static_cast<size_t>(row_words | 1) * 8;
    int fit = 1;
    while (static_cast<size_t>(fit) * 2 * row_bytes <= ctx->smem_optin / 2 - 2048) fit *= 2;
    smem_slots = cfg.smem_slots > 0 ? static_cast<int>(next_pow2(cfg.smem_slots)) : 1024;
    smem_slots = std::max(64, std::min(smem_slots, fit));
    smem_insert = 1;
  } else {
    smem_slots = 0;
  }
  part_cap = static_cast<uint64_t>(ctx->sms) * 32 * (smem_slots + 2) + 64;
  spill_parts.alloc(part_cap * row_words * 8, ctx->stream);
  if (go_part && smem_slots > 0) setup_partitioned(nrows);
}

bool AggState::part_eligible(const std::vector<StagedCol>& staged) const {
  if (mode != 1 || packed || packable || bucket_width != 0 || staged.size() != types.size()) return false;
  for (uint32_t v : val_cols) {
    if (v == keys[0]) return false;  // a key column that is also aggregated keeps its raw values
    if (!staged[v].dev.all_valid) return false;
  }
  return true;
}

// Partition count and second-pass table size: the largest power-of-two table
// of shared memory rows one CTA can hold (at most 8192 slots), and enough
// partitions that each expects about 45% of that many groups.
int AggState::part_table_slots() const {
  const size_t rb = static_cast<size_t>(row_words | 1) * 8;
  int slots = 64;
  while (slots < 8192 && static_cast<size_t>(slots) * 2 * rb <= ctx->smem_optin - 4096) slots *= 2;
  return slots;
}

void AggState::setup_partitioned(uint64_t nrows) {
  pb_slots = part_table_slots();
  // Without an estimate the row count bounds the group count.
  const double g = est_groups > 0 ? est_groups : std::max<double>(1.0, static_cast<double>(nrows));
  int bits = static_cast<int>(std::ceil(std::log2(std::max(2.0, g / (0.45 * pb_slots)))));
  if (const char* e = std::getenv("QEG_AGG_PART_BITS")) bits = std::atoi(e);
  // At most 2^15 partitions: the sizing pass keeps a 32-bit counter per
  // partition in shared memory.
  part_bits = std::max(1, std::min(bits, kPartMaxBits));
  strategy = QEG_AGG_PARTITIONED;
  // The heavy hitters' perfect hash (ranks = positions in the candidate list).
  std::vector<uint64_t> words;
  hot_phf_build(heavy_candidates.data(), nhot, &phf_lgT, &phf_lgB, words);
  phf_words = static_cast<int>(words.size());
  phf_dev.alloc(words.size() * 8, ctx->stream);
  QEG_CUDA(cudaMemcpyAsync(phf_dev.get(), words.data(), words.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
}

// Builds the perfect hash of the first n candidate key words (rank = index;
// key word 0, which has a row of its own, and repeats are left out) by hash
// and displace: 2^lgT slots for at least twice the keys, buckets of about four
// keys by the hash's top bits, and for each bucket, largest first, the first
// displacement that puts all its keys in free slots. Layout of `words`: slot
// keys, then u16 slot ranks, then u16 bucket displacements.
void hot_phf_build(const uint64_t* keys, int n, int* lgT_out, int* lgB_out, std::vector<uint64_t>& words) {
  std::vector<std::pair<uint64_t, int>> ks;
  {
    std::unordered_map<uint64_t, int> seen;
    for (int i = 0; i < n; ++i)
      if (keys[i] != 0 && seen.emplace(keys[i], i).second) ks.emplace_back(keys[i], i);
  }
  int lgT = 6;
  while ((size_t{1} << lgT) < 2 * ks.size()) ++lgT;
  for (;; ++lgT) {
    require(lgT <= 16, "heavy-hitter perfect hash could not be built");
    const int lgB = lgT - 3;
    const size_t T = size_t{1} << lgT, B = size_t{1} << lgB;
    std::vector<std::vector<int>> buckets(B);
    std::vector<uint64_t> hs(ks.size());
    for (size_t i = 0; i < ks.size(); ++i) {
      hs[i] = hot_phf_hash(ks[i].first);
      buckets[hs[i] >> (64 - lgB)].push_back(static_cast<int>(i));
    }
    std::vector<uint32_t> order(B);
    for (size_t b = 0; b < B; ++b) order[b] = static_cast<uint32_t>(b);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return buckets[a].size() > buckets[b].size(); });
    std::vector<uint64_t> skey(T, 0);
    std::vector<uint16_t> srank(T, 0), disp(B, 0);
    bool ok = true;
    for (uint32_t b : order) {
      const auto& bk = buckets[b];
      if (bk.empty()) break;
      bool placed = false;
      for (uint32_t d = 0; d < 65536 && !placed; ++d) {
        std::vector<uint32_t> slots;
        bool free_all = true;
        for (int i : bk) {
          const uint32_t sl = hot_phf_slot(hs[i], d, lgT);
          if (skey[sl] != 0 || std::find(slots.begin(), slots.end(), sl) != slots.end()) {
            free_all = false;
            break;
          }
          slots.push_back(sl);
        }
        if (!free_all) continue;
        for (size_t j = 0; j < bk.size(); ++j) {
          skey[slots[j]] = ks[bk[j]].first;
          srank[slots[j]] = static_cast<uint16_t>(ks[bk[j]].second);
        }
        disp[b] = static_cast<uint16_t>(d);
        placed = true;
      }
      if (!placed) {
        ok = false;
        break;
      }
    }
    if (!ok) continue;
    words.assign(T + (T * 2 + B * 2 + 7) / 8, 0);
    std::memcpy(words.data(), skey.data(), T * 8);
    std::memcpy(reinterpret_cast<uint8_t*>(words.data() + T), srank.data(), T * 2);
    std::memcpy(reinterpret_cast<uint8_t*>(words.data() + T) + T * 2, disp.data(), B * 2);
    *lgT_out = lgT;
    *lgB_out = lgB;
    return;
  }
}

// One batch through the partitioned passes: the sizing pass counts the rows
// of every partition that will go to the pool, a scan turns the counts into
// exact regions, the first pass aggregates the heavy hitters in the private
// tables and appends every other row to its region, the second pass
// aggregates each partition in shared memory.
void AggState::consume_partitioned(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len,
                                   const uint32_t* dsel) {
  if (ntails) merge_tails();  // an earlier batch's groups join the global table
  const uint64_t np = 1ull << part_bits;
  AggK P = kparams(staged, dsel, nrows, len);
  P.part_shift = 64 - part_bits;
  PartA A{};
  A.nhot = nhot;
  A.rw = nfields | 1;
  A.lgT = phf_lgT;
  A.lgB = phf_lgB;
  A.phf = phf_dev.get<uint64_t>();
  A.phf_words = phf_words;
  const size_t hot_bytes = static_cast<size_t>(phf_words) * 8;
  if (part_hist.bytes() < np * 8) part_hist.alloc(np * 8, ctx->stream);
  if (part_off.bytes() < (np + 1) * 8) part_off.alloc((np + 1) * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(part_hist.get(), 0, np * 8, ctx->stream));
  A.hist = part_hist.get<unsigned long long>();
  {
    const size_t sb = hot_bytes + np * 4;
    constexpr int kHistRows = 8;
    const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(part_hist_kernel<kHistRows>), 1024, sb);
    require(per_sm > 0, "partition sizing kernel does not fit on an SM");
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>((nrows + 65535) / 65536, static_cast<uint64_t>(ctx->sms) * per_sm));
    part_hist_kernel<kHistRows><<<(unsigned)grid, 1024, sb, ctx->stream>>>(P, A);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  // Region starts: a prefix sum of the (at most 2^15) counts on the host.
  std::vector<uint64_t> offs(np + 1, 0);
  QEG_CUDA(cudaMemcpyAsync(offs.data() + 1, part_hist.get(), np * 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (uint64_t p = 0; p < np; ++p) offs[p + 1] += offs[p];
  const uint64_t pooled = offs[np];
  QEG_CUDA(cudaMemcpyAsync(part_off.get(), offs.data(), (np + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
  const size_t pool_bytes = std::max<uint64_t>(pooled, 1) * 8;
  if (pool_key.bytes() < pool_bytes) {
    pool_key.alloc(pool_bytes, ctx->stream);
    pool_vals.clear();
    pool_vals.resize(val_cols.size());
    for (auto& b : pool_vals) b.alloc(pool_bytes, ctx->stream);
  }
  if (part_fill.bytes() < np * 8) part_fill.alloc(np * 8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(part_fill.get(), 0, np * 8, ctx->stream));
  P.pool_key = pool_key.get<uint64_t>();
  for (size_t c = 0; c < val_cols.size(); ++c) P.pool_val[c] = pool_vals[c].get<uint64_t>();
  P.part_fill = part_fill.get<unsigned long long>();
  P.part_off = part_off.get<uint64_t>();
  {
    const uint32_t spec = field_spec(P);
    const int nv = static_cast<int>(val_cols.size());
    void (*kern)(AggK, PartA) = nullptr;
    if (spec == kSpecIntF64) kern = part_pass1_kernel<2, kSpecIntF64, part_rows<2>()>;
    else if (spec == kSpecIntF64Nulls) kern = part_pass1_kernel<2, kSpecIntF64Nulls, part_rows<2>()>;
    else if (spec == kSpecF64) kern = part_pass1_kernel<1, kSpecF64, part_rows<1>()>;
    else if (spec == kSpecF64Nulls) kern = part_pass1_kernel<1, kSpecF64Nulls, part_rows<1>()>;
    else if (spec == kSpecCount) kern = part_pass1_kernel<1, kSpecCount, part_rows<1>()>;
    else if (spec == kSpecIntSumF64Stats) kern = part_pass1_kernel<2, kSpecIntSumF64Stats, part_rows<2>()>;
    else if (nv <= 1) kern = part_pass1_kernel<1, kGenericSpec, part_rows<1>()>;
    else if (nv <= 2) kern = part_pass1_kernel<2, kGenericSpec, part_rows<2>()>;
    else if (nv <= 4) kern = part_pass1_kernel<4, kGenericSpec, part_rows<4>()>;
    else kern = part_pass1_kernel<8, kGenericSpec, part_rows<8>()>;
    const size_t sb = hot_bytes + static_cast<size_t>(nhot + 2) * A.rw * 8;
    const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), 512, sb);
    require(per_sm > 0, "partitioned first pass does not fit on an SM");
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>((nrows + 8191) / 8192, static_cast<uint64_t>(ctx->sms) * per_sm));
    kern<<<(unsigned)grid, 512, sb, ctx->stream>>>(P, A);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  settle(staged, len);
  part_second_pass();
}

// The pool as kernel columns: key words (I64) and 8-byte values (F64 for F64
// inputs, I64 for every other type), rows [first, first + n) of the pool.
static std::vector<StagedCol> pool_columns(const AggState& st, uint64_t first) {
  std::vector<StagedCol> ps(st.types.size());
  DevCol k{};
  k.type = QEG_I64;
  k.all_valid = 1;
  k.data = st.pool_key.get<uint64_t>() + first;
  ps[st.keys[0]].dev = k;
  for (size_t c = 0; c < st.val_cols.size(); ++c) {
    DevCol v{};
    v.type = st.types[st.val_cols[c]] == QEG_F64 ? QEG_F64 : QEG_I64;
    v.all_valid = 1;
    v.data = st.pool_vals[c].get<uint64_t>() + first;
    ps[st.val_cols[c]].dev = v;
  }
  return ps;
}

void AggState::part_second_pass() {
  const uint64_t np = 1ull << part_bits;
  AggK P = kparams_base();
  // The second-pass table slot comes from the partition hash bits below the
  // partition bits.
  P.part_shift = 64 - part_bits;
  for (size_t c = 0; c < val_cols.size(); ++c) {
    P.val[c].type = types[val_cols[c]] == QEG_F64 ? QEG_F64 : QEG_I64;
    P.val[c].all_valid = 1;
  }
  const uint32_t spec = field_spec(P);
  const int nv = static_cast<int>(val_cols.size());
  void (*kern)(AggK, PartB) = nullptr;
  if (spec == kSpecIntF64) kern = part_agg_kernel<2, kSpecIntF64, part_rows<2>()>;
  else if (spec == kSpecF64) kern = part_agg_kernel<1, kSpecF64, part_rows<1>()>;
  else if (spec == kSpecCount) kern = part_agg_kernel<1, kSpecCount, part_rows<1>()>;
  else if (spec == kSpecIntSumF64Stats) kern = part_agg_kernel<2, kSpecIntSumF64Stats, part_rows<2>()>;
  else if (nv <= 1) kern = part_agg_kernel<1, kGenericSpec, part_rows<1>()>;
  else if (nv <= 2) kern = part_agg_kernel<2, kGenericSpec, part_rows<2>()>;
  else if (nv <= 4) kern = part_agg_kernel<4, kGenericSpec, part_rows<4>()>;
  else kern = part_agg_kernel<8, kGenericSpec, part_rows<8>()>;
  const int block = 1024;
  const size_t sb = static_cast<size_t>(pb_slots) * (row_words | 1) * 8;
  const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), block, sb);
  require(per_sm > 0, "partitioned aggregate kernel does not fit on an SM");
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(np, static_cast<uint64_t>(ctx->sms) * per_sm));
  if (!part_counters.get()) part_counters.alloc(16, ctx->stream);
  if (part_failed.bytes() < np * 4) part_failed.alloc(np * 4, ctx->stream);
  if (tails_cap == 0) {
    tails_cap = static_cast<uint64_t>(std::max(1.25 * est_groups, 4096.0));
    tails.alloc((tails_cap + 2) * row_words * 8, ctx->stream);
  }
  PartB B{};
  B.pool_key = pool_key.get<uint64_t>();
  for (size_t c = 0; c < val_cols.size(); ++c) B.pool_val[c] = pool_vals[c].get<uint64_t>();
  B.part_off = part_off.get<uint64_t>();
  B.nparts = static_cast<uint32_t>(np);
  B.slots = pb_slots;
  B.counters = part_counters.get<unsigned long long>();
  B.failed = part_failed.get<uint32_t>();
  unsigned long long cnt[2];
  for (int round = 0;; ++round) {
    require(round < 4, "partitioned aggregate: tail buffer sizing failed");
    B.tails = tails.get<uint64_t>();
    B.tails_cap = tails_cap;
    QEG_CUDA(cudaMemsetAsync(part_counters.get(), 0, 16, ctx->stream));
    kern<<<grid, block, sb, ctx->stream>>>(P, B);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
    QEG_CUDA(cudaMemcpyAsync(cnt, part_counters.get(), 16, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (cnt[0] <= tails_cap) break;
    // More groups than the tail buffer holds: size it to the count and re-run
    // (the pass only reads the pool).
    tails_cap = cnt[0] + cnt[0] / 8 + 4096;
    tails.alloc((tails_cap + 2) * row_words * 8, ctx->stream);
  }
  ntails = cnt[0];
  // Two empty rows after the tails: the finalize pass reads a single-key
  // table's side rows there.
  QEG_CUDA(cudaMemsetAsync(tails.get<uint64_t>() + ntails * row_words, 0, 2 * row_words * 8, ctx->stream));
  const uint64_t nfailed = std::min<uint64_t>(cnt[1], np);
  if (nfailed) {
    std::vector<uint32_t> ids(nfailed);
    QEG_CUDA(cudaMemcpyAsync(ids.data(), part_failed.get(), nfailed * 4, cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<uint64_t> offs(np + 1);
    QEG_CUDA(cudaMemcpyAsync(offs.data(), part_off.get(), (np + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (uint32_t p : ids) {
      const uint64_t n = offs[p + 1] - offs[p];
      if (n == 0) continue;
      const std::vector<StagedCol> ps = pool_columns(*this, offs[p]);
      if (n > spill_cap) {
        spill_cap = n;
        spill_rows.alloc(spill_cap * 4, ctx->stream);
      }
      AggK Q = kparams(ps, nullptr, n, n);
      launch(Q, n);
      settle(ps, n);
    }
  }
}

// Moves the tail rows into the global table (grown to hold them).
void AggState::merge_tails() {
  if (ntails == 0) return;
  const uint64_t need = next_pow2(2 * (inserted + ntails));
  if (cap < need) grow(need);
  AggK Q = kparams_base();
  merge_parts_kernel<1><<<grid_for(ctx, ntails, 256, 8), 256, 0, ctx->stream>>>(Q, tails.get<uint64_t>(), ntails);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  uint64_t c[3];
  read_counters(c);
  check_device_error(ctx);
  inserted = c[2];
  ntails = 0;
}

void AggState::finish(uint64_t* nrows_out) {
  if (finished) {
    *nrows_out = nout;
    return;
  }
  if (!table.get()) {
    // Nothing consumed: set up an empty table so the global case emits its row.
    std::vector<StagedCol> none;
    first_consume(none, 0, 0, nullptr);
  }
  const uint64_t out_cap = (mode == 0) ? 1 : std::max<uint64_t>(inserted + 2 + ntails, 1);
  const int ncolsout = static_cast<int>(keys.size() + aggs.size());
  out_vals.clear();
  out_valid.clear();
  out_vals.resize(ncolsout);
  out_valid.resize(ncolsout);
  FinK F{};
  F.naggs = static_cast<int>(aggs.size());
  for (int c = 0; c < ncolsout; ++c) {
    out_vals[c].alloc(out_cap * 8, ctx->stream);
    out_valid[c].alloc(out_cap, ctx->stream);
    F.vals[c] = out_vals[c].get();
    F.valid[c] = out_valid[c].get<uint8_t>();
    F.rtype[c] = rtypes[c];
  }
  for (size_t a = 0; a < aggs.size(); ++a) {
    F.func[a] = aggs[a].func;
    F.vfield[a] = vfield[a];
    F.nfield[a] = nfield[a];
  }
  DevBuf cnt(8, ctx->stream);
  QEG_CUDA(cudaMemsetAsync(cnt.get(), 0, 8, ctx->stream));
  F.out_count = cnt.get<unsigned long long>();
  F.out_cap = out_cap;
  F.packed_width = packed ? bucket_width : 0;
  AggK P = kparams_base();
  if (mode == 1 && ntails > 0) {
    // Partitioned strategy: the tail rows first, each merged into the global
    // table instead when its key is there too; then the global table.
    AggK T = P;
    T.table = tails.get<uint64_t>();
    T.cap = ntails;
    FinK FT = F;
    FT.merge_table = table.get<uint64_t>();
    FT.merge_cap = cap;
    finalize_kernel<1><<<grid_for(ctx, ntails + 2, 1024, 2), 1024, 0, ctx->stream>>>(T, FT);
    ctx->launches++;
    QEG_CUDA(cudaGetLastError());
  }
  const uint64_t total = (mode == 0) ? 1 : (mode == 1 ? cap + 2 : cap);
  const unsigned g = grid_for(ctx, total, 1024, 2);
  if (mode == 0) finalize_kernel<0><<<g, 1024, 0, ctx->stream>>>(P, F);
  else if (mode == 1) finalize_kernel<1><<<g, 1024, 0, ctx->stream>>>(P, F);
  else finalize_kernel<2><<<g, 1024, 0, ctx->stream>>>(P, F);
  ctx->launches++;
  QEG_CUDA(cudaGetLastError());
  unsigned long long n = 0;
  QEG_CUDA(cudaMemcpyAsync(&n, cnt.get(), 8, cudaMemcpyDeviceToHost, ctx->stream));
  QEG_CUDA(cudaStreamSynchronize(ctx->stream));
  check_device_error(ctx);
  nout = n;
  finished = true;
  *nrows_out = nout;
}

void AggState::fetch(uint64_t first, uint64_t count, const qeg_out_column* outs) {
  require(finished, "fetch() before finish()");
  require(first <= nout && count <= nout - first, "fetch range outside the result");
  require(outs != nullptr, "outs is NULL");
  for (size_t c = 0; c < out_vals.size(); ++c)
    fetch_column(ctx, out_vals[c].get(), out_valid[c].get<uint8_t>(), type_width(rtypes[c]), first, count, outs[c]);
}

}  // namespace qeg

using qeg::AggState;

struct qeg_agg {
  AggState st;
};

extern "C" {

qeg_status qeg_agg_create(qeg_ctx* ctx, const int32_t* col_types, int ncols, const uint32_t* key_cols,
                          int nkeys, const qeg_agg_spec* aggs, int naggs, const qeg_agg_config* cfg,
                          qeg_agg** out) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr && out != nullptr, "ctx/out is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    auto a = std::make_unique<qeg_agg>();
    a->st.ctx = ctx;
    if (cfg) a->st.cfg = *cfg;
    const int bt = a->st.cfg.block_threads;
    qeg::require(bt == 0 || (bt >= 32 && bt <= 1024 && bt % 32 == 0),
                 "block_threads must be 0 or a multiple of 32 in [32, 1024]");
    a->st.plan(col_types, ncols, key_cols, nkeys, aggs, naggs);
    *out = a.release();
  });
}

qeg_status qeg_window_create(qeg_ctx* ctx, const int32_t* col_types, int ncols, const uint32_t* key_cols,
                             int nkeys, uint32_t time_col, int64_t width, const qeg_agg_spec* aggs, int naggs,
                             const qeg_agg_config* cfg, qeg_agg** out) {
  return qeg::guarded(ctx, [&] {
    qeg::require(ctx != nullptr && out != nullptr, "ctx/out is NULL");
    qeg::require(ncols > 0 && col_types != nullptr, "window needs an input schema");
    qeg::require(nkeys >= 0 && (nkeys == 0 || key_cols != nullptr), "key_cols is NULL");
    qeg::require(nkeys + 1 <= qeg::kMaxKeys, "GPU window supports at most 7 partition keys");
    qeg::require(naggs >= 1 && aggs != nullptr, "Window needs >=1 aggregate");
    qeg::require(time_col < static_cast<uint32_t>(ncols), "window time column out of range");
    for (int k = 0; k < nkeys; ++k) {
      qeg::require(key_cols[k] < static_cast<uint32_t>(ncols), "window key column out of range");
      qeg::require(col_types[key_cols[k]] != QEG_STR,
                   "Window: STR partition keys are not supported (out of grammar)");
    }
    for (int a = 0; a < naggs; ++a)
      if (aggs[a].func != QEG_COUNT_STAR && aggs[a].input_col < static_cast<uint32_t>(ncols))
        qeg::require(col_types[aggs[a].input_col] != QEG_STR,
                     "Window: STR aggregate inputs are not supported (out of grammar)");
    const int32_t tt = col_types[time_col];
    qeg::require(tt == QEG_I32 || tt == QEG_I64 || tt == QEG_TS, "Window: time column must be I32/I64/TS");
    qeg::require(width > 0, "Window: tumbling width W must be > 0");
    std::vector<uint32_t> k(key_cols, key_cols + nkeys);
    k.push_back(time_col);
    QEG_CUDA(cudaSetDevice(ctx->device));
    auto a = std::make_unique<qeg_agg>();
    a->st.ctx = ctx;
    if (cfg) a->st.cfg = *cfg;
    const int bt = a->st.cfg.block_threads;
    qeg::require(bt == 0 || (bt >= 32 && bt <= 1024 && bt % 32 == 0),
                 "block_threads must be 0 or a multiple of 32 in [32, 1024]");
    a->st.plan(col_types, ncols, k.data(), nkeys + 1, aggs, naggs);
    a->st.bucket_width = width;
    const int32_t kt = nkeys == 1 ? col_types[key_cols[0]] : -1;
    a->st.packable = kt == QEG_I32 || kt == QEG_I64 || kt == QEG_TS;
    *out = a.release();
  });
}

qeg_status qeg_agg_consume(qeg_agg* agg, const qeg_column* cols, int ncols, const uint32_t* sel,
                           uint64_t sel_len) {
  qeg::NvtxRange nvtx_range("qeg_agg_consume");
  qeg_ctx* ctx = agg ? agg->st.ctx : nullptr;
  return qeg::guarded(ctx, [&] {
    qeg::require(agg != nullptr, "agg is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    agg->st.consume(cols, ncols, sel, sel_len);
  });
}

qeg_status qeg_agg_finish(qeg_agg* agg, uint64_t* num_rows) {
  qeg::NvtxRange nvtx_range("qeg_agg_finish");
  qeg_ctx* ctx = agg ? agg->st.ctx : nullptr;
  return qeg::guarded(ctx, [&] {
    qeg::require(agg != nullptr && num_rows != nullptr, "agg/num_rows is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    agg->st.finish(num_rows);
  });
}

qeg_status qeg_agg_result_types(const qeg_agg* agg, int32_t* types) {
  qeg_ctx* ctx = agg ? agg->st.ctx : nullptr;
  return qeg::guarded(ctx, [&] {
    qeg::require(agg != nullptr && types != nullptr, "agg/types is NULL");
    for (size_t c = 0; c < agg->st.rtypes.size(); ++c) types[c] = agg->st.rtypes[c];
  });
}

qeg_status qeg_agg_fetch(qeg_agg* agg, uint64_t first, uint64_t count, const qeg_out_column* outs) {
  qeg::NvtxRange nvtx_range("qeg_agg_fetch");
  qeg_ctx* ctx = agg ? agg->st.ctx : nullptr;
  return qeg::guarded(ctx, [&] {
    qeg::require(agg != nullptr, "agg is NULL");
    QEG_CUDA(cudaSetDevice(ctx->device));
    agg->st.fetch(first, count, outs);
  });
}

qeg_status qeg_agg_stats(const qeg_agg* agg, uint64_t* capacity, uint32_t* resizes, int32_t* strategy,
                         int32_t* hot_keys, double* est_groups) {
  qeg_ctx* ctx = agg ? agg->st.ctx : nullptr;
  return qeg::guarded(ctx, [&] {
    qeg::require(agg != nullptr, "agg is NULL");
    if (capacity) *capacity = agg->st.cap;
    if (resizes) *resizes = agg->st.resizes;
    if (strategy) *strategy = agg->st.strategy;
    if (hot_keys) *hot_keys = agg->st.nhot;
    if (est_groups) *est_groups = agg->st.est_groups;
  });
}

void qeg_agg_destroy(qeg_agg* agg) {
  if (!agg) return;
  cudaSetDevice(agg->st.ctx->device);
  delete agg;
}

}  // extern "C"
