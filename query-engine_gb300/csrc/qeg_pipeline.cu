// qeg_pipeline.cu -- fused filter -> inner join -> GROUP BY for a small build
// side: the plan
//   scan(probe).filter(col <op> literal)
//              .join(scan(build), {probe_key}, {build_key}, Inner)
//              .aggregate({build column}, {aggs over probe columns})
// of the reference's plan builder (plan/plan.cpp:340-404), run as one pass over
// the probe side. The reference executes it as Filter (ops/filter.cpp:28-66,
// with compact_column), HashJoin (per-row STR interning, ops/join.cpp:48-71)
// and Aggregate; here nothing is compacted or materialised:
//   * the predicate is evaluated in registers (a NULL operand drops the row,
//     as Kleene logic does for a filter);
//   * the probe key is a small dense domain (dictionary codes of a STR column,
//     or integers with a small range); the host resolves each probe key value
//     once -- through the shared by-value id space for STR -- to the list of
//     group ids of its matching build rows, so the join + grouping becomes one
//     shared-memory table lookup per row;
//   * the aggregates accumulate in warp-private shared-memory copies of the
//     (few) groups' states, merged once per block.
// Semantics are those of the reference's operators: NULL keys never join,
// a NULL group value is its own group, COUNT/SUM/AVG/MIN/MAX per
// ops/agg_internal.h:169-229.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

#include "qeg_agg.h"
#include "qeg_warpagg.cuh"

namespace qeg {

namespace {

constexpr int kPipeMaxAggs = 16;
constexpr int kPipeMaxVals = 4;
// COUNT(*), AVG/SUM(F64 column 0), SUM(integer column 1) without and with NULL
// counts (qeg_warpagg.cuh field-set codes).
constexpr uint32_t kPipeSpecAvgSum = 4u | spec_field(1, 0, 0) | spec_field(2, F_SUMF, 0) | spec_field(3, 0, 1) |
                                     spec_field(4, F_SUMI, 1);
constexpr uint32_t kPipeSpecAvgSumNulls = 4u | spec_field(1, F_NULLS, 0) | spec_field(2, F_SUMF, 0) |
                                          spec_field(3, F_NULLS, 1) | spec_field(4, F_SUMI, 1);

enum CmpOp : int32_t { kLT = 0, kLE = 1, kGT = 2, kGE = 3, kEQ = 4, kNE = 5, kNever = -1, kAlways = -2 };

struct PipeK {
  DevCol fcol;  // filter column (type -1: none)
  int32_t fop;
  double flit_f;
  int64_t flit_i;
  DevCol key;
  int64_t key_min;       // probe key value -> slot = value - key_min
  uint64_t key_domain;   // slots in the translation table
  const uint32_t* kstart;  // [key_domain]
  const uint32_t* kcount;  // [key_domain]
  // [key_domain]: the group id when the key matches exactly one build row,
  // 0x80000000 | slot when it matches several (kstart / kcount), ~0 when none.
  const uint32_t* kfirst;
  // The same as u16 group ids (0xffff: no match, 0xfffe: several) when the
  // groups number at most 65533, for the trades kernel's shared-memory copy.
  const uint16_t* kf16;
  const uint32_t* glist;   // group ids
  DevCol val[kPipeMaxVals];
  int nvals;
  uint8_t fkind[kMaxFields];
  uint8_t cfirst[kPipeMaxVals];
  uint8_t cnf[kPipeMaxVals];
  int nfields;
  int ngroups;
  int per_warp;  // 1: warp-private shared copies; 0: one shared copy per block
  int lane_reds;  // 1: every lane applies its own row with shared reductions
  uint64_t n;
  unsigned long long* state;  // [ngroups][nfields] global
};

__device__ __forceinline__ bool pass_filter(const PipeK& P, uint64_t p) {
  if (P.fcol.type < 0) return true;
  if (!col_valid(P.fcol, p)) return false;
  bool r;
  if (P.fcol.type == kF64) {
    const double v = f64_value(P.fcol, p);
    const double l = P.flit_f;
    switch (P.fop) {
      case kLT: r = v < l; break;
      case kLE: r = v <= l; break;
      case kGT: r = v > l; break;
      case kGE: r = v >= l; break;
      case kEQ: r = v == l; break;
      default: r = v != l; break;
    }
  } else {
    if (P.fop == kNever) return false;
    if (P.fop == kAlways) return true;
    const int64_t v = int_value(P.fcol, p);
    const int64_t l = P.flit_i;
    switch (P.fop) {
      case kLT: r = v < l; break;
      case kLE: r = v <= l; break;
      case kGT: r = v > l; break;
      case kGE: r = v >= l; break;
      case kEQ: r = v == l; break;
      default: r = v != l; break;
    }
  }
  return r;
}

// SPEC: the aggregate fields' set (qeg_warpagg.cuh), or kGenericSpec. The
// field-set kernels are held to 32 registers, four 512-thread CTAs per SM
// (full occupancy: 2.56 ms per 200M trades on GB300, against 2.9 ms at 39
// registers and three CTAs, and 4.0 ms at 47 registers and two).
template <uint32_t SPEC>
__global__ void __launch_bounds__(512, SPEC == kGenericSpec ? 2 : 4) pipeline_kernel(const PipeK P) {
  extern __shared__ unsigned long long sst[];
  const int warps = blockDim.x >> 5;
  const int copies = P.per_warp ? warps : 1;
  // A group's fields at an odd stride (in 8-byte words), so the same field of
  // different groups falls in different shared-memory banks.
  const int GS = P.nfields | 1;
  const int stride_g = P.ngroups * GS;
  for (int i = threadIdx.x; i < copies * stride_g; i += blockDim.x) sst[i] = 0;
  __syncthreads();
  unsigned long long* mine = sst + (P.per_warp ? (threadIdx.x >> 5) * stride_g : 0);
  const unsigned lane = threadIdx.x & 31u;
  // Warps walk the rows 32 at a time. For every (row, matching build row)
  // pair, lanes with the same group combine their rows in registers (warp peer
  // aggregation) and the group's leader applies the result: without atomics
  // to a warp-private copy, with shared atomics to the block's single copy.
  for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); base < P.n;
       base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = base + lane;
    bool ok = p < P.n && pass_filter(P, p) && col_valid(P.key, p);  // NULL keys never join
    uint32_t cnt = 0, s0 = 0;
    if (ok) {
      const uint64_t slot = static_cast<uint64_t>(int_value(P.key, p) - P.key_min);
      if (slot < P.key_domain) {
        cnt = __ldg(P.kcount + slot);
        if (cnt) s0 = __ldg(P.kstart + slot);
      }
      ok = cnt > 0;
    }
    bool vv[kPipeMaxVals];
    uint64_t vb[kPipeMaxVals];
#pragma unroll
    for (int c = 0; c < kPipeMaxVals; ++c) {
      vv[c] = false;
      vb[c] = 0;
      if (ok && c < P.nvals) {
        vv[c] = col_valid(P.val[c], p);
        if (vv[c]) vb[c] = P.val[c].type == kF64 ? static_cast<uint64_t>(__double_as_longlong(f64_value(P.val[c], p)))
                                                 : static_cast<uint64_t>(int_value(P.val[c], p));
      }
    }
    if (P.lane_reds) {
      // No peer combining: with few groups, the rows of a warp mostly fall in
      // different groups, and a shared reduction per field and row is cheaper
      // than matching and combining the lanes.
      for (uint32_t m = 0; ok && m < cnt; ++m) {
        uint64_t* f = reinterpret_cast<uint64_t*>(mine + static_cast<size_t>(__ldg(P.glist + s0 + m)) * GS);
        field_red<kRowShared>(f, F_ROWS, 1);
        if constexpr (SPEC != kGenericSpec) {
#pragma unroll
          for (int i = 1; i <= spec_n(SPEC); ++i) {
            const int kind = spec_kind(SPEC, i);
            if (kind == 0) continue;
            const int c = spec_col(SPEC, i);
            field_red<kRowShared>(f + i, kind, field_contrib(kind, vv[c], vb[c]));
          }
        } else {
          for (int c = 0; c < P.nvals; ++c)
            for (int k = 0; k < P.cnf[c]; ++k) {
              const int fi = P.cfirst[c] + k;
              field_red<kRowShared>(f + fi, P.fkind[fi], field_contrib(P.fkind[fi], vv[c], vb[c]));
            }
        }
      }
      continue;
    }
    const uint32_t rounds = __reduce_max_sync(0xffffffffu, ok ? cnt : 0u);
    for (uint32_t m = 0; m < rounds; ++m) {
      const bool act = ok && m < cnt;
      const uint32_t g = act ? __ldg(P.glist + s0 + m) : 0xffffffffu;
      const unsigned amask = __ballot_sync(0xffffffffu, act);
      const unsigned same = __match_any_sync(0xffffffffu, g);
      const unsigned peers = act ? (same & amask) : (1u << lane);
      const bool leader = act && __ffs(peers) - 1 == static_cast<int>(lane);
      const PeerPlan pp = plan_peers(peers, lane);
      unsigned long long* f = leader ? mine + static_cast<size_t>(g) * GS : nullptr;
      const int space = P.per_warp ? kRowPrivate : kRowShared;
      if constexpr (SPEC != kGenericSpec) {
        bool v8[8] = {vv[0], vv[1]};
        uint64_t b8[8] = {vb[0], vb[1]};
        spec_apply<SPEC, 2>(reinterpret_cast<uint64_t*>(f), leader, space, peers, pp, v8, b8);
      } else {
        if (leader) field_red_at(space, reinterpret_cast<uint64_t*>(f), F_ROWS, static_cast<uint64_t>(__popc(peers)));
#pragma unroll
        for (int c = 0; c < kPipeMaxVals; ++c) {
          if (c >= P.nvals) break;
          for (int k = 0; k < P.cnf[c]; ++k) {
            const int fi = P.cfirst[c] + k;
            const uint8_t kind = P.fkind[fi];
            const uint64_t x = peer_reduce(field_contrib(kind, vv[c], vb[c]), kind, pp);
            if (leader) field_red_at(space, reinterpret_cast<uint64_t*>(f + fi), kind, x);
          }
        }
      }
    }
  }
  __syncthreads();
  // Merge the shared copies into the global state (zero is every identity).
  for (int i = threadIdx.x; i < stride_g; i += blockDim.x) {
    const int f = i % GS;
    if (f >= P.nfields) continue;
    const int gi = (i / GS) * P.nfields + f;  // index into the unpadded global state
    const uint8_t kind = P.fkind[f];
    unsigned long long acc = 0;
    double accf = 0;
    for (int c = 0; c < copies; ++c) {
      const unsigned long long v = sst[c * stride_g + i];
      if (kind == F_SUMF) accf += __longlong_as_double(static_cast<long long>(v));
      else if (kind >= F_MINI) acc = max(acc, v);
      else acc += v;
    }
    if (kind == F_SUMF) {
      if (accf != 0.0) atomicAdd(reinterpret_cast<double*>(P.state + gi), accf);
    } else if (acc) {
      if (kind >= F_MINI) atomicMax(P.state + gi, acc);
      else atomicAdd(P.state + gi, acc);
    }
  }
}

// Raw word of row p of column c at its type's width (I32/STR zero-extended,
// no code map), so loads of different columns and rows never wait on each
// other; bits_int widens an integer column's word to int64.
__device__ __forceinline__ uint64_t raw_bits(const DevCol& c, uint64_t p) {
  switch (c.type) {
    case kI32:
    case kSTR: return static_cast<uint32_t>(__ldg(static_cast<const int32_t*>(c.data) + p));
    case kBOOL: return __ldg(static_cast<const uint8_t*>(c.data) + p);
    default: return static_cast<uint64_t>(__ldg(static_cast<const long long*>(c.data) + p));
  }
}
__device__ __forceinline__ int64_t bits_int(int32_t type, uint64_t b) {
  return (type == kI32 || type == kSTR) ? static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(b)))
                                        : static_cast<int64_t>(b);
}
__device__ __forceinline__ bool bit_valid(const DevCol& c, uint64_t p) {
  if (c.all_valid) return true;
  return (__ldg(c.validity + (p >> 6)) >> (p & 63)) & 1ull;
}
// The filter predicate on the filter column's raw word (a valid row).
__device__ __forceinline__ bool filter_bits(const PipeK& P, uint64_t b) {
  if (P.fcol.type == kF64) {
    const double v = __longlong_as_double(static_cast<long long>(b));
    const double l = P.flit_f;
    switch (P.fop) {
      case kLT: return v < l;
      case kLE: return v <= l;
      case kGT: return v > l;
      case kGE: return v >= l;
      case kEQ: return v == l;
      default: return v != l;
    }
  }
  if (P.fop == kNever) return false;
  if (P.fop == kAlways) return true;
  const int64_t v = bits_int(P.fcol.type, b);
  const int64_t l = P.flit_i;
  switch (P.fop) {
    case kLT: return v < l;
    case kLE: return v <= l;
    case kGT: return v > l;
    case kGE: return v >= l;
    case kEQ: return v == l;
    default: return v != l;
  }
}

// Largest CTA of the thread-private kernels (the typed trades kernel fits 320
// threads' states for 32 groups beside its translation table).
constexpr int kLanesMaxThreads = 384;

// Active fields of a field set: field 0 (the row count) and every field
// whose kind is not 0, in field order ("compact" indexes).
__host__ __device__ constexpr int spec_nactive(uint32_t spec) {
  int n = 1;
  for (int i = 1; i <= spec_n(spec); ++i)
    if (spec_kind(spec, i) != 0) ++n;
  return n;
}
// Field index of compact index c.
__host__ __device__ constexpr int spec_active_field(uint32_t spec, int c) {
  int k = 0;
  for (int i = 1; i <= spec_n(spec); ++i)
    if (spec_kind(spec, i) != 0 && ++k == c) return i;
  return 0;
}
// Compact index of field i (a field whose kind is not 0).
__host__ __device__ constexpr int spec_compact(uint32_t spec, int i) {
  int k = 0;
  for (int j = 1; j <= i; ++j)
    if (spec_kind(spec, j) != 0) ++k;
  return k;
}

// The same plan with thread-private aggregate states: every thread owns one
// copy of every group's active fields in shared memory, word
// (g * NA + c) * blockDim.x + threadIdx.x, so the lanes of a warp touch
// consecutive words whatever their groups (no bank conflicts) and a row is
// applied with plain loads and stores, no atomics and no combining across
// lanes. (On GB300, 64-bit shared-memory reductions cost 10 clocks per warp
// instruction for integers and 56 for F64 without contention, several times
// more with it; a plain read-modify-write costs 2.) Each warp takes R chunks
// of 32 consecutive rows per tile, all their loads issued before any row is
// applied. At the end the copies are reduced warp by warp and added to the
// global state. NA = the active field count (spec_nactive, or nfields for
// the generic field set).
template <uint32_t SPEC, int R, int FASTOP>
__global__ void __launch_bounds__(kLanesMaxThreads, 1) pipeline_lanes_kernel(const PipeK P, int NA) {
  extern __shared__ unsigned long long acc[];
  constexpr int NVR = SPEC == kGenericSpec ? kPipeMaxVals : 2;  // value columns a row carries
  const int T = blockDim.x;
  const int total = P.ngroups * NA;
  if constexpr (FASTOP < 0) {
    for (int i = threadIdx.x; i < total * T; i += T) acc[i] = 0;
    __syncthreads();
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint64_t tile = static_cast<uint64_t>(T) * R;
  // The filter column is value column 0 (the trades plan filters on price):
  // its loaded words serve both.
  const bool fsame = P.fcol.type >= 0 && P.nvals > 0 && P.fcol.data == P.val[0].data &&
                     P.fcol.type == P.val[0].type && P.fcol.validity == P.val[0].validity &&
                     P.fcol.all_valid == P.val[0].all_valid;
  if constexpr (FASTOP >= 0) {
    // The trades shape: a 4-byte key (dictionary codes or I32), the F64
    // filter column as value column 0, a 4-byte integer value column 1, no
    // NULLs, fields rows / SUM(F64) / SUM(int) (kPipeSpecAvgSum), at most
    // 65533 groups, every probe key matching at most one build row, and a
    // translation domain the host put in shared memory as u16 group ids (kf16:
    // 0xffff = no match). Each lane takes 4 consecutive rows per chunk
    // with 16-byte loads, R / 4 chunks per tile, all loads of a full tile
    // issued before any row is applied; the last partial tile goes row by row.
    static_assert(SPEC == kPipeSpecAvgSum, "the trades kernel has one field set");
    constexpr int C = R / 4;  // chunks of 4 rows per lane per tile
    const int32_t* __restrict__ key = static_cast<const int32_t*>(P.key.data);
    const double* __restrict__ price = static_cast<const double*>(P.val[0].data);
    const int32_t* __restrict__ qty = static_cast<const int32_t*>(P.val[1].data);
    const double lit = P.flit_f;
    // Shared memory: the row counts as u32 (a thread counts fewer than 2^32
    // rows), [group][thread]; then the sums, [group][SUM(F64), SUM(int)]
    // [thread]; then the u16 translation table. 20 bytes per group and
    // thread instead of 24 leave room for more threads.
    const size_t cnt_words = (static_cast<size_t>(P.ngroups) * T + 1) / 2;
    uint32_t* const cnt = reinterpret_cast<uint32_t*>(acc);
    unsigned long long* const sums = acc + cnt_words;
    uint16_t* kf16 = reinterpret_cast<uint16_t*>(sums + static_cast<size_t>(P.ngroups) * 2 * T);
    for (size_t i = threadIdx.x; i < cnt_words + static_cast<size_t>(P.ngroups) * 2 * T; i += T) acc[i] = 0;
    for (uint64_t i = threadIdx.x; i < P.key_domain; i += T) kf16[i] = P.kf16[i];
    __syncthreads();
    auto pass_of = [&](double v) {
      if constexpr (FASTOP == kLT) return v < lit;
      else if constexpr (FASTOP == kLE) return v <= lit;
      else if constexpr (FASTOP == kGT) return v > lit;
      else if constexpr (FASTOP == kGE) return v >= lit;
      else if constexpr (FASTOP == kEQ) return v == lit;
      else return v != lit;
    };
    // Every key matches at most one build row here (the host checked), and
    // 4-byte keys and their domain need 32-bit arithmetic only.
    const int32_t kmin32 = static_cast<int32_t>(P.key_min);
    const uint32_t dom32 = static_cast<uint32_t>(P.key_domain);
    uint32_t* const my_cnt = cnt + threadIdx.x;
    unsigned long long* const my_sum = sums + threadIdx.x;
    auto apply = [&](int32_t k, double v, int32_t q) {
      const uint32_t sl = static_cast<uint32_t>(k) - static_cast<uint32_t>(kmin32);
      if (!pass_of(v) || k < kmin32 || sl >= dom32) return;
      const uint32_t g = kf16[sl];
      if (g == 0xffffu) return;
      my_cnt[g * T] += 1u;
      unsigned long long* a = my_sum + 2 * g * T;
      a[0] = static_cast<unsigned long long>(__double_as_longlong(__longlong_as_double(static_cast<long long>(a[0])) + v));
      a[T] += static_cast<unsigned long long>(static_cast<long long>(q));
    };
    const uint64_t full = P.n / tile * tile;  // rows in full tiles
    for (uint64_t base = blockIdx.x * tile; base < full; base += static_cast<uint64_t>(gridDim.x) * tile) {
      int4 kv[C], qv[C];
      double2 pv[C][2];
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const uint64_t p = base + (static_cast<uint64_t>(warp) * C + c) * 128 + lane * 4;
        kv[c] = __ldg(reinterpret_cast<const int4*>(key + p));
        qv[c] = __ldg(reinterpret_cast<const int4*>(qty + p));
        pv[c][0] = __ldg(reinterpret_cast<const double2*>(price + p));
        pv[c][1] = __ldg(reinterpret_cast<const double2*>(price + p + 2));
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        apply(kv[c].x, pv[c][0].x, qv[c].x);
        apply(kv[c].y, pv[c][0].y, qv[c].y);
        apply(kv[c].z, pv[c][1].x, qv[c].z);
        apply(kv[c].w, pv[c][1].y, qv[c].w);
      }
    }
    // The rows after the last full tile (fewer than one tile), one per thread.
    if (blockIdx.x == gridDim.x - 1)
      for (uint64_t p = full + threadIdx.x; p < P.n; p += T) apply(__ldg(key + p), __ldg(price + p), __ldg(qty + p));
    __syncthreads();
    // Reduce the thread copies (a warp per (group, field)) into the global
    // state: rows, SUM(F64), SUM(int) are the field set's active fields 0-2.
    for (int pr = static_cast<int>(warp); pr < P.ngroups * 3; pr += static_cast<int>(nwarps)) {
      const int g = pr / 3, c = pr % 3;
      const int f = spec_active_field(SPEC, c);
      const uint8_t kind = static_cast<uint8_t>(c == 0 ? F_ROWS : spec_kind(SPEC, f));
      uint64_t x = 0;
      for (int t = static_cast<int>(lane); t < T; t += 32)
        x = field_combine(kind, x, c == 0 ? static_cast<uint64_t>(cnt[g * T + t]) : sums[(2 * g + c - 1) * T + t]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = field_combine(kind, x, __shfl_xor_sync(0xffffffffu, x, o));
      if (lane == 0 && x)
        field_red<kRowGlobal>(reinterpret_cast<uint64_t*>(P.state + static_cast<size_t>(g) * P.nfields + f), kind, x);
    }
    return;
  } else
  for (uint64_t base = blockIdx.x * tile; base < P.n; base += static_cast<uint64_t>(gridDim.x) * tile) {
    uint32_t slot[R];
    bool vv[R][NVR];
    uint64_t vb[R][NVR];
    // Loads: every column word of every row of the tile, none of them behind a
    // test of another load, so all of them are in flight together.
    uint64_t fb[R], kb[R];
    bool fok[R], kok[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint64_t p = base + (static_cast<uint64_t>(warp) * R + j) * 32 + lane;
      const bool in = p < P.n;
      fb[j] = (in && P.fcol.type >= 0 && !fsame) ? raw_bits(P.fcol, p) : 0;
      fok[j] = in && (P.fcol.type < 0 || bit_valid(P.fcol, p));
      kb[j] = in ? raw_bits(P.key, p) : 0;
      kok[j] = in && bit_valid(P.key, p);
#pragma unroll
      for (int c = 0; c < NVR; ++c) {
        const bool use = in && c < P.nvals;
        vb[j][c] = use ? raw_bits(P.val[c], p) : 0;
        vv[j][c] = use && bit_valid(P.val[c], p);
      }
    }
    // Filter (a NULL operand drops the row), key -> translation slot.
#pragma unroll
    for (int j = 0; j < R; ++j) {
      bool ok = kok[j] && fok[j];  // NULL keys never join
      if (ok && P.fcol.type >= 0) ok = filter_bits(P, fsame ? vb[j][0] : fb[j]);
      uint64_t s = ~0ull;
      if (ok) s = static_cast<uint64_t>(bits_int(P.key.type, kb[j]) - P.key_min);
      slot[j] = s < P.key_domain ? static_cast<uint32_t>(s) : 0xffffffffu;
      // Integer values as int64 bits (F64 values stay as their bits).
#pragma unroll
      for (int c = 0; c < NVR; ++c)
        if (c < P.nvals && P.val[c].type != kF64) vb[j][c] = static_cast<uint64_t>(bits_int(P.val[c].type, vb[j][c]));
    }
    // The translation table (small: cached).
    uint32_t gi[R];
#pragma unroll
    for (int j = 0; j < R; ++j) gi[j] = slot[j] != 0xffffffffu ? __ldg(P.kfirst + slot[j]) : 0xffffffffu;
    // Apply.
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const uint32_t g0 = gi[j];
      if (g0 == 0xffffffffu) continue;
      const bool multi = (g0 & 0x80000000u) != 0;
      uint32_t cnt = 1, s0 = 0;
      if (multi) {
        cnt = __ldg(P.kcount + (g0 & 0x7fffffffu));
        s0 = __ldg(P.kstart + (g0 & 0x7fffffffu));
      }
      for (uint32_t m = 0; m < cnt; ++m) {
        const uint32_t g = multi ? __ldg(P.glist + s0 + m) : g0;
        unsigned long long* a = acc + static_cast<size_t>(g) * NA * T + threadIdx.x;
        a[0] += 1;  // the row count
        if constexpr (SPEC != kGenericSpec) {
#pragma unroll
          for (int i = 1; i <= spec_n(SPEC); ++i) {
            const int kind = spec_kind(SPEC, i);
            if (kind == 0) continue;
            const int c = spec_col(SPEC, i);
            unsigned long long* w = a + static_cast<size_t>(spec_compact(SPEC, i)) * T;
            *w = field_combine(static_cast<uint8_t>(kind), *w, field_contrib(static_cast<uint8_t>(kind), vv[j][c], vb[j][c]));
          }
        } else {
#pragma unroll
          for (int c = 0; c < NVR; ++c) {
            if (c >= P.nvals) break;
            for (int k = 0; k < P.cnf[c]; ++k) {
              const int fi = P.cfirst[c] + k;
              const uint8_t kind = P.fkind[fi];
              unsigned long long* w = a + static_cast<size_t>(fi) * T;
              *w = field_combine(kind, *w, field_contrib(kind, vv[j][c], vb[j][c]));
            }
          }
        }
      }
    }
  }
  __syncthreads();
  // Reduce the thread copies of each (group, field) in one warp, then add the
  // result to the global state (zero is every field's identity).
  for (int pr = static_cast<int>(warp); pr < total; pr += static_cast<int>(nwarps)) {
    const int g = pr / NA, c = pr % NA;
    const int f = SPEC != kGenericSpec ? spec_active_field(SPEC, c) : c;
    const uint8_t kind = SPEC != kGenericSpec ? static_cast<uint8_t>(f == 0 ? F_ROWS : spec_kind(SPEC, f)) : P.fkind[f];
    const unsigned long long* src = acc + static_cast<size_t>(pr) * T;
    uint64_t x = 0;
    for (int t = static_cast<int>(lane); t < T; t += 32) x = field_combine(kind, x, src[t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = field_combine(kind, x, __shfl_xor_sync(0xffffffffu, x, o));
    if (lane == 0 && x) field_red<kRowGlobal>(reinterpret_cast<uint64_t*>(P.state + static_cast<size_t>(g) * P.nfields + f), kind, x);
  }
}

}  // namespace

}  // namespace qeg

using namespace qeg;

extern "C" {

qeg_status qeg_filter_join_agg(qeg_ctx* ctx, const qeg_column* probe, int nprobe, const qeg_column* build, int nbuild,
                               const qeg_pipeline_desc* d, uint64_t out_capacity, const qeg_out_column* outs,
                               uint64_t* num_groups) {
  qeg::NvtxRange nvtx_range("qeg_filter_join_agg");
  return guarded(ctx, [&] {
    require(ctx && probe && build && d && outs && num_groups, "NULL argument");
    require(nprobe >= 1 && nbuild >= 1, "both sides need columns");
    require(d->probe_key < static_cast<uint32_t>(nprobe) && d->build_key < static_cast<uint32_t>(nbuild),
            "join key column index out of range");
    require(probe[d->probe_key].type == build[d->build_key].type,
            "HashJoin: join key column types must match positionally");
    const int32_t kt = probe[d->probe_key].type;
    require(kt == QEG_STR || kt == QEG_I32 || kt == QEG_I64 || kt == QEG_TS,
            "the fused pipeline joins STR or integer keys");
    require(d->group_col >= static_cast<uint32_t>(nprobe) && d->group_col < static_cast<uint32_t>(nprobe + nbuild),
            "the fused pipeline groups by a build-side column");
    require(d->naggs >= 1 && d->naggs <= kPipeMaxAggs, "the fused pipeline takes 1..16 aggregates");
    require(d->filter_col < nprobe, "filter column index out of range");
    QEG_CUDA(cudaSetDevice(ctx->device));
    const uint64_t np = probe[0].len, nb = build[0].len;
    for (int c = 0; c < nprobe; ++c) require(probe[c].len == np, "probe columns differ in length");
    for (int c = 0; c < nbuild; ++c) require(build[c].len == nb, "build columns differ in length");
    require(nb <= (1u << 22), "the fused pipeline takes a build side of at most 2^22 rows");

    // ---- host: the build side, the group ids, the probe-key translation ----
    // The small build-side arrays (and the STR code maps) come to the host in
    // one batch: device ones by asynchronous copies into the context's
    // page-locked buffer and one stream synchronisation, host ones in place.
    const qeg_column& bk = build[d->build_key];
    const qeg_column& gcol = build[d->group_col - nprobe];
    const bool bk_all = bk.all_valid || !bk.validity;
    const bool g_all = gcol.all_valid || !gcol.validity;
    struct Fetch {
      const void* src;
      size_t bytes, off;
      bool dev;
    };
    std::vector<Fetch> fetches;
    size_t fetch_bytes = 0;
    auto want = [&](const void* src, size_t bytes) {
      fetches.push_back(Fetch{src, bytes, fetch_bytes, bytes > 0 && is_device_ptr(src)});
      fetch_bytes += (bytes + 15) & ~size_t{15};
      return fetches.size() - 1;
    };
    const size_t f_bkv = want(bk.data, nb * type_width(bk.type));
    const size_t f_bkw = bk_all ? SIZE_MAX : want(bk.validity, ((nb + 63) / 64) * 8);
    const size_t f_gv = want(gcol.data, nb * type_width(gcol.type));
    const size_t f_gw = g_all ? SIZE_MAX : want(gcol.validity, ((nb + 63) / 64) * 8);
    size_t f_gcm = SIZE_MAX, f_bmap = SIZE_MAX, f_pmap = SIZE_MAX;
    if (gcol.type == QEG_STR) {
      require(gcol.code_map != nullptr, "STR group column needs a code map");
      f_gcm = want(gcol.code_map, gcol.code_map_len * 4);
    }
    if (kt == QEG_STR) {
      require(bk.code_map && probe[d->probe_key].code_map, "STR join keys need code maps");
      f_bmap = want(bk.code_map, bk.code_map_len * 4);
      f_pmap = want(probe[d->probe_key].code_map, probe[d->probe_key].code_map_len * 4);
    }
    uint8_t* fetched = static_cast<uint8_t*>(ctx->pinned_in.reserve(std::max<size_t>(fetch_bytes, 16)));
    bool any_dev = false;
    for (const Fetch& f : fetches) {
      if (f.bytes == 0) continue;
      if (f.dev) {
        QEG_CUDA(cudaMemcpyAsync(fetched + f.off, f.src, f.bytes, cudaMemcpyDeviceToHost, ctx->stream));
        any_dev = true;
      } else {
        std::memcpy(fetched + f.off, f.src, f.bytes);
      }
    }
    if (any_dev) QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    auto at = [&](size_t i) -> const uint8_t* { return i == SIZE_MAX ? nullptr : fetched + fetches[i].off; };
    auto valid_at = [](const uint8_t* words, uint64_t i) {
      if (!words) return true;
      uint64_t w;
      std::memcpy(&w, words + (i >> 6) * 8, 8);
      return ((w >> (i & 63)) & 1ull) != 0;
    };
    auto ival = [](const uint8_t* v, int32_t t, uint64_t i) -> int64_t {
      if (t == QEG_I32 || t == QEG_STR) {
        int32_t x;
        std::memcpy(&x, v + i * 4, 4);
        return x;
      }
      if (t == QEG_BOOL) return v[i];
      int64_t x;
      std::memcpy(&x, v + i * 8, 8);
      return x;
    };
    const uint8_t* bkv = at(f_bkv);
    const uint8_t* bkw = at(f_bkw);
    const uint8_t* gv = at(f_gv);
    const uint8_t* gw = at(f_gw);
    const uint8_t* gcm = at(f_gcm);
    // Group ids over the distinct group values of build rows (NULL is a
    // group): a dense table over the value range for integer group columns
    // spanning at most 2^20 values, a hash map otherwise.
    std::vector<uint64_t> gword;  // canonical group word per group
    std::vector<uint8_t> gnull;
    int32_t null_gid = -1;
    std::vector<int32_t> row_group(nb, -1);
    std::vector<uint64_t> words(nb);
    for (uint64_t b = 0; b < nb; ++b) {
      if (!valid_at(gw, b)) continue;
      uint64_t w;
      if (gcol.type == QEG_F64) {
        double x;
        std::memcpy(&x, gv + b * 8, 8);
        uint64_t bits;
        std::memcpy(&bits, &x, 8);
        if (std::isnan(x)) bits = kCanonNaN;
        else if (x == 0.0) bits = 0;
        w = bits;
      } else if (gcol.type == QEG_STR) {
        const int32_t code = static_cast<int32_t>(ival(gv, QEG_STR, b));
        require(code >= 0 && static_cast<uint64_t>(code) < gcol.code_map_len, "STR code outside its code map");
        int32_t id;
        std::memcpy(&id, gcm + static_cast<size_t>(code) * 4, 4);
        w = static_cast<uint64_t>(static_cast<int64_t>(id));
      } else {
        w = static_cast<uint64_t>(ival(gv, gcol.type, b));
      }
      words[b] = w;
    }
    const bool gint = gcol.type == QEG_I32 || gcol.type == QEG_I64 || gcol.type == QEG_TS || gcol.type == QEG_BOOL ||
                      gcol.type == QEG_STR;
    int64_t gmin = INT64_MAX, gmax = INT64_MIN;
    if (gint)
      for (uint64_t b = 0; b < nb; ++b)
        if (valid_at(gw, b)) {
          gmin = std::min(gmin, static_cast<int64_t>(words[b]));
          gmax = std::max(gmax, static_cast<int64_t>(words[b]));
        }
    const bool dense_groups =
        gint && gmin <= gmax && static_cast<uint64_t>(gmax) - static_cast<uint64_t>(gmin) < (uint64_t{1} << 20);
    std::vector<int32_t> dense_gid(dense_groups ? static_cast<size_t>(gmax - gmin) + 1 : 0, -1);
    std::unordered_map<uint64_t, uint32_t> gid;
    for (uint64_t b = 0; b < nb; ++b) {
      if (!valid_at(gw, b)) {
        if (null_gid < 0) {
          null_gid = static_cast<int32_t>(gword.size());
          gword.push_back(0);
          gnull.push_back(1);
        }
        row_group[b] = null_gid;
        continue;
      }
      const uint64_t w = words[b];
      if (dense_groups) {
        int32_t& g = dense_gid[static_cast<size_t>(static_cast<int64_t>(w) - gmin)];
        if (g < 0) {
          g = static_cast<int32_t>(gword.size());
          gword.push_back(w);
          gnull.push_back(0);
        }
        row_group[b] = g;
        continue;
      }
      auto it = gid.find(w);
      if (it == gid.end()) {
        it = gid.emplace(w, static_cast<uint32_t>(gword.size())).first;
        gword.push_back(w);
        gnull.push_back(0);
      }
      row_group[b] = static_cast<int32_t>(it->second);
    }
    const int ngroups = static_cast<int>(gword.size());
    // Build key -> value id (STR: by value through the code map).
    std::vector<int32_t> bmap, pmap;
    if (kt == QEG_STR) {
      bmap.resize(bk.code_map_len);
      pmap.resize(probe[d->probe_key].code_map_len);
      std::memcpy(bmap.data(), at(f_bmap), bmap.size() * 4);
      std::memcpy(pmap.data(), at(f_pmap), pmap.size() * 4);
    }
    // (join value, group id) of every build row with a non-NULL key.
    std::vector<int64_t> bval;
    std::vector<uint32_t> bgrp;
    bval.reserve(nb);
    bgrp.reserve(nb);
    int64_t vmin = INT64_MAX, vmax = INT64_MIN;
    for (uint64_t b = 0; b < nb; ++b) {
      if (!valid_at(bkw, b)) continue;
      int64_t v = ival(bkv, bk.type, b);
      if (kt == QEG_STR) {
        require(v >= 0 && static_cast<uint64_t>(v) < bmap.size(), "STR code outside its code map");
        v = bmap[static_cast<size_t>(v)];
      }
      bval.push_back(v);
      bgrp.push_back(static_cast<uint32_t>(row_group[b]));
      vmin = std::min(vmin, v);
      vmax = std::max(vmax, v);
    }
    // Probe-key domain: the probe dictionary (STR) or the build keys' range.
    int64_t kmin = 0;
    uint64_t domain = 0;
    if (kt == QEG_STR) {
      domain = pmap.size();
    } else if (!bval.empty()) {
      require(static_cast<uint64_t>(vmax - vmin) < (1ull << 24),
              "integer join keys must span fewer than 2^24 values for the fused pipeline");
      kmin = vmin;
      domain = static_cast<uint64_t>(vmax - vmin) + 1;
    }
    // Counting sort of the build rows by join value (values span < 2^24, STR
    // value ids are dense): glist holds the group ids value by value, and a
    // probe key's run is [vstart[v], vstart[v] + vcount[v]).
    const uint64_t vrange = bval.empty() ? 0 : static_cast<uint64_t>(vmax - vmin) + 1;
    require(vrange < (1ull << 26), "join key values span too many values for the fused pipeline");
    std::vector<uint32_t> vstart(vrange + 1, 0), glist(bval.size());
    for (int64_t v : bval) ++vstart[static_cast<size_t>(v - vmin) + 1];
    for (uint64_t i = 0; i < vrange; ++i) vstart[i + 1] += vstart[i];
    {
      std::vector<uint32_t> fill(vstart.begin(), vstart.end() - 1);
      for (size_t i = 0; i < bval.size(); ++i) glist[fill[static_cast<size_t>(bval[i] - vmin)]++] = bgrp[i];
    }
    std::vector<uint32_t> kstart(std::max<uint64_t>(domain, 1), 0), kcount(std::max<uint64_t>(domain, 1), 0);
    for (uint64_t s = 0; s < domain; ++s) {
      const int64_t v = kt == QEG_STR ? pmap[s] : kmin + static_cast<int64_t>(s);
      if (v < vmin || v > vmax) continue;
      const size_t i = static_cast<size_t>(v - vmin);
      kstart[s] = vstart[i];
      kcount[s] = vstart[i + 1] - vstart[i];
    }

    // ---- aggregate fields over probe columns (the AggState encodings) ------
    std::vector<uint32_t> vcols;
    std::vector<std::vector<uint8_t>> per;
    std::vector<int> vfield(d->naggs, -1), nfield(d->naggs, -1);
    std::vector<int32_t> rtypes{gcol.type};
    std::vector<uint8_t> fk{F_ROWS};
    for (int a = 0; a < d->naggs; ++a) {
      const qeg_agg_spec s = d->aggs[a];
      require(s.func >= QEG_COUNT_STAR && s.func <= QEG_AVG, "unknown aggregate function");
      if (s.func == QEG_COUNT_STAR) {
        rtypes.push_back(QEG_I64);
        continue;
      }
      require(s.input_col < static_cast<uint32_t>(nprobe), "the fused pipeline aggregates probe-side columns");
      const int32_t in = probe[s.input_col].type;
      require(in != QEG_STR || (s.func != QEG_SUM && s.func != QEG_AVG), "SUM/AVG are not defined on STR (VARCHAR)");
      rtypes.push_back(s.func == QEG_COUNT ? QEG_I64
                       : s.func == QEG_AVG ? QEG_F64
                       : s.func == QEG_SUM ? (in == QEG_F64 ? QEG_F64 : QEG_I64) : in);
      auto it = std::find(vcols.begin(), vcols.end(), s.input_col);
      if (it == vcols.end()) {
        require(vcols.size() < kPipeMaxVals, "the fused pipeline reads at most 4 probe value columns");
        vcols.push_back(s.input_col);
        per.push_back({F_NULLS});
        it = vcols.end() - 1;
      }
      const size_t c = it - vcols.begin();
      const bool f = in == QEG_F64;
      uint8_t kind = F_NULLS;
      if (s.func == QEG_SUM || s.func == QEG_AVG) kind = f ? F_SUMF : F_SUMI;
      if (s.func == QEG_MIN) kind = f ? F_MINF : F_MINI;
      if (s.func == QEG_MAX) kind = f ? F_MAXF : F_MAXI;
      if (std::find(per[c].begin(), per[c].end(), kind) == per[c].end()) per[c].push_back(kind);
    }
    PipeK P{};
    P.nvals = static_cast<int>(vcols.size());
    for (size_t c = 0; c < vcols.size(); ++c) {
      P.cfirst[c] = static_cast<uint8_t>(fk.size());
      P.cnf[c] = static_cast<uint8_t>(per[c].size());
      for (uint8_t k : per[c]) fk.push_back(k);
    }
    require(fk.size() <= static_cast<size_t>(kMaxFields), "too many aggregate state fields");
    for (int a = 0; a < d->naggs; ++a) {
      const qeg_agg_spec s = d->aggs[a];
      if (s.func == QEG_COUNT_STAR) continue;
      const size_t c = std::find(vcols.begin(), vcols.end(), s.input_col) - vcols.begin();
      const bool f = probe[s.input_col].type == QEG_F64;
      uint8_t kind = F_NULLS;
      if (s.func == QEG_SUM || s.func == QEG_AVG) kind = f ? F_SUMF : F_SUMI;
      if (s.func == QEG_MIN) kind = f ? F_MINF : F_MINI;
      if (s.func == QEG_MAX) kind = f ? F_MAXF : F_MAXI;
      for (int k = 0; k < P.cnf[c]; ++k) {
        if (fk[P.cfirst[c] + k] == F_NULLS) nfield[a] = P.cfirst[c] + k;
        if (fk[P.cfirst[c] + k] == kind) vfield[a] = P.cfirst[c] + k;
      }
    }
    P.nfields = static_cast<int>(fk.size());
    for (int f = 0; f < P.nfields; ++f) P.fkind[f] = fk[f];
    P.ngroups = std::max(ngroups, 1);
    *num_groups = 0;

    // ---- device ---------------------------------------------------------
    std::vector<StagedCol> staged(nprobe);
    std::vector<bool> need(nprobe, false);
    need[d->probe_key] = true;
    for (uint32_t c : vcols) need[c] = true;
    if (d->filter_col >= 0) need[d->filter_col] = true;
    for (int c = 0; c < nprobe; ++c)
      if (need[c]) stage_column(ctx, probe[c], staged[c]);
    P.fcol.type = -1;
    if (d->filter_col >= 0) {
      P.fcol = staged[d->filter_col].dev;
      P.fop = d->filter_op;
      P.flit_f = d->filter_value;
      P.flit_i = static_cast<int64_t>(d->filter_value);
      require(P.fop >= kLT && P.fop <= kNE, "unknown comparison");
      if (P.fcol.type != kF64) {
        // An integer column compared with a non-integral literal: adjust the
        // bound so the integer comparison gives the same answer.
        const double l = d->filter_value;
        const double fl = std::floor(l);
        if (fl != l) {
          if (P.fop == kLT || P.fop == kLE) { P.flit_i = static_cast<int64_t>(fl); P.fop = kLE; }
          else if (P.fop == kGT || P.fop == kGE) { P.flit_i = static_cast<int64_t>(fl); P.fop = kGT; }
          else if (P.fop == kEQ) P.fop = kNever;  // an integer never equals it
          else P.fop = kAlways;                   // and always differs from it
        }
      }
    }
    P.key = staged[d->probe_key].dev;
    if (kt == QEG_STR) P.key.code_map = nullptr;  // the translation table is indexed by code
    P.key_min = kmin;
    P.key_domain = domain;
    for (size_t c = 0; c < vcols.size(); ++c) P.val[c] = staged[vcols[c]].dev;
    P.n = np;
    // One-load translation for keys that match exactly one build row.
    std::vector<uint32_t> kfirst(kstart.size(), 0xffffffffu);
    for (uint64_t sl = 0; sl < domain; ++sl) {
      if (kcount[sl] == 1) kfirst[sl] = glist[kstart[sl]];
      else if (kcount[sl] > 1) kfirst[sl] = 0x80000000u | static_cast<uint32_t>(sl);
    }
    std::vector<uint16_t> kf16;
    if (ngroups <= 65533) {
      kf16.resize(kfirst.size());
      for (size_t i = 0; i < kfirst.size(); ++i)
        kf16[i] = kfirst[i] == 0xffffffffu ? 0xffffu : (kfirst[i] & 0x80000000u) ? 0xfffeu : static_cast<uint16_t>(kfirst[i]);
    }
    // The translation tables go to the device in one copy from the context's
    // page-locked buffer into one device buffer: kstart, kcount, kfirst,
    // glist (u32 each), then kf16 (u16); the state is zeroed beside them.
    const size_t n_kst = kstart.size(), n_kfi = kfirst.size(), n_gl = std::max<size_t>(glist.size(), 1);
    const size_t o_kst = 0, o_kct = o_kst + n_kst * 4, o_kfi = o_kct + n_kst * 4, o_gl = o_kfi + n_kfi * 4;
    const size_t o_k16 = (o_gl + n_gl * 4 + 15) & ~size_t{15};
    const size_t tbl_bytes = o_k16 + ((std::max<size_t>(kf16.size(), 1) * 2 + 15) & ~size_t{15});
    uint8_t* tbl = static_cast<uint8_t*>(ctx->pinned_out.reserve(tbl_bytes));
    std::memcpy(tbl + o_kst, kstart.data(), n_kst * 4);
    std::memcpy(tbl + o_kct, kcount.data(), n_kst * 4);
    std::memcpy(tbl + o_kfi, kfirst.data(), n_kfi * 4);
    if (!glist.empty()) std::memcpy(tbl + o_gl, glist.data(), glist.size() * 4);
    if (!kf16.empty()) std::memcpy(tbl + o_k16, kf16.data(), kf16.size() * 2);
    DevBuf dtbl(tbl_bytes, ctx->stream), dstate(static_cast<size_t>(P.ngroups) * P.nfields * 8, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(dtbl.get(), tbl, tbl_bytes, cudaMemcpyHostToDevice, ctx->stream));
    QEG_CUDA(cudaMemsetAsync(dstate.get(), 0, dstate.bytes(), ctx->stream));
    uint8_t* dt = dtbl.get<uint8_t>();
    P.kstart = reinterpret_cast<const uint32_t*>(dt + o_kst);
    P.kcount = reinterpret_cast<const uint32_t*>(dt + o_kct);
    P.kfirst = reinterpret_cast<const uint32_t*>(dt + o_kfi);
    P.kf16 = kf16.empty() ? nullptr : reinterpret_cast<const uint16_t*>(dt + o_k16);
    P.glist = reinterpret_cast<const uint32_t*>(dt + o_gl);
    P.state = dstate.get<unsigned long long>();
    const int block = 512;
    // The kernel for this field set: COUNT(*) with SUM/AVG over an F64 column
    // and SUM over an integer column (the trades pipeline's AVG(price),
    // SUM(qty)), with or without NULL counts, has its own kernel.
    void (*kern)(PipeK) = pipeline_kernel<kGenericSpec>;
    if (P.nvals == 2 && P.nfields == 5) {
      uint32_t spec = 4u;
      for (int i = 1; i <= 4; ++i) {
        const int col = i <= P.cnf[0] ? 0 : 1;
        int kind = P.fkind[i];
        if (kind == F_NULLS && P.val[col].all_valid) kind = 0;
        spec |= spec_field(i, kind, col);
      }
      if (spec == kPipeSpecAvgSum) kern = pipeline_kernel<kPipeSpecAvgSum>;
      else if (spec == kPipeSpecAvgSumNulls) kern = pipeline_kernel<kPipeSpecAvgSumNulls>;
    }
    // Thread-private states (pipeline_lanes_kernel) while 256, 128 or 64
    // threads' copies of every group's active fields fit in shared memory;
    // QEG_PIPE_KERNEL=shared selects the shared-state kernel below.
    {
      const char* e = std::getenv("QEG_PIPE_KERNEL");
      const bool want_lanes = !(e && std::strcmp(e, "shared") == 0);
      uint32_t spec = kGenericSpec;
      if (kern == pipeline_kernel<kPipeSpecAvgSum>) spec = kPipeSpecAvgSum;
      else if (kern == pipeline_kernel<kPipeSpecAvgSumNulls>) spec = kPipeSpecAvgSumNulls;
      const int na = spec == kGenericSpec ? P.nfields : spec_nactive(spec);
      int T = 256;
      while (T >= 64 && static_cast<size_t>(P.ngroups) * na * 8 * T > ctx->smem_optin) T >>= 1;
      if (want_lanes && T >= 64) {
        size_t lsb_fast = 0;
        void (*lk)(PipeK, int) = spec == kPipeSpecAvgSum        ? pipeline_lanes_kernel<kPipeSpecAvgSum, 16, -1>
                                 : spec == kPipeSpecAvgSumNulls ? pipeline_lanes_kernel<kPipeSpecAvgSumNulls, 16, -1>
                                                                : pipeline_lanes_kernel<kGenericSpec, 8, -1>;
        // The trades shape (see the kernel) takes the typed variant.
        const bool key4 = P.key.type == kI32 || P.key.type == kSTR;
        const bool fsame = P.fcol.type == kF64 && P.val[0].type == kF64 && P.fcol.data == P.val[0].data &&
                           P.fcol.all_valid && P.val[0].all_valid;
        // (16-byte loads: column starts 16-byte aligned; the u16 translation
        // table beside the states in shared memory.)
        const bool aligned = (reinterpret_cast<uintptr_t>(P.key.data) % 16) == 0 &&
                             (reinterpret_cast<uintptr_t>(P.val[0].data) % 16) == 0 &&
                             (reinterpret_cast<uintptr_t>(P.val[1].data) % 16) == 0;
        // Threads of the typed kernel: the most (a multiple of 32, at most
        // kLanesMaxThreads) whose states (20 bytes per group and thread) and
        // the translation table fit.
        auto fast_bytes = [&](int t) {
          const size_t cw = (static_cast<size_t>(P.ngroups) * t + 1) / 2;
          return (cw + static_cast<size_t>(P.ngroups) * 2 * t) * 8 + ((domain * 2 + 15) / 16) * 16;
        };
        int T_fast = kLanesMaxThreads;
        while (T_fast > 64 && fast_bytes(T_fast) > ctx->smem_optin) T_fast -= 32;
        const size_t fast_sb = fast_bytes(T_fast);
        const bool single = std::none_of(kf16.begin(), kf16.end(), [](uint16_t x) { return x == 0xfffeu; });
        if (spec == kPipeSpecAvgSum && key4 && P.key.all_valid && fsame && P.val[1].type == kI32 &&
            P.val[1].all_valid && aligned && P.kf16 && single && domain < (1ull << 31) &&
            fast_sb <= ctx->smem_optin) {
          lsb_fast = fast_sb;
          T = T_fast;
          switch (P.fop) {
            case kLT: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kLT>; break;
            case kLE: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kLE>; break;
            case kGT: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kGT>; break;
            case kGE: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kGE>; break;
            case kEQ: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kEQ>; break;
            case kNE: lk = pipeline_lanes_kernel<kPipeSpecAvgSum, 16, kNE>; break;
            default: break;
          }
        }
        const size_t lsb = lsb_fast ? lsb_fast : static_cast<size_t>(P.ngroups) * na * 8 * T;
        const int lper = blocks_per_sm(reinterpret_cast<const void*>(lk), T, lsb);
        const int rows_per_tile = T * (spec == kGenericSpec ? 8 : 16);
        const uint64_t lwant = (np + rows_per_tile - 1) / rows_per_tile;
        const unsigned lgrid = static_cast<unsigned>(
            std::max<uint64_t>(1, std::min<uint64_t>(lwant, static_cast<uint64_t>(ctx->sms) * std::max(lper, 1))));
        if (np > 0 && domain > 0 && ngroups > 0) {
          lk<<<lgrid, T, lsb, ctx->stream>>>(P, na);
          ctx->launches++;
          QEG_CUDA(cudaGetLastError());
        }
        kern = nullptr;  // done
      }
    }
    if (kern) {
      const size_t per_copy = static_cast<size_t>(P.ngroups) * (P.nfields | 1) * 8;
      P.per_warp = per_copy * (block / 32) <= 96 * 1024 ? 1 : 0;
      // Per-lane shared reductions by default (measured 2.95 vs 3.10 ms per
      // 200M-row call against warp peer aggregation); QEG_PIPE_LANES=0 selects
      // the peer-aggregating variant.
      {
        const char* e = std::getenv("QEG_PIPE_LANES");
        P.lane_reds = e ? (std::atoi(e) != 0 ? 1 : 0) : 1;
      }
      const size_t sb = P.per_warp ? per_copy * (block / 32) : per_copy;
      require(sb <= ctx->smem_optin, "too many groups for the fused pipeline's shared-memory state");
      const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), block, sb);
      const uint64_t want = (np + block * 16 - 1) / (block * 16);
      const unsigned grid = static_cast<unsigned>(
          std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
      if (np > 0 && domain > 0 && ngroups > 0) {
        kern<<<grid, block, sb, ctx->stream>>>(P);
        ctx->launches++;
        QEG_CUDA(cudaGetLastError());
      }
    }
    std::vector<unsigned long long> st(static_cast<size_t>(P.ngroups) * P.nfields);
    QEG_CUDA(cudaMemcpyAsync(st.data(), dstate.get(), st.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    check_device_error(ctx);

    // ---- finalise (ops/agg_internal.h:169-229) into the caller's columns ---
    uint64_t out = 0;
    const int ncol = 1 + d->naggs;
    std::vector<std::vector<uint8_t>> vals(ncol);
    std::vector<std::vector<uint8_t>> ok(ncol);
    for (int g = 0; g < ngroups; ++g) {
      const unsigned long long* f = &st[static_cast<size_t>(g) * P.nfields];
      if (f[0] == 0) continue;  // no joined row landed in this group
      auto put = [&](int c, uint64_t w, bool valid) {
        const size_t wd = type_width(rtypes[c]);
        const size_t o = vals[c].size();
        vals[c].resize(o + wd);
        std::memcpy(vals[c].data() + o, &w, wd);  // little-endian low bytes
        ok[c].push_back(valid ? 1 : 0);
      };
      put(0, gnull[g] ? 0 : gword[g], !gnull[g]);
      for (int a = 0; a < d->naggs; ++a) {
        const uint64_t rows = f[0];
        const uint64_t nn = rows - (nfield[a] >= 0 ? f[nfield[a]] : 0);
        const qeg_agg_spec s = d->aggs[a];
        uint64_t w = 0;
        bool valid = true;
        if (s.func == QEG_COUNT_STAR) w = rows;
        else if (s.func == QEG_COUNT) w = nn;
        else if (nn == 0) valid = false;
        else if (s.func == QEG_SUM) w = f[vfield[a]];
        else if (s.func == QEG_AVG) {
          const double sum = fk[vfield[a]] == F_SUMF ? [&] { double x; std::memcpy(&x, &f[vfield[a]], 8); return x; }()
                                                      : static_cast<double>(static_cast<int64_t>(f[vfield[a]]));
          const double avg = sum / static_cast<double>(nn);
          std::memcpy(&w, &avg, 8);
        } else {
          const uint8_t k = fk[vfield[a]];
          const uint64_t e = f[vfield[a]];
          w = k == F_MINF ? dec_f64_bits(~e) : k == F_MAXF ? dec_f64_bits(e)
              : k == F_MINI ? static_cast<uint64_t>(dec_i64(~e)) : static_cast<uint64_t>(dec_i64(e));
        }
        put(1 + a, w, valid);
      }
      ++out;
    }
    require(out <= out_capacity, "output capacity too small for the groups");
    for (int c = 0; c < ncol; ++c) {
      const qeg_out_column& oc = outs[c];
      if ((!oc.data || !is_device_ptr(oc.data)) && (!oc.validity || !is_device_ptr(oc.validity))) {
        // Host outputs: write the (few) group rows directly.
        if (oc.data && out) std::memcpy(oc.data, vals[c].data(), vals[c].size());
        bool all = true;
        const uint64_t nw = (out + 63) / 64;
        std::vector<uint64_t> words(nw, ~0ull);  // padding bits set, as in the column format
        for (uint64_t i = 0; i < out; ++i) {
          if (!ok[c][i]) {
            words[i >> 6] &= ~(1ull << (i & 63));
            all = false;
          }
        }
        if (oc.validity && nw) std::memcpy(oc.validity, words.data(), nw * 8);
        if (oc.all_valid) *oc.all_valid = all ? 1 : 0;
        continue;
      }
      DevBuf dv(std::max<size_t>(vals[c].size(), 8), ctx->stream), dok(std::max<uint64_t>(out, 1), ctx->stream);
      if (out) {
        QEG_CUDA(cudaMemcpyAsync(dv.get(), vals[c].data(), vals[c].size(), cudaMemcpyHostToDevice, ctx->stream));
        QEG_CUDA(cudaMemcpyAsync(dok.get(), ok[c].data(), out, cudaMemcpyHostToDevice, ctx->stream));
      }
      fetch_column(ctx, dv.get(), dok.get<uint8_t>(), type_width(rtypes[c]), 0, out, outs[c]);
    }
    *num_groups = out;
  });
}

}  // extern "C"
