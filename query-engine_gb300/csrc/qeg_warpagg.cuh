// qeg_warpagg.cuh -- warp-level peer aggregation shared by the GROUP BY
// kernels (qeg_agg.cu, qeg_batch.cu).
#pragma once

#include "qeg_agg.h"
#include "qeg_device.cuh"

namespace qeg {

// ---------------------------------------------------------------------------
// Warp peer aggregation. Lanes of a warp whose rows fall in the same group
// ("peers", found with __match_any_sync) combine their contributions in
// registers before the group's lowest lane applies them with one atomic per
// field, so a heavy hitter costs one shared/global atomic per warp instead of
// one per row. The combine is a pairwise tree over the peers in lane order
// (at most 5 rounds); its shuffle schedule depends only on the peer masks, so
// it is computed once per row batch and replayed for every field.
// ---------------------------------------------------------------------------
struct PeerPlan {
  uint32_t src;   // 5 bits per round: the lane to read from
  uint32_t take;  // bit r: combine what round r read
  int rounds;     // warp-uniform
};

__device__ __forceinline__ PeerPlan plan_peers(unsigned peers, unsigned lane) {
  PeerPlan pp{0u, 0u, 0};
  unsigned alive = peers;
  unsigned rank = __popc(peers & ((1u << lane) - 1u));
  const unsigned higher = lane == 31 ? 0u : (~0u << (lane + 1));
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    const unsigned above = alive & higher;
    if (!__any_sync(0xffffffffu, above != 0)) break;
    const unsigned nxt = above ? static_cast<unsigned>(__ffs(above) - 1) : lane;
    pp.src |= nxt << (5 * r);
    if (above && !(rank & 1u)) pp.take |= 1u << r;
    // Odd ranks were just read by their even neighbour and leave the tree.
    alive &= ~__ballot_sync(0xffffffffu, rank & 1u);
    rank >>= 1;
    pp.rounds = r + 1;
  }
  return pp;
}

// Lanes of the warp whose 64-bit word w equals this lane's (all lanes call
// it). The match runs on a 32-bit fold of the word -- on GB300 a 64-bit
// __match_any_sync costs twice a 32-bit one (106 against 53 clocks per warp
// instruction per SM) -- and, unless the words are known to fit 32 bits, a
// lane whose word differs from its match group's first lane's (a fold
// collision) is left alone: exact, at worst less combining.
__device__ __forceinline__ unsigned match_word64(uint64_t w, unsigned lane, bool fits32) {
  const unsigned same = __match_any_sync(0xffffffffu, static_cast<uint32_t>(w ^ (w >> 32)));
  if (fits32) return same;
  const int ref = __ffs(same) - 1;
  const bool eq = __shfl_sync(0xffffffffu, w, ref) == w;
  const unsigned eqmask = __ballot_sync(0xffffffffu, eq);
  return eq ? (same & eqmask) : (1u << lane);
}

// How a field merges: integer add (row / NULL counts, integer sums), F64 add
// (F64 sums) or unsigned max (every MIN/MAX encoding). The kind of a field is
// the same in every lane, so the branches below never diverge, and they are
// plain compares rather than jump tables.
enum FieldOp : int { kOpAdd = 0, kOpFAdd = 1, kOpMax = 2 };

__device__ __forceinline__ int field_op(uint8_t kind) {
  return kind <= F_SUMI ? kOpAdd : (kind == F_SUMF ? kOpFAdd : kOpMax);
}

// The contribution of one (valid, value bits) input to a field, in the
// field's identity-is-zero encoding.
__device__ __forceinline__ uint64_t field_contrib(uint8_t kind, bool valid, uint64_t bits) {
  if (kind == F_ROWS) return 1;
  if (kind == F_NULLS) return valid ? 0 : 1;
  if (!valid) return 0;
  if (kind <= F_SUMF) return bits;
  const uint64_t e = (kind <= F_MAXI) ? enc_i64(static_cast<int64_t>(bits)) : enc_f64_bits(bits);
  return (kind & 1) ? e : ~e;  // MAXI / MAXF are odd, MINI / MINF even
}

template <int OP>
__device__ __forceinline__ uint64_t op_combine(uint64_t a, uint64_t b) {
  if (OP == kOpAdd) return a + b;
  if (OP == kOpFAdd)
    return static_cast<uint64_t>(__double_as_longlong(__longlong_as_double(static_cast<long long>(a)) +
                                                      __longlong_as_double(static_cast<long long>(b))));
  return a > b ? a : b;
}

__device__ __forceinline__ uint64_t field_combine(uint8_t kind, uint64_t a, uint64_t b) {
  const int op = field_op(kind);
  if (op == kOpAdd) return op_combine<kOpAdd>(a, b);
  if (op == kOpFAdd) return op_combine<kOpFAdd>(a, b);
  return op_combine<kOpMax>(a, b);
}

// Merges one combined contribution into a table word (shared or global).
__device__ __forceinline__ void field_apply(uint64_t* w, uint8_t kind, uint64_t x) {
  if (!x) return;  // zero is the identity of every field
  const int op = field_op(kind);
  unsigned long long* u = reinterpret_cast<unsigned long long*>(w);
  if (op == kOpAdd) atomicAdd(u, static_cast<unsigned long long>(x));
  else if (op == kOpFAdd) atomicAdd(reinterpret_cast<double*>(w), __longlong_as_double(static_cast<long long>(x)));
  else atomicMax(u, static_cast<unsigned long long>(x));
}

// Where a field block lives, so a merge uses the matching instruction: a
// warp-private row (plain read-modify-write), a CTA table row (shared-memory
// reduction) or a global table row (global reduction).
enum RowSpace : int { kRowPrivate = 0, kRowShared = 1, kRowGlobal = 2 };

// Merges `x` into a field word with a reduction of the given state space.
// Zero is the identity of every field and is skipped.
template <int SPACE>
__device__ __forceinline__ void field_red(uint64_t* w, uint8_t kind, uint64_t x) {
  if (!x) return;
  const int op = field_op(kind);
  if (SPACE == kRowPrivate) {
    *w = field_combine(kind, *w, x);
  } else if (SPACE == kRowShared) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(w));
    if (op == kOpAdd) asm volatile("red.shared.add.u64 [%0], %1;" ::"r"(a), "l"(x) : "memory");
    else if (op == kOpFAdd) asm volatile("red.shared.add.f64 [%0], %1;" ::"r"(a), "d"(__longlong_as_double(static_cast<long long>(x))) : "memory");
    else asm volatile("red.shared.max.u64 [%0], %1;" ::"r"(a), "l"(x) : "memory");
  } else {
    if (op == kOpAdd) asm volatile("red.global.add.u64 [%0], %1;" ::"l"(w), "l"(x) : "memory");
    else if (op == kOpFAdd) asm volatile("red.global.add.f64 [%0], %1;" ::"l"(w), "d"(__longlong_as_double(static_cast<long long>(x))) : "memory");
    else asm volatile("red.global.max.u64 [%0], %1;" ::"l"(w), "l"(x) : "memory");
  }
}

// field_red with the space chosen at run time.
__device__ __forceinline__ void field_red_at(int space, uint64_t* w, uint8_t kind, uint64_t x) {
  if (space == kRowPrivate) field_red<kRowPrivate>(w, kind, x);
  else if (space == kRowShared) field_red<kRowShared>(w, kind, x);
  else field_red<kRowGlobal>(w, kind, x);
}

template <int OP>
__device__ __forceinline__ uint64_t peer_reduce_op(uint64_t x, const PeerPlan& pp) {
#pragma unroll 1
  for (int r = 0; r < pp.rounds; ++r) {
    const uint64_t t = __shfl_sync(0xffffffffu, x, (pp.src >> (5 * r)) & 31u);
    if ((pp.take >> r) & 1u) x = op_combine<OP>(x, t);
  }
  return x;
}

__device__ __forceinline__ uint64_t peer_reduce(uint64_t x, uint8_t kind, const PeerPlan& pp) {
  if (pp.rounds == 0) return x;
  const int op = field_op(kind);
  if (op == kOpAdd) return peer_reduce_op<kOpAdd>(x, pp);
  if (op == kOpFAdd) return peer_reduce_op<kOpFAdd>(x, pp);
  return peer_reduce_op<kOpMax>(x, pp);
}

// ---------------------------------------------------------------------------
// Field-set specialisation. A SPEC packs the value fields of a row (fields
// 1..n; field 0 is the row count): bits 0-3 hold n (<= 7), and field i (1-based)
// has 4 bits at 4*i: the FieldKind in bits 0-2 (0 = skip: a NULL count of a
// column without NULLs, which stays 0) and the value column (0 or 1) in bit 3.
// Kernels instantiated for a SPEC unroll the field loop with every kind known
// at compile time; kGenericSpec means "read the kinds from the parameter block".
// ---------------------------------------------------------------------------
constexpr uint32_t kGenericSpec = 0xffffffffu;

__host__ __device__ constexpr int spec_n(uint32_t spec) { return static_cast<int>(spec & 15u); }
__host__ __device__ constexpr int spec_kind(uint32_t spec, int i) { return static_cast<int>((spec >> (4 * i)) & 7u); }
__host__ __device__ constexpr int spec_col(uint32_t spec, int i) { return static_cast<int>((spec >> (4 * i + 3)) & 1u); }
__host__ __device__ constexpr uint32_t spec_field(int i, int kind, int col) {
  return (static_cast<uint32_t>(kind) | (static_cast<uint32_t>(col) << 3)) << (4 * i);
}

// Reduces every field of SPEC across the peers (all lanes call it), then lets
// the leader merge the results into the field block `f` in state space SPACE.
template <uint32_t SPEC, int SPACE>
__device__ __forceinline__ void spec_merge(uint64_t* f, const uint64_t (&xs)[8]) {
#pragma unroll
  for (int i = 1; i <= spec_n(SPEC); ++i)
    if (spec_kind(SPEC, i) != 0) field_red<SPACE>(f + i, static_cast<uint8_t>(spec_kind(SPEC, i)), xs[i]);
}

template <uint32_t SPEC, int NV>
__device__ __forceinline__ void spec_apply(uint64_t* f, bool leader, int space, unsigned peers, const PeerPlan& pp,
                                           const bool (&vv)[8], const uint64_t (&vb)[8]) {
  uint64_t xs[8];
  xs[0] = static_cast<uint64_t>(__popc(peers));
#pragma unroll
  for (int i = 1; i <= spec_n(SPEC); ++i) {
    const int kind = spec_kind(SPEC, i);
    const int col = spec_col(SPEC, i) < NV ? spec_col(SPEC, i) : 0;
    xs[i] = 0;
    if (kind != 0) {
      const uint64_t x = field_contrib(static_cast<uint8_t>(kind), vv[col], vb[col]);
      if (field_op(static_cast<uint8_t>(kind)) == kOpAdd) xs[i] = peer_reduce_op<kOpAdd>(x, pp);
      else if (field_op(static_cast<uint8_t>(kind)) == kOpFAdd) xs[i] = peer_reduce_op<kOpFAdd>(x, pp);
      else xs[i] = peer_reduce_op<kOpMax>(x, pp);
    }
  }
  if (!leader) return;
  if (space == kRowPrivate) {
    field_red<kRowPrivate>(f, F_ROWS, xs[0]);
    spec_merge<SPEC, kRowPrivate>(f, xs);
  } else if (space == kRowShared) {
    field_red<kRowShared>(f, F_ROWS, xs[0]);
    spec_merge<SPEC, kRowShared>(f, xs);
  } else {
    field_red<kRowGlobal>(f, F_ROWS, xs[0]);
    spec_merge<SPEC, kRowGlobal>(f, xs);
  }
}

}  // namespace qeg
