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

// The contribution of one (valid, value bits) input to a field, in the
// field's identity-is-zero encoding.
__device__ __forceinline__ uint64_t field_contrib(uint8_t kind, bool valid, uint64_t bits) {
  switch (kind) {
    case F_ROWS: return 1;
    case F_NULLS: return valid ? 0 : 1;
    case F_SUMI:
    case F_SUMF: return valid ? bits : 0;
    case F_MINI: return valid ? ~enc_i64(static_cast<int64_t>(bits)) : 0;
    case F_MAXI: return valid ? enc_i64(static_cast<int64_t>(bits)) : 0;
    case F_MINF: return valid ? ~enc_f64_bits(bits) : 0;
    case F_MAXF: return valid ? enc_f64_bits(bits) : 0;
    default: return 0;
  }
}

__device__ __forceinline__ uint64_t field_combine(uint8_t kind, uint64_t a, uint64_t b) {
  switch (kind) {
    case F_ROWS:
    case F_NULLS:
    case F_SUMI: return a + b;
    case F_SUMF:
      return static_cast<uint64_t>(__double_as_longlong(__longlong_as_double(static_cast<long long>(a)) +
                                                        __longlong_as_double(static_cast<long long>(b))));
    default: return a > b ? a : b;
  }
}

// Merges one combined contribution into a table word (shared or global).
__device__ __forceinline__ void field_apply(uint64_t* w, uint8_t kind, uint64_t x) {
  unsigned long long* u = reinterpret_cast<unsigned long long*>(w);
  switch (kind) {
    case F_ROWS:
    case F_NULLS:
    case F_SUMI:
      if (x) atomicAdd(u, static_cast<unsigned long long>(x));
      break;
    case F_SUMF:
      if (x) atomicAdd(reinterpret_cast<double*>(w), __longlong_as_double(static_cast<long long>(x)));
      break;
    default:
      if (x) atomicMax(u, static_cast<unsigned long long>(x));
      break;
  }
}

__device__ __forceinline__ uint64_t peer_reduce(uint64_t x, uint8_t kind, const PeerPlan& pp) {
  for (int r = 0; r < pp.rounds; ++r) {
    const uint64_t t = __shfl_sync(0xffffffffu, x, (pp.src >> (5 * r)) & 31u);
    if ((pp.take >> r) & 1u) x = field_combine(kind, x, t);
  }
  return x;
}

}  // namespace qeg
