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
    auto host_copy = [&](const void* src, size_t bytes) {
      std::vector<uint8_t> h(bytes);
      if (bytes) {
        if (is_device_ptr(src)) {
          QEG_CUDA(cudaMemcpy(h.data(), src, bytes, cudaMemcpyDeviceToHost));
        } else {
          std::memcpy(h.data(), src, bytes);
        }
      }
      return h;
    };
    auto valid_at = [](const std::vector<uint8_t>& words, bool all_valid, uint64_t i) {
      if (all_valid) return true;
      uint64_t w;
      std::memcpy(&w, words.data() + (i >> 6) * 8, 8);
      return ((w >> (i & 63)) & 1ull) != 0;
    };
    auto ival = [](const std::vector<uint8_t>& v, int32_t t, uint64_t i) -> int64_t {
      if (t == QEG_I32 || t == QEG_STR) {
        int32_t x;
        std::memcpy(&x, v.data() + i * 4, 4);
        return x;
      }
      if (t == QEG_BOOL) return v[i];
      int64_t x;
      std::memcpy(&x, v.data() + i * 8, 8);
      return x;
    };
    const qeg_column& bk = build[d->build_key];
    const qeg_column& gcol = build[d->group_col - nprobe];
    const auto bkv = host_copy(bk.data, nb * type_width(bk.type));
    const bool bk_all = bk.all_valid || !bk.validity;
    const auto bkw = bk_all ? std::vector<uint8_t>() : host_copy(bk.validity, ((nb + 63) / 64) * 8);
    const auto gv = host_copy(gcol.data, nb * type_width(gcol.type));
    const bool g_all = gcol.all_valid || !gcol.validity;
    const auto gw = g_all ? std::vector<uint8_t>() : host_copy(gcol.validity, ((nb + 63) / 64) * 8);
    // Group ids over the distinct group values of build rows (NULL is a group).
    std::unordered_map<uint64_t, uint32_t> gid;
    std::vector<uint64_t> gword;  // canonical group word per group
    std::vector<uint8_t> gnull;
    int32_t null_gid = -1;
    std::vector<int32_t> row_group(nb, -1);
    std::vector<uint8_t> gcm;
    if (gcol.type == QEG_STR) {
      require(gcol.code_map != nullptr, "STR group column needs a code map");
      gcm = host_copy(gcol.code_map, gcol.code_map_len * 4);
    }
    for (uint64_t b = 0; b < nb; ++b) {
      if (!valid_at(gw, g_all, b)) {
        if (null_gid < 0) {
          null_gid = static_cast<int32_t>(gword.size());
          gword.push_back(0);
          gnull.push_back(1);
        }
        row_group[b] = null_gid;
        continue;
      }
      uint64_t w;
      if (gcol.type == QEG_F64) {
        double x;
        std::memcpy(&x, gv.data() + b * 8, 8);
        uint64_t bits;
        std::memcpy(&bits, &x, 8);
        if (std::isnan(x)) bits = kCanonNaN;
        else if (x == 0.0) bits = 0;
        w = bits;
      } else if (gcol.type == QEG_STR) {
        const int32_t code = static_cast<int32_t>(ival(gv, QEG_STR, b));
        require(code >= 0 && static_cast<uint64_t>(code) < gcol.code_map_len, "STR code outside its code map");
        int32_t id;
        std::memcpy(&id, gcm.data() + static_cast<size_t>(code) * 4, 4);
        w = static_cast<uint64_t>(static_cast<int64_t>(id));
      } else {
        w = static_cast<uint64_t>(ival(gv, gcol.type, b));
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
      require(bk.code_map && probe[d->probe_key].code_map, "STR join keys need code maps");
      const auto b = host_copy(bk.code_map, bk.code_map_len * 4);
      const auto p = host_copy(probe[d->probe_key].code_map, probe[d->probe_key].code_map_len * 4);
      bmap.resize(bk.code_map_len);
      pmap.resize(probe[d->probe_key].code_map_len);
      std::memcpy(bmap.data(), b.data(), b.size());
      std::memcpy(pmap.data(), p.data(), p.size());
    }
    // (join value, group id) of every build row with a non-NULL key.
    std::vector<int64_t> bval;
    std::vector<uint32_t> bgrp;
    bval.reserve(nb);
    bgrp.reserve(nb);
    int64_t vmin = INT64_MAX, vmax = INT64_MIN;
    for (uint64_t b = 0; b < nb; ++b) {
      if (!valid_at(bkw, bk_all, b)) continue;
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
    DevBuf dk(kstart.size() * 4, ctx->stream), dc(kcount.size() * 4, ctx->stream),
        dg(std::max<size_t>(glist.size(), 1) * 4, ctx->stream),
        dstate(static_cast<size_t>(P.ngroups) * P.nfields * 8, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(dk.get(), kstart.data(), kstart.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    QEG_CUDA(cudaMemcpyAsync(dc.get(), kcount.data(), kcount.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (!glist.empty())
      QEG_CUDA(cudaMemcpyAsync(dg.get(), glist.data(), glist.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    QEG_CUDA(cudaMemsetAsync(dstate.get(), 0, dstate.bytes(), ctx->stream));
    P.kstart = dk.get<uint32_t>();
    P.kcount = dc.get<uint32_t>();
    P.glist = dg.get<uint32_t>();
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
    if (sb > 48 * 1024)
      QEG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
    int per_sm = 1;
    QEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, sb));
    const uint64_t want = (np + block * 16 - 1) / (block * 16);
    const unsigned grid = static_cast<unsigned>(
        std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(ctx->sms) * std::max(per_sm, 1))));
    if (np > 0 && domain > 0 && ngroups > 0) {
      kern<<<grid, block, sb, ctx->stream>>>(P);
      ctx->launches++;
      QEG_CUDA(cudaGetLastError());
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
