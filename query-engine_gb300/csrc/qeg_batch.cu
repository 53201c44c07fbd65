// qeg_batch.cu -- many independent GROUP BY queries in one persistent kernel.
//
// The reference answers each query with its own Aggregate tree
// (ops/aggregate.cpp; exec/parallel.cpp runs one plan at a time). Here a batch
// of queries -- each a key column and a value column, stored back to back --
// is planned once and then executed by replaying a captured CUDA graph:
//   plan   : per query, a sketch of its keys and the learned estimator give
//            the expected group count and heavy-hitter share; a tuning table
//            (filled by the autotuner per (group-count, skew) bucket) gives the
//            strategy (CTA-private shared-memory table or global table only)
//            and the rows per work item. Tables of all queries live in one
//            arena, sized from the estimates.
//   run    : a persistent kernel pulls (query, row range) work items from an
//            atomic counter -- uneven query sizes balance themselves -- and
//            aggregates each item into its query's table; a finalize kernel
//            (one block per query) compacts every table into the output arena
//            and clears it for the next replay.
// A query whose table overflowed (its estimate was far too low) is re-run
// exactly through the ordinary GROUP BY path, so results never depend on the
// estimates.
#include <algorithm>
#include <cmath>

#include "qeg_agg.h"
#include "qeg_mlp.h"
#include "qeg_warpagg.cuh"

namespace qeg {

namespace {

constexpr int kBatchMaxSlots = 4096;
// COUNT(*), SUM, AVG, MIN, MAX over an F64 value column, without and with its
// NULL count (qeg_warpagg.cuh field-set codes).
constexpr uint32_t kBatchSpecF64 = 4u | spec_field(1, 0, 0) | spec_field(2, F_SUMF, 0) | spec_field(3, F_MINF, 0) |
                                   spec_field(4, F_MAXF, 0);
constexpr uint32_t kBatchSpecF64Nulls = 4u | spec_field(1, F_NULLS, 0) | spec_field(2, F_SUMF, 0) |
                                        spec_field(3, F_MINF, 0) | spec_field(4, F_MAXF, 0);

struct BatchQ {
  uint64_t table_off;  // first row of the query's table in the arena
  uint64_t cap;        // hash slots (+2 side rows follow)
  uint64_t out_off;    // first output row
  int32_t smem;        // 1: CTA-private shared-memory table first
  int32_t smem_slots;  // power of two <= kBatchMaxSlots
  int32_t peer;        // 1: lanes of a warp combine rows of one group first
  int32_t pad;
};

struct BatchK {
  DevCol key, val;
  const BatchQ* qs;
  const uint32_t* item_q;
  const uint64_t* item_start;
  const uint32_t* item_len;
  uint32_t nitems;
  unsigned int* next;
  uint64_t* arena;
  int W;  // words per row: key + fields
  int nfields;
  uint8_t fkind[kMaxFields];
  int val_first, val_nf;  // value-column fields (cfirst/cnf of column 0)
  uint32_t* overflow;     // per query
};

__device__ __forceinline__ uint64_t* batch_global_row(const BatchK& P, const BatchQ& Q, bool kv, uint64_t k) {
  uint64_t* T = P.arena + Q.table_off * P.W;
  if (!kv) return T + (Q.cap + 1) * P.W;
  if (k == 0) return T + Q.cap * P.W;
  // Linear probing: the home slot alone, then four slots per step whose key
  // words are loaded together (see global_row1 in qeg_agg.cu).
  uint64_t s = __umul64hi(hash_fold(kHashSeed, k), Q.cap);
  for (int t = 0; t < 128;) {
    const int width = t == 0 ? 1 : 4;
    uint64_t idx[4];
    unsigned long long cur[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < width) {
        uint64_t x = s + j;
        if (x >= Q.cap) x -= Q.cap;
        idx[j] = x;
        cur[j] = *reinterpret_cast<volatile unsigned long long*>(T + x * P.W);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < width) {
        uint64_t* r = T + idx[j] * P.W;
        if (cur[j] == k) return r;
        if (cur[j] == 0) {
          const unsigned long long old =
              atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, static_cast<unsigned long long>(k));
          if (old == 0 || old == k) return r;
        }
      }
    }
    t += width;
    s += width;
    if (s >= Q.cap) s -= Q.cap;
  }
  return nullptr;
}

// SPEC: the value fields' set (qeg_warpagg.cuh), or kGenericSpec.
template <uint32_t SPEC>
__global__ void __launch_bounds__(1024) batch_agg_kernel(const BatchK P) {
  extern __shared__ uint64_t sm[];
  const int SW = P.W | 1;  // odd row stride in shared memory: fewer bank conflicts
  __shared__ uint32_t s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(P.next, 1u);
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= P.nitems) break;
    const uint32_t q = P.item_q[item];
    const BatchQ Q = P.qs[q];
    const int S = Q.smem ? Q.smem_slots : 0;
    if (S) {
      for (int i = threadIdx.x; i < (S + 2) * SW; i += blockDim.x) sm[i] = 0;
      __syncthreads();
    }
    const uint64_t start = P.item_start[item];
    const uint32_t len = P.item_len[item];
    bool ovf = false;
    const unsigned lane = threadIdx.x & 31u;
    // Warps walk the item 32 rows at a time. With Q.peer, lanes of one group
    // combine their rows first (warp peer aggregation) and the group's leader
    // applies them; otherwise every lane applies its own row.
    for (uint32_t wb = threadIdx.x & ~31u; wb < len; wb += blockDim.x) {
      const uint32_t i = wb + lane;
      const bool live = i < len;
      const uint64_t p = start + i;
      const bool kv = live && col_valid(P.key, p);
      const uint64_t k = kv ? key_word(P.key, p) : 0;
      const bool v = live && col_valid(P.val, p);
      const uint64_t b = !v ? 0
                         : (P.val.type == kF64 ? static_cast<uint64_t>(__double_as_longlong(f64_value(P.val, p)))
                                               : static_cast<uint64_t>(int_value(P.val, p)));
      unsigned peers = 1u << lane;
      if (Q.peer) {
        const unsigned livemask = __ballot_sync(0xffffffffu, live);
        const unsigned same = match_word64(k, lane, P.key.type == kI32 || P.key.type == kSTR || P.key.type == kBOOL);
        const unsigned vmask = __ballot_sync(0xffffffffu, kv);
        if (live) peers = same & livemask & (kv ? vmask : ~vmask);
      }
      const bool leader = live && __ffs(peers) - 1 == static_cast<int>(lane);
      uint64_t* f = nullptr;
      int space = kRowGlobal;
      if (leader) {
        int srow = -1;
        if (S) {
          if (!kv) {
            srow = S + 1;
          } else if (k == 0) {
            srow = S;
          } else {
            uint64_t s = hash_fold(kHashSeed, k) & (S - 1);
            for (int t = 0; t < 8; ++t) {
              unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&sm[s * SW]);
              if (cur == 0)
                cur = atomicCAS(reinterpret_cast<unsigned long long*>(&sm[s * SW]), 0ull,
                                static_cast<unsigned long long>(k));
              if (cur == 0 || cur == k) {
                srow = static_cast<int>(s);
                break;
              }
              s = (s + 1) & (S - 1);
            }
          }
        }
        if (srow >= 0) {
          f = &sm[srow * SW + 1];
          space = kRowShared;
        } else {
          uint64_t* r = batch_global_row(P, Q, kv, k);
          if (r) f = r + 1;
          else ovf = true;  // the query is recomputed exactly after the run
        }
      }
      const PeerPlan pp = plan_peers(peers, lane);
      const bool apply = leader && f != nullptr;
      if constexpr (SPEC != kGenericSpec) {
        bool vv[8] = {v};
        uint64_t vb[8] = {b};
        spec_apply<SPEC, 1>(f, apply, space, peers, pp, vv, vb);
      } else {
        if (apply) field_red_at(space, f, F_ROWS, static_cast<uint64_t>(__popc(peers)));
        for (int j = 0; j < P.val_nf; ++j) {
          const uint8_t kind = P.fkind[P.val_first + j];
          const uint64_t x = peer_reduce(field_contrib(kind, v, b), kind, pp);
          if (apply) field_red_at(space, f + P.val_first + j, kind, x);
        }
      }
    }
    if (ovf) atomicOr(P.overflow + q, 1u);
    if (S) {
      __syncthreads();
      for (int sr = threadIdx.x; sr < S + 2; sr += blockDim.x) {
        const uint64_t* src = &sm[sr * SW];
        if (src[1] == 0) continue;
        uint64_t* dst;
        if (sr == S + 1) dst = batch_global_row(P, Q, false, 0);
        else if (sr == S) dst = batch_global_row(P, Q, true, 0);
        else dst = batch_global_row(P, Q, true, src[0]);
        if (!dst) {
          atomicOr(P.overflow + q, 1u);
          continue;
        }
        for (int f = 0; f < P.nfields; ++f) {
          const uint64_t x = src[1 + f];
          if (!x) continue;
          unsigned long long* d = reinterpret_cast<unsigned long long*>(dst + 1 + f);
          const uint8_t kind = P.fkind[f];
          if (kind == F_SUMF) atomicAdd(reinterpret_cast<double*>(d), __longlong_as_double(static_cast<long long>(x)));
          else if (kind >= F_MINI) atomicMax(d, static_cast<unsigned long long>(x));
          else atomicAdd(d, static_cast<unsigned long long>(x));
        }
      }
    }
    __syncthreads();
  }
}

struct BatchFinK {
  const BatchQ* qs;
  const uint32_t* fin_q;      // per block: query
  const uint64_t* fin_start;  // per block: first table row
  const uint32_t* fin_len;    // per block: table rows
  uint64_t* arena;
  int W;
  int32_t key_type;
  FinK F;  // output columns (arena-wide) and aggregate finalisation
  uint8_t fkind[kMaxFields];
  unsigned long long* counts;  // per query output rows (zeroed before the launch)
};

__device__ __forceinline__ void put_typed(void* base, uint64_t i, int32_t t, uint64_t w) {
  switch (t) {
    case kI32:
    case kSTR: static_cast<int32_t*>(base)[i] = static_cast<int32_t>(static_cast<uint32_t>(w)); break;
    case kBOOL: static_cast<uint8_t*>(base)[i] = static_cast<uint8_t>(w & 1ull); break;
    default: static_cast<uint64_t*>(base)[i] = w; break;
  }
}

// Each block compacts one range of one query's table (hash slots, then the
// key-0 and NULL side rows) into that query's output rows (keys then
// aggregates, ops/agg_internal.h:169-229), reserving output rows with one
// atomic per warp, and zeroes every row it read, leaving the arena ready for
// the next replay.
__global__ void batch_finalize_kernel(const BatchFinK P) {
  const uint32_t q = P.fin_q[blockIdx.x];
  const BatchQ Q = P.qs[q];
  uint64_t* T = P.arena + Q.table_off * P.W;
  const uint64_t first = P.fin_start[blockIdx.x];
  const uint64_t total = first + P.fin_len[blockIdx.x];
  const int lane = threadIdx.x & 31;
  for (uint64_t base = first; base < total; base += blockDim.x) {
    const uint64_t s = base + threadIdx.x;
    bool occ = false;
    uint64_t* r = nullptr;
    if (s < total) {
      r = T + s * P.W;
      occ = (s < Q.cap) ? (r[0] != 0) : (r[1] != 0);
    }
    const unsigned m = __ballot_sync(0xffffffffu, occ);
    unsigned long long wb = 0;
    if (lane == 0 && m) wb = atomicAdd(P.counts + q, static_cast<unsigned long long>(__popc(m)));
    wb = __shfl_sync(0xffffffffu, wb, 0);
    if (occ) {
      const uint64_t o = Q.out_off + wb + __popc(m & ((1u << lane) - 1u));
      const bool knull = (s == Q.cap + 1);
      P.F.valid[0][o] = knull ? 0 : 1;
      put_typed(P.F.vals[0], o, P.key_type, knull || s == Q.cap ? 0 : r[0]);
      const uint64_t* f = r + 1;
      const uint64_t rows = f[0];
      for (int a = 0; a < P.F.naggs; ++a) {
        const int vf = P.F.vfield[a];
        const uint64_t nn = rows - (P.F.nfield[a] >= 0 ? f[P.F.nfield[a]] : 0);
        uint8_t ok = 1;
        uint64_t w = 0;
        switch (P.F.func[a]) {
          case 0: w = rows; break;
          case 1: w = nn; break;
          case 2:
            if (nn == 0) ok = 0;
            else w = f[vf];
            break;
          case 5:
            if (nn == 0) {
              ok = 0;
            } else {
              const double sum = P.fkind[vf] == F_SUMF ? __longlong_as_double(static_cast<long long>(f[vf]))
                                                        : static_cast<double>(static_cast<int64_t>(f[vf]));
              w = static_cast<uint64_t>(__double_as_longlong(sum / static_cast<double>(nn)));
            }
            break;
          default: {
            if (nn == 0) {
              ok = 0;
              break;
            }
            const uint8_t k = P.fkind[vf];
            const uint64_t e = f[vf];
            if (k == F_MINF) w = dec_f64_bits(~e);
            else if (k == F_MAXF) w = dec_f64_bits(e);
            else if (k == F_MINI) w = static_cast<uint64_t>(dec_i64(~e));
            else w = static_cast<uint64_t>(dec_i64(e));
          }
        }
        P.F.valid[1 + a][o] = ok;
        put_typed(P.F.vals[1 + a], o, P.F.rtype[1 + a], ok ? w : 0);
      }
    }
    if (s < total && (occ || s >= Q.cap))
      for (int w = 0; w < P.W; ++w) r[w] = 0;
  }
}

uint64_t pow2_floor(uint64_t v) {
  uint64_t c = 1;
  while (c * 2 <= v) c *= 2;
  return c;
}

}  // namespace

// One execution round: a set of queries with their tables in one arena, the
// work items of the persistent kernel and the finalize ranges. The first
// round holds every query and is captured into a CUDA graph; queries whose
// table overflowed are re-run together in a further round with larger tables.
struct Round {
  std::vector<uint32_t> qids;  // batch query id of each local query
  std::vector<BatchQ> qs;
  uint32_t nitems = 0, nfin = 0;
  int32_t max_slots = 0;  // largest CTA-private table of the round (sizes the shared memory)
  DevBuf dqs, ditem_q, ditem_start, ditem_len, dfin_q, dfin_start, dfin_len, dnext, arena, overflow, counts;
  std::vector<DevBuf> out_vals, out_valid;
};

constexpr uint32_t kFinRows = 1u << 16;  // table rows per finalize block

struct BatchState {
  qeg_ctx* ctx = nullptr;
  AggState plan;  // field layout of [key, value] with the batch's aggregates
  std::vector<uint64_t> offsets;
  std::vector<double> est;
  std::vector<float> hot;
  std::vector<int32_t> slots;   // per query: CTA-private table slots (0 = global table only)
  std::vector<uint64_t> chunk;  // per query: rows per work item
  std::vector<int32_t> peer;    // per query: warp peer aggregation
  StagedCol key, val;
  uint32_t nq = 0;
  int block = 512;
  DevBuf doffs;
  std::vector<Round> rounds;  // [0] = every query; later rounds = overflow re-runs
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> group_counts;
  std::vector<uint32_t> where_round, where_local;  // result location of each query
  std::vector<uint32_t> fell_back;
  // Queries still overflowing after the re-run rounds: recomputed exactly.
  std::vector<std::unique_ptr<AggState>> fallback;

  ~BatchState() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }

  uint64_t rows_of(uint32_t q) const { return offsets[q + 1] - offsets[q]; }

  // Lays out round R over `qids` with table capacities `caps`.
  void setup_round(Round& R, const std::vector<uint32_t>& qids, const std::vector<uint64_t>& caps) {
    R.qids = qids;
    const uint32_t n = static_cast<uint32_t>(qids.size());
    R.qs.assign(n, BatchQ{});
    R.max_slots = 0;
    std::vector<uint32_t> iq, il, fq, fl;
    std::vector<uint64_t> is, fs;
    uint64_t table_rows = 0;
    for (uint32_t l = 0; l < n; ++l) {
      const uint32_t q = qids[l];
      const uint64_t cap = caps[l];
      R.qs[l] = BatchQ{table_rows, cap, table_rows, slots[q] > 0 ? 1 : 0, std::max(slots[q], 64), peer[q], 0};
      R.max_slots = std::max(R.max_slots, slots[q]);
      table_rows += cap + 2;
      const uint64_t rows = rows_of(q);
      for (uint64_t s0 = 0; s0 < rows; s0 += chunk[q]) {
        iq.push_back(l);
        is.push_back(offsets[q] + s0);
        il.push_back(static_cast<uint32_t>(std::min<uint64_t>(chunk[q], rows - s0)));
      }
      for (uint64_t s0 = 0; s0 < cap + 2; s0 += kFinRows) {
        fq.push_back(l);
        fs.push_back(s0);
        fl.push_back(static_cast<uint32_t>(std::min<uint64_t>(kFinRows, cap + 2 - s0)));
      }
    }
    R.nitems = static_cast<uint32_t>(iq.size());
    R.nfin = static_cast<uint32_t>(fq.size());
    // Longest items first, so the tail of the queue holds only small ones.
    std::vector<uint32_t> order(R.nitems);
    for (uint32_t i = 0; i < R.nitems; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return il[a] > il[b]; });
    std::vector<uint32_t> oq(R.nitems), ol(R.nitems);
    std::vector<uint64_t> os(R.nitems);
    for (uint32_t i = 0; i < R.nitems; ++i) {
      oq[i] = iq[order[i]];
      ol[i] = il[order[i]];
      os[i] = is[order[i]];
    }
    auto up = [&](DevBuf& d, const void* src, size_t bytes) {
      d.alloc(std::max<size_t>(bytes, 8), ctx->stream);
      if (bytes) QEG_CUDA(cudaMemcpyAsync(d.get(), src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    };
    up(R.dqs, R.qs.data(), R.qs.size() * sizeof(BatchQ));
    up(R.ditem_q, oq.data(), oq.size() * 4);
    up(R.ditem_start, os.data(), os.size() * 8);
    up(R.ditem_len, ol.data(), ol.size() * 4);
    up(R.dfin_q, fq.data(), fq.size() * 4);
    up(R.dfin_start, fs.data(), fs.size() * 8);
    up(R.dfin_len, fl.data(), fl.size() * 4);
    R.dnext.alloc(8, ctx->stream);
    R.arena.alloc(std::max<uint64_t>(table_rows, 1) * plan.row_words * 8, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(R.arena.get(), 0, R.arena.bytes(), ctx->stream));
    R.overflow.alloc(std::max<uint32_t>(n, 1) * 4, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(R.overflow.get(), 0, R.overflow.bytes(), ctx->stream));
    R.counts.alloc(std::max<uint32_t>(n, 1) * 8, ctx->stream);
    R.out_vals.resize(plan.rtypes.size());
    R.out_valid.resize(plan.rtypes.size());
    for (size_t c = 0; c < plan.rtypes.size(); ++c) {
      R.out_vals[c].alloc(std::max<uint64_t>(table_rows, 1) * 8, ctx->stream);
      R.out_valid[c].alloc(std::max<uint64_t>(table_rows, 1), ctx->stream);
    }
  }

  BatchK kparams(Round& R) {
    BatchK P{};
    P.key = key.dev;
    P.val = val.dev;
    P.qs = R.dqs.get<BatchQ>();
    P.item_q = R.ditem_q.get<uint32_t>();
    P.item_start = R.ditem_start.get<uint64_t>();
    P.item_len = R.ditem_len.get<uint32_t>();
    P.nitems = R.nitems;
    P.next = R.dnext.get<unsigned int>();
    P.arena = R.arena.get<uint64_t>();
    P.W = plan.row_words;
    P.nfields = plan.nfields;
    for (int f = 0; f < plan.nfields; ++f) P.fkind[f] = plan.fkind[f];
    P.val_first = plan.cfirst.empty() ? 0 : plan.cfirst[0];
    P.val_nf = plan.cnf.empty() ? 0 : plan.cnf[0];
    P.overflow = R.overflow.get<uint32_t>();
    return P;
  }

  BatchFinK finparams(Round& R) {
    BatchFinK F{};
    F.qs = R.dqs.get<BatchQ>();
    F.fin_q = R.dfin_q.get<uint32_t>();
    F.fin_start = R.dfin_start.get<uint64_t>();
    F.fin_len = R.dfin_len.get<uint32_t>();
    F.arena = R.arena.get<uint64_t>();
    F.W = plan.row_words;
    F.key_type = plan.rtypes[0];
    F.F.naggs = static_cast<int>(plan.aggs.size());
    for (size_t c = 0; c < plan.rtypes.size(); ++c) {
      F.F.vals[c] = R.out_vals[c].get();
      F.F.valid[c] = R.out_valid[c].get<uint8_t>();
      F.F.rtype[c] = plan.rtypes[c];
    }
    for (size_t a = 0; a < plan.aggs.size(); ++a) {
      F.F.func[a] = plan.aggs[a].func;
      F.F.vfield[a] = plan.vfield[a];
      F.F.nfield[a] = plan.nfield[a];
    }
    for (int f = 0; f < plan.nfields; ++f) F.fkind[f] = plan.fkind[f];
    F.counts = R.counts.get<unsigned long long>();
    return F;
  }

  // The batch kernel for this plan's field set: COUNT/SUM/AVG/MIN/MAX over
  // one value column (with or without its NULL count) has its own kernel.
  void (*agg_kernel_for() const)(BatchK) {
    const int n = plan.nfields - 1;
    if (n > 7) return batch_agg_kernel<kGenericSpec>;
    uint32_t spec = static_cast<uint32_t>(n);
    for (int i = 1; i <= n; ++i) {
      int kind = plan.fkind[i];
      if (kind == F_NULLS && val.dev.all_valid) kind = 0;
      spec |= spec_field(i, kind, 0);
    }
    if (spec == kBatchSpecF64) return batch_agg_kernel<kBatchSpecF64>;
    if (spec == kBatchSpecF64Nulls) return batch_agg_kernel<kBatchSpecF64Nulls>;
    return batch_agg_kernel<kGenericSpec>;
  }

  size_t smem_bytes(int32_t max_slots) const { return static_cast<size_t>(max_slots + 2) * (plan.row_words | 1) * 8; }

  void enqueue(Round& R) {
    QEG_CUDA(cudaMemsetAsync(R.dnext.get(), 0, 4, ctx->stream));
    QEG_CUDA(cudaMemsetAsync(R.counts.get(), 0, R.counts.bytes(), ctx->stream));
    const size_t sb = smem_bytes(R.max_slots);
    int per_sm = 1;
    void (*kern)(BatchK) = agg_kernel_for();
    QEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, sb));
    const unsigned grid = static_cast<unsigned>(
        std::max(1, std::min<int>(ctx->sms * std::max(per_sm, 1), static_cast<int>(std::max<uint32_t>(R.nitems, 1)))));
    kern<<<grid, block, sb, ctx->stream>>>(kparams(R));
    if (R.nfin) batch_finalize_kernel<<<R.nfin, 512, 0, ctx->stream>>>(finparams(R));
  }

  // Reads the overflow flags and counts of round r into the per-query results.
  std::vector<uint32_t> collect(uint32_t r) {
    Round& R = rounds[r];
    const size_t n = R.qids.size();
    std::vector<uint32_t> ovf(n);
    std::vector<uint64_t> cnt(n);
    if (n) {
      QEG_CUDA(cudaMemcpyAsync(ovf.data(), R.overflow.get(), n * 4, cudaMemcpyDeviceToHost, ctx->stream));
      QEG_CUDA(cudaMemcpyAsync(cnt.data(), R.counts.get(), n * 8, cudaMemcpyDeviceToHost, ctx->stream));
      QEG_CUDA(cudaMemsetAsync(R.overflow.get(), 0, n * 4, ctx->stream));
    }
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    check_device_error(ctx);
    std::vector<uint32_t> again;
    for (size_t l = 0; l < n; ++l) {
      const uint32_t q = R.qids[l];
      if (ovf[l]) {
        again.push_back(static_cast<uint32_t>(l));
        continue;
      }
      group_counts[q] = cnt[l];
      where_round[q] = r;
      where_local[q] = static_cast<uint32_t>(l);
    }
    return again;
  }
};

}  // namespace qeg

using namespace qeg;

struct qeg_batch {
  BatchState st;
};

extern "C" {

qeg_status qeg_batch_create(qeg_ctx* ctx, uint32_t nqueries, const uint64_t* row_offsets, const qeg_column* key,
                            const qeg_column* val, const qeg_agg_spec* aggs, int naggs, const qeg_batch_tuning* tuning,
                            int ntuning, int block_threads, qeg_batch** out) {
  return guarded(ctx, [&] {
    require(ctx && row_offsets && key && val && aggs && out, "NULL argument");
    require(nqueries >= 1, "a batch needs >= 1 query");
    require(key->len == val->len && row_offsets[nqueries] == key->len, "row offsets must cover the columns");
    for (uint32_t q = 0; q < nqueries; ++q) require(row_offsets[q] <= row_offsets[q + 1], "row offsets must ascend");
    require(key->type != QEG_F64 && key->type != QEG_STR, "batched GROUP BY keys are integer columns");
    require(block_threads == 0 || (block_threads >= 32 && block_threads <= 1024 && block_threads % 32 == 0),
            "block_threads must be 0 or a multiple of 32 in [32, 1024]");
    QEG_CUDA(cudaSetDevice(ctx->device));
    auto b = std::make_unique<qeg_batch>();
    BatchState& S = b->st;
    S.ctx = ctx;
    S.plan.ctx = ctx;
    const int32_t types[2] = {key->type, val->type};
    const uint32_t kc = 0;
    for (int a = 0; a < naggs; ++a)
      require(aggs[a].func == QEG_COUNT_STAR || aggs[a].input_col == 1, "batch aggregates read column 1 (the value)");
    S.plan.plan(types, 2, &kc, 1, aggs, naggs);
    require(S.plan.val_cols.size() <= 1, "batch aggregates read one value column");
    S.nq = nqueries;
    S.offsets.assign(row_offsets, row_offsets + nqueries + 1);
    stage_column(ctx, *key, S.key);
    stage_column(ctx, *val, S.val);
    S.block = block_threads > 0 ? block_threads : 512;
    for (uint32_t q = 0; q < nqueries; ++q)
      require((S.key.dev.all_valid && S.val.dev.all_valid) || S.offsets[q] % 64 == 0,
              "queries over columns with NULLs must start on 64-row boundaries");
    // ---- plan every query: one sketch launch, one batched network pass ----
    S.doffs.alloc((nqueries + 1) * 8, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(S.doffs.get(), S.offsets.data(), (nqueries + 1) * 8, cudaMemcpyHostToDevice,
                             ctx->stream));
    std::vector<SketchResult> sk;
    batch_sketch(ctx, S.key.dev, S.doffs.get<uint64_t>(), S.offsets, 1u << 16, sk);
    std::vector<float> feats((size_t)nqueries * kSketchFeatures);
    for (uint32_t q = 0; q < nqueries; ++q)
      std::copy(sk[q].features, sk[q].features + kSketchFeatures, feats.begin() + (size_t)q * kSketchFeatures);
    const bool learned = ctx->mlp && ctx->mlp->loaded;
    std::vector<float> y;
    if (learned) {
      Mlp& m = *ctx->mlp;
      m.ensure(ctx, static_cast<int>(nqueries));
      QEG_CUDA(cudaMemcpyAsync(m.x.get(), feats.data(), feats.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
      m.forward(m.x.get<float>(), static_cast<int>(nqueries));
      y.resize((size_t)nqueries * kOut);
      QEG_CUDA(cudaMemcpyAsync(y.data(), m.y.get(), y.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
      QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    S.est.resize(nqueries);
    S.hot.resize(nqueries);
    S.slots.resize(nqueries);
    S.chunk.resize(nqueries);
    S.peer.resize(nqueries);
    std::vector<uint32_t> all(nqueries);
    std::vector<uint64_t> caps(nqueries);
    for (uint32_t q = 0; q < nqueries; ++q) {
      const uint64_t n = S.rows_of(q);
      double g = classic_estimate(sk[q]);
      double share = sk[q].top_share[11];
      if (learned) {
        g = learned_groups(sk[q], y[(size_t)q * kOut], ctx->mlp->deadband) + (sk[q].null_frac > 0 ? 1.0 : 0.0);
        g = std::max(g, sk[q].hll_estimate * 0.95);
        share = std::min(1.0, std::max(0.0, static_cast<double>(y[(size_t)q * kOut + 1])));
      }
      g = std::min(std::max(g, 1.0), static_cast<double>(std::max<uint64_t>(n, 1)));
      S.est[q] = g;
      S.hot[q] = static_cast<float>(share);
      // Built-in defaults, then the tuning table: the first entry whose bucket
      // covers this query's (log2 groups, skew class).
      int32_t sl = (g <= 0.5 * kBatchMaxSlots || share >= 0.3)
                       ? static_cast<int32_t>(std::min<uint64_t>(kBatchMaxSlots, pow2_floor(std::max(64.0, 2.0 * g))))
                       : 0;
      uint64_t ch = 1u << 16;
      // Few groups: many lanes of a warp land on the same group.
      int32_t pr = g <= 256 ? 1 : 0;
      const double lg = std::log2(std::max(g, 1.0));
      for (int t = 0; t < ntuning; ++t) {
        if (lg <= tuning[t].max_log2_groups && (share >= 0.3 ? 1 : 0) == tuning[t].skewed) {
          sl = tuning[t].smem_slots > 0
                   ? static_cast<int32_t>(pow2_floor(std::min<int32_t>(kBatchMaxSlots, std::max(64, tuning[t].smem_slots))))
                   : 0;
          if (tuning[t].rows_per_item > 0) ch = tuning[t].rows_per_item;
          if (tuning[t].peer_rows >= 0) pr = tuning[t].peer_rows ? 1 : 0;
          break;
        }
      }
      S.slots[q] = sl;
      S.chunk[q] = std::max<uint64_t>(ch, 256);
      S.peer[q] = pr;
      all[q] = q;
      caps[q] = std::max<uint64_t>(64, static_cast<uint64_t>(kEstimateHeadroom * g / kTargetLoad) + 16);
    }
    const size_t sb = S.smem_bytes(kBatchMaxSlots);
    require(sb <= ctx->smem_optin, "batch rows are too wide for the shared-memory tables");
    raise_dynamic_smem(reinterpret_cast<const void*>(S.agg_kernel_for()), sb);
    S.rounds.resize(1);
    S.setup_round(S.rounds[0], all, caps);
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    // ---- capture the first round into a CUDA graph ----
    QEG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    S.enqueue(S.rounds[0]);
    QEG_CUDA(cudaStreamEndCapture(ctx->stream, &S.graph));
    QEG_CUDA(cudaGraphInstantiate(&S.exec, S.graph, 0));
    *out = b.release();
  });
}

qeg_status qeg_batch_run(qeg_batch* b) {
  qeg::NvtxRange nvtx_range("qeg_batch_run");
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr, "batch is NULL");
    BatchState& S = b->st;
    QEG_CUDA(cudaSetDevice(ctx->device));
    QEG_CUDA(cudaGraphLaunch(S.exec, ctx->stream));
    ctx->launches += S.rounds[0].nfin ? 2 : 1;
  });
}

qeg_status qeg_batch_finish(qeg_batch* b, uint64_t* groups) {
  qeg::NvtxRange nvtx_range("qeg_batch_finish");
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr, "batch is NULL");
    BatchState& S = b->st;
    QEG_CUDA(cudaSetDevice(ctx->device));
    S.group_counts.assign(S.nq, 0);
    S.where_round.assign(S.nq, 0);
    S.where_local.assign(S.nq, 0);
    S.fell_back.clear();
    S.fallback.clear();
    S.fallback.resize(S.nq);
    std::vector<uint32_t> again = S.collect(0);
    // Overflowed queries (their estimate was far too low) run again, together,
    // with 8x larger tables, up to the bound of one group per row.
    uint32_t r = 0;
    while (!again.empty() && r < 3) {
      const Round& prev = S.rounds[r];
      std::vector<uint32_t> qids;
      std::vector<uint64_t> caps;
      for (uint32_t l : again) {
        const uint32_t q = prev.qids[l];
        qids.push_back(q);
        const uint64_t bound = static_cast<uint64_t>(static_cast<double>(S.rows_of(q)) / kTargetLoad) + 64;
        caps.push_back(std::min<uint64_t>(8 * prev.qs[l].cap, bound));
        S.fell_back.push_back(q);
      }
      ++r;
      if (S.rounds.size() <= r) S.rounds.resize(r + 1);
      Round& R = S.rounds[r];
      if (R.qids != qids) S.setup_round(R, qids, caps);
      S.enqueue(R);
      ctx->launches += R.nfin ? 2 : 1;
      again = S.collect(r);
    }
    // Still overflowing (not expected: the last tables hold one group per row
    // at the target load): recompute exactly through the GROUP BY path.
    for (uint32_t l : again) {
      const uint32_t q = S.rounds[r].qids[l];
      auto a = std::make_unique<AggState>();
      a->ctx = ctx;
      a->cfg.sizing = QEG_SIZE_FIXED;
      a->cfg.initial_capacity = 2 * S.rounds[r].qs[l].cap;
      const int32_t types[2] = {S.key.dev.type, S.val.dev.type};
      const uint32_t kc = 0;
      a->plan(types, 2, &kc, 1, S.plan.aggs.data(), static_cast<int>(S.plan.aggs.size()));
      qeg_column cols[2];
      const uint64_t off = S.offsets[q], n = S.rows_of(q);
      const DevCol* dv[2] = {&S.key.dev, &S.val.dev};
      for (int c = 0; c < 2; ++c) {
        const size_t w = type_width(dv[c]->type);
        cols[c] = qeg_column{dv[c]->type, dv[c]->all_valid, n, static_cast<const uint8_t*>(dv[c]->data) + off * w,
                             dv[c]->all_valid ? nullptr : dv[c]->validity + off / 64, nullptr, 0};
      }
      a->consume(cols, 2, nullptr, 0);
      uint64_t g = 0;
      a->finish(&g);
      S.group_counts[q] = g;
      S.fallback[q] = std::move(a);
    }
    std::sort(S.fell_back.begin(), S.fell_back.end());
    S.fell_back.erase(std::unique(S.fell_back.begin(), S.fell_back.end()), S.fell_back.end());
    if (groups) std::copy(S.group_counts.begin(), S.group_counts.end(), groups);
  });
}

qeg_status qeg_batch_fetch(qeg_batch* b, uint32_t query, const qeg_out_column* outs) {
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr && outs != nullptr, "NULL argument");
    BatchState& S = b->st;
    require(query < S.nq, "query index out of range");
    require(!S.group_counts.empty(), "fetch before qeg_batch_finish");
    QEG_CUDA(cudaSetDevice(ctx->device));
    if (S.fallback[query]) {
      S.fallback[query]->fetch(0, S.group_counts[query], outs);
      return;
    }
    Round& R = S.rounds[S.where_round[query]];
    const BatchQ& Q = R.qs[S.where_local[query]];
    for (size_t c = 0; c < S.plan.rtypes.size(); ++c)
      fetch_column(ctx, R.out_vals[c].get(), R.out_valid[c].get<uint8_t>(), type_width(S.plan.rtypes[c]),
                   Q.out_off, S.group_counts[query], outs[c]);
  });
}

qeg_status qeg_batch_stats(const qeg_batch* b, uint32_t query, double* est_groups, float* hot_share,
                           int32_t* strategy, uint32_t* fell_back) {
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr && query < b->st.nq, "bad batch or query index");
    const BatchState& S = b->st;
    if (est_groups) *est_groups = S.est[query];
    if (hot_share) *hot_share = S.hot[query];
    if (strategy) *strategy = S.slots[query] > 0 ? QEG_AGG_SMEM : QEG_AGG_GLOBAL;
    if (fell_back) *fell_back = std::binary_search(S.fell_back.begin(), S.fell_back.end(), query) ? 1 : 0;
  });
}

void qeg_batch_destroy(qeg_batch* b) {
  if (!b) return;
  cudaSetDevice(b->st.ctx->device);
  delete b;
}

}  // extern "C"
