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

struct BatchQ {
  uint64_t table_off;  // first row of the query's table in the arena
  uint64_t cap;        // hash slots (+2 side rows follow)
  uint64_t out_off;    // first output row
  int32_t smem;        // 1: CTA-private shared-memory table first
  int32_t smem_slots;  // power of two <= kBatchMaxSlots
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
  uint64_t s = __umul64hi(hash_fold(kHashSeed, k), Q.cap);
  for (int t = 0; t < 128; ++t) {
    uint64_t* r = T + s * P.W;
    unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(r);
    if (cur == k) return r;
    if (cur == 0) {
      cur = atomicCAS(reinterpret_cast<unsigned long long*>(r), 0ull, static_cast<unsigned long long>(k));
      if (cur == 0 || cur == k) return r;
    }
    s = (s + 1 == Q.cap) ? 0 : s + 1;
  }
  return nullptr;
}

__global__ void __launch_bounds__(1024) batch_agg_kernel(const BatchK P) {
  extern __shared__ uint64_t sm[];
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
      for (int i = threadIdx.x; i < (S + 2) * P.W; i += blockDim.x) sm[i] = 0;
      __syncthreads();
    }
    const uint64_t start = P.item_start[item];
    const uint32_t len = P.item_len[item];
    bool ovf = false;
    const unsigned lane = threadIdx.x & 31u;
    // Warps walk the item 32 rows at a time; lanes of one group combine their
    // rows first (warp peer aggregation) and the group's leader applies them.
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
      const unsigned livemask = __ballot_sync(0xffffffffu, live);
      const unsigned same = __match_any_sync(0xffffffffu, k);
      const unsigned vmask = __ballot_sync(0xffffffffu, kv);
      const unsigned peers = live ? (same & livemask & (kv ? vmask : ~vmask)) : (1u << lane);
      const bool leader = live && __ffs(peers) - 1 == static_cast<int>(lane);
      uint64_t* f = nullptr;
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
              unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&sm[s * P.W]);
              if (cur == 0)
                cur = atomicCAS(reinterpret_cast<unsigned long long*>(&sm[s * P.W]), 0ull,
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
          f = &sm[srow * P.W + 1];
        } else {
          uint64_t* r = batch_global_row(P, Q, kv, k);
          if (r) f = r + 1;
          else ovf = true;  // the query is recomputed exactly after the run
        }
      }
      const PeerPlan pp = plan_peers(peers, lane);
      const bool apply = leader && f != nullptr;
      if (apply) atomicAdd(reinterpret_cast<unsigned long long*>(f), static_cast<unsigned long long>(__popc(peers)));
      for (int j = 0; j < P.val_nf; ++j) {
        const uint8_t kind = P.fkind[P.val_first + j];
        const uint64_t x = peer_reduce(field_contrib(kind, v, b), kind, pp);
        if (apply) field_apply(f + P.val_first + j, kind, x);
      }
    }
    if (ovf) atomicOr(P.overflow + q, 1u);
    if (S) {
      __syncthreads();
      for (int sr = threadIdx.x; sr < S + 2; sr += blockDim.x) {
        const uint64_t* src = &sm[sr * P.W];
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
  uint64_t* arena;
  int W;
  int32_t key_type;
  FinK F;  // output columns (arena-wide) and aggregate finalisation
  uint8_t fkind[kMaxFields];
  unsigned long long* counts;  // per query output rows
};

__device__ __forceinline__ void put_typed(void* base, uint64_t i, int32_t t, uint64_t w) {
  switch (t) {
    case kI32:
    case kSTR: static_cast<int32_t*>(base)[i] = static_cast<int32_t>(static_cast<uint32_t>(w)); break;
    case kBOOL: static_cast<uint8_t*>(base)[i] = static_cast<uint8_t>(w & 1ull); break;
    default: static_cast<uint64_t*>(base)[i] = w; break;
  }
}

// One block per query: compacts the query's occupied rows into the output
// arena (keys then aggregates, ops/agg_internal.h:169-229) and zeroes every
// row it read, leaving the arena ready for the next replay.
__global__ void batch_finalize_kernel(const BatchFinK P) {
  __shared__ unsigned long long s_n;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const BatchQ Q = P.qs[blockIdx.x];
  uint64_t* T = P.arena + Q.table_off * P.W;
  const uint64_t total = Q.cap + 2;
  const int lane = threadIdx.x & 31;
  for (uint64_t base = 0; base < total; base += blockDim.x) {
    const uint64_t s = base + threadIdx.x;
    bool occ = false;
    uint64_t* r = nullptr;
    if (s < total) {
      r = T + s * P.W;
      occ = (s < Q.cap) ? (r[0] != 0) : (r[1] != 0);
    }
    const unsigned m = __ballot_sync(0xffffffffu, occ);
    unsigned long long wb = 0;
    if (lane == 0 && m) wb = atomicAdd(&s_n, static_cast<unsigned long long>(__popc(m)));
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
  __syncthreads();
  if (threadIdx.x == 0) P.counts[blockIdx.x] = s_n;
}

uint64_t pow2_floor(uint64_t v) {
  uint64_t c = 1;
  while (c * 2 <= v) c *= 2;
  return c;
}

}  // namespace

struct BatchState {
  qeg_ctx* ctx = nullptr;
  AggState plan;  // field layout of [key, value] with the batch's aggregates
  std::vector<uint64_t> offsets;
  std::vector<BatchQ> qs;
  std::vector<double> est;
  std::vector<float> hot;
  StagedCol key, val;
  uint32_t nq = 0, nitems = 0;
  int block = 512;
  DevBuf doffs, dqs, ditem_q, ditem_start, ditem_len, dnext, arena, overflow, counts;
  std::vector<DevBuf> out_vals, out_valid;
  uint64_t arena_rows = 0, out_rows = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> group_counts;
  std::vector<uint32_t> fell_back;
  // Results of queries re-run exactly after an overflow.
  std::vector<std::unique_ptr<AggState>> fallback;

  ~BatchState() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }

  BatchK kparams() {
    BatchK P{};
    P.key = key.dev;
    P.val = val.dev;
    P.qs = dqs.get<BatchQ>();
    P.item_q = ditem_q.get<uint32_t>();
    P.item_start = ditem_start.get<uint64_t>();
    P.item_len = ditem_len.get<uint32_t>();
    P.nitems = nitems;
    P.next = dnext.get<unsigned int>();
    P.arena = arena.get<uint64_t>();
    P.W = plan.row_words;
    P.nfields = plan.nfields;
    for (int f = 0; f < plan.nfields; ++f) P.fkind[f] = plan.fkind[f];
    P.val_first = plan.cfirst.empty() ? 0 : plan.cfirst[0];
    P.val_nf = plan.cnf.empty() ? 0 : plan.cnf[0];
    P.overflow = overflow.get<uint32_t>();
    return P;
  }

  BatchFinK finparams() {
    BatchFinK F{};
    F.qs = dqs.get<BatchQ>();
    F.arena = arena.get<uint64_t>();
    F.W = plan.row_words;
    F.key_type = plan.rtypes[0];
    F.F.naggs = static_cast<int>(plan.aggs.size());
    for (size_t c = 0; c < plan.rtypes.size(); ++c) {
      F.F.vals[c] = out_vals[c].get();
      F.F.valid[c] = out_valid[c].get<uint8_t>();
      F.F.rtype[c] = plan.rtypes[c];
    }
    for (size_t a = 0; a < plan.aggs.size(); ++a) {
      F.F.func[a] = plan.aggs[a].func;
      F.F.vfield[a] = plan.vfield[a];
      F.F.nfield[a] = plan.nfield[a];
    }
    for (int f = 0; f < plan.nfields; ++f) F.fkind[f] = plan.fkind[f];
    F.counts = counts.get<unsigned long long>();
    return F;
  }

  void enqueue_run() {
    QEG_CUDA(cudaMemsetAsync(dnext.get(), 0, 4, ctx->stream));
    const size_t sb = static_cast<size_t>(kBatchMaxSlots + 2) * plan.row_words * 8;
    batch_agg_kernel<<<ctx->sms * std::max(1, 2048 / block / 2), block, sb, ctx->stream>>>(kparams());
    batch_finalize_kernel<<<nq, 512, 0, ctx->stream>>>(finparams());
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
    // ---- plan every query ----
    S.qs.resize(nqueries);
    S.est.resize(nqueries);
    S.hot.resize(nqueries);
    for (uint32_t q = 0; q < nqueries; ++q)
      require((S.key.dev.all_valid && S.val.dev.all_valid) || S.offsets[q] % 64 == 0,
              "queries over columns with NULLs must start on 64-row boundaries");
    S.doffs.alloc((nqueries + 1) * 8, ctx->stream);
    QEG_CUDA(cudaMemcpyAsync(S.doffs.get(), S.offsets.data(), (nqueries + 1) * 8, cudaMemcpyHostToDevice,
                             ctx->stream));
    std::vector<SketchResult> sk;
    batch_sketch(ctx, S.key.dev, S.doffs.get<uint64_t>(), S.offsets, 1u << 16, sk);
    std::vector<float> feats((size_t)nqueries * kSketchFeatures);
    std::vector<double> classic(nqueries);
    for (uint32_t q = 0; q < nqueries; ++q) {
      std::copy(sk[q].features, sk[q].features + kSketchFeatures, feats.begin() + (size_t)q * kSketchFeatures);
      classic[q] = classic_estimate(sk[q]);
    }
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
    uint64_t table_rows = 0, out_rows = 0;
    std::vector<uint32_t> item_q, item_len;
    std::vector<uint64_t> item_start;
    for (uint32_t q = 0; q < nqueries; ++q) {
      const uint64_t n = S.offsets[q + 1] - S.offsets[q];
      double g = classic[q];
      double share = sk[q].top_share[11];
      if (learned) {
        g = learned_groups(sk[q], y[(size_t)q * kOut]) + (sk[q].null_frac > 0 ? 1.0 : 0.0);
        g = std::max(g, sk[q].hll_estimate * 0.95);
        share = std::min(1.0, std::max(0.0, static_cast<double>(y[(size_t)q * kOut + 1])));
      }
      g = std::min(std::max(g, 1.0), static_cast<double>(std::max<uint64_t>(n, 1)));
      S.est[q] = g;
      S.hot[q] = static_cast<float>(share);
      // Tuning table: the first entry whose bucket covers this query.
      int smem = g <= 0.5 * kBatchMaxSlots || share >= 0.3 ? 1 : 0;
      int slots = static_cast<int>(std::min<uint64_t>(kBatchMaxSlots, pow2_floor(std::max(64.0, 2.0 * g))));
      uint64_t chunk = 1u << 16;
      const double lg = std::log2(std::max(g, 1.0));
      for (int t = 0; t < ntuning; ++t) {
        if (lg <= tuning[t].max_log2_groups && (share >= 0.3 ? 1 : 0) == tuning[t].skewed) {
          smem = tuning[t].smem_slots > 0 ? 1 : 0;
          if (tuning[t].smem_slots > 0) slots = std::min(kBatchMaxSlots, tuning[t].smem_slots);
          chunk = tuning[t].rows_per_item;
          break;
        }
      }
      const uint64_t cap = std::max<uint64_t>(64, static_cast<uint64_t>(1.15 * g / kTargetLoad) + 16);
      S.qs[q] = BatchQ{table_rows, cap, out_rows, smem, static_cast<int32_t>(pow2_floor(slots))};
      table_rows += cap + 2;
      out_rows += cap + 2;
      for (uint64_t s0 = 0; s0 < n; s0 += chunk) {
        item_q.push_back(q);
        item_start.push_back(S.offsets[q] + s0);
        item_len.push_back(static_cast<uint32_t>(std::min<uint64_t>(chunk, n - s0)));
      }
    }
    S.nitems = static_cast<uint32_t>(item_q.size());
    S.arena_rows = table_rows;
    S.out_rows = out_rows;
    // Longest items first, so the tail of the queue holds only small ones.
    std::vector<uint32_t> order(S.nitems);
    for (uint32_t i = 0; i < S.nitems; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b2) { return item_len[a] > item_len[b2]; });
    std::vector<uint32_t> iq(S.nitems), il(S.nitems);
    std::vector<uint64_t> is(S.nitems);
    for (uint32_t i = 0; i < S.nitems; ++i) {
      iq[i] = item_q[order[i]];
      il[i] = item_len[order[i]];
      is[i] = item_start[order[i]];
    }
    auto up = [&](DevBuf& d, const void* src, size_t bytes) {
      d.alloc(std::max<size_t>(bytes, 8), ctx->stream);
      if (bytes) QEG_CUDA(cudaMemcpyAsync(d.get(), src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    };
    up(S.dqs, S.qs.data(), S.qs.size() * sizeof(BatchQ));
    up(S.ditem_q, iq.data(), iq.size() * 4);
    up(S.ditem_start, is.data(), is.size() * 8);
    up(S.ditem_len, il.data(), il.size() * 4);
    S.dnext.alloc(8, ctx->stream);
    S.arena.alloc(S.arena_rows * S.plan.row_words * 8, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(S.arena.get(), 0, S.arena.bytes(), ctx->stream));
    S.overflow.alloc(nqueries * 4, ctx->stream);
    QEG_CUDA(cudaMemsetAsync(S.overflow.get(), 0, nqueries * 4, ctx->stream));
    S.counts.alloc(nqueries * 8, ctx->stream);
    S.out_vals.resize(S.plan.rtypes.size());
    S.out_valid.resize(S.plan.rtypes.size());
    for (size_t c = 0; c < S.plan.rtypes.size(); ++c) {
      S.out_vals[c].alloc(S.out_rows * 8, ctx->stream);
      S.out_valid[c].alloc(S.out_rows, ctx->stream);
    }
    const size_t sb = static_cast<size_t>(kBatchMaxSlots + 2) * S.plan.row_words * 8;
    require(sb <= ctx->smem_optin, "batch rows are too wide for the shared-memory tables");
    QEG_CUDA(cudaFuncSetAttribute(batch_agg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    // ---- capture the run into a CUDA graph ----
    QEG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    S.enqueue_run();
    QEG_CUDA(cudaStreamEndCapture(ctx->stream, &S.graph));
    QEG_CUDA(cudaGraphInstantiate(&S.exec, S.graph, 0));
    *out = b.release();
  });
}

qeg_status qeg_batch_run(qeg_batch* b) {
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr, "batch is NULL");
    BatchState& S = b->st;
    QEG_CUDA(cudaSetDevice(ctx->device));
    QEG_CUDA(cudaGraphLaunch(S.exec, ctx->stream));
    ctx->launches += 2;
  });
}

qeg_status qeg_batch_finish(qeg_batch* b, uint64_t* groups) {
  qeg_ctx* ctx = b ? b->st.ctx : nullptr;
  return guarded(ctx, [&] {
    require(b != nullptr, "batch is NULL");
    BatchState& S = b->st;
    QEG_CUDA(cudaSetDevice(ctx->device));
    std::vector<uint32_t> ovf(S.nq);
    S.group_counts.assign(S.nq, 0);
    QEG_CUDA(cudaMemcpyAsync(ovf.data(), S.overflow.get(), S.nq * 4, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaMemcpyAsync(S.group_counts.data(), S.counts.get(), S.nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QEG_CUDA(cudaStreamSynchronize(ctx->stream));
    check_device_error(ctx);
    // Queries whose table overflowed are recomputed exactly (grow-and-replay).
    S.fallback.clear();
    S.fallback.resize(S.nq);
    S.fell_back.clear();
    for (uint32_t q = 0; q < S.nq; ++q) {
      if (!ovf[q]) continue;
      S.fell_back.push_back(q);
      auto a = std::make_unique<AggState>();
      a->ctx = ctx;
      a->cfg.sizing = QEG_SIZE_FIXED;
      a->cfg.initial_capacity = 2 * S.qs[q].cap;
      const int32_t types[2] = {S.key.dev.type, S.val.dev.type};
      const uint32_t kc = 0;
      a->plan(types, 2, &kc, 1, S.plan.aggs.data(), static_cast<int>(S.plan.aggs.size()));
      qeg_column cols[2];
      const uint64_t off = S.offsets[q], n = S.offsets[q + 1] - off;
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
    QEG_CUDA(cudaMemsetAsync(S.overflow.get(), 0, S.nq * 4, ctx->stream));
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
    for (size_t c = 0; c < S.plan.rtypes.size(); ++c)
      fetch_column(ctx, S.out_vals[c].get(), S.out_valid[c].get<uint8_t>(), type_width(S.plan.rtypes[c]),
                   S.qs[query].out_off, S.group_counts[query], outs[c]);
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
    if (strategy) *strategy = S.qs[query].smem ? QEG_AGG_SMEM : QEG_AGG_GLOBAL;
    if (fell_back) *fell_back = std::count(S.fell_back.begin(), S.fell_back.end(), query) ? 1 : 0;
  });
}

void qeg_batch_destroy(qeg_batch* b) {
  if (!b) return;
  cudaSetDevice(b->st.ctx->device);
  delete b;
}

}  // extern "C"
