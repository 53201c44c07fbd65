// qeg_agg.h -- GROUP BY plan, kernel parameter blocks and host state.
#pragma once

#include "qeg_internal.h"

namespace qeg {

// Aggregate state fields of one group (see qeg_agg.cu for the encodings).
enum FieldKind : uint8_t {
  F_ROWS = 0,   // COUNT(*) of the group; also the occupancy marker of side rows
  F_NULLS = 1,  // NULL inputs of one column (non-null count = rows - nulls)
  F_SUMI = 2,   // SUM over I32/I64/TS/BOOL, two's complement
  F_SUMF = 3,   // SUM over F64
  F_MINI = 4,   // MIN over an integer column, ~enc_i64
  F_MAXI = 5,   // MAX over an integer column, enc_i64
  F_MINF = 6,   // MIN over F64, ~enc_f64 (NaN-greatest order)
  F_MAXF = 7,   // MAX over F64, enc_f64
};

constexpr int kMaxKeys = 8;
constexpr int kMaxVals = 8;
constexpr int kMaxFields = 24;
constexpr int kMaxAggs = 32;
// Target occupancy of a global GROUP BY table sized from a group-count estimate.
constexpr double kTargetLoad = 0.6;
// Tables sized from an estimate hold this many times the estimated groups at
// the target load: an underestimate costs a grow-and-replay pass, an
// overestimate only memory, so the margin leans high.
constexpr double kEstimateHeadroom = 1.5;
// Batches smaller than this are sized from their row count, not sketched.
constexpr uint64_t kSketchMinRows = 1ull << 22;

// Parameter block of the aggregation kernels (passed by value).
struct AggK {
  DevCol key[kMaxKeys];
  DevCol val[kMaxVals];
  int nkeys, nvals, nfields, row_words;
  uint8_t fkind[kMaxFields];
  uint8_t fcol[kMaxFields];  // value column of each field (field 0: rows)
  uint8_t cfirst[kMaxVals];
  uint8_t cnf[kMaxVals];
  uint64_t* table;
  uint64_t cap;  // slots; a key's first slot is mulhi(hash, cap)
  const uint32_t* sel;
  uint64_t nrows;  // rows to process (sel length, or len when dense)
  uint64_t len;    // physical column length
  int smem_slots;  // power of two, 0 = no private table
  int smem_insert; // 1: first-come insertion into the private table
  int smem_probe;
  const uint64_t* hot;  // heavy hitters preloaded into the private table
  int nhot;
  int warp_hot;  // the first warp_hot heavy hitters also get warp-private rows
  int probe_limit;
  uint32_t* spill_rows;
  uint64_t spill_cap;
  uint64_t* spill_parts;
  uint64_t part_cap;
  unsigned long long* counters;  // [0] spilled rows, [1] spilled partials, [2] inserted keys,
                                 // [3] running insert count, [4] table-full flag (u32)
  uint32_t* full_flag;           // NULL: no table-full signal
  uint64_t full_at;              // running insert count that raises the flag
  uint32_t* err;
  // Partitioned strategy, first pass (pool_key != nullptr): a row whose key is
  // not in its CTA's private table (read-only: the sketch's heavy hitters) is
  // appended to the region of its key's hash partition (key word + each value
  // column's 8-byte value) instead of going to the global table. Region p
  // holds rows [part_off[p], part_off[p + 1]) of the pool.
  uint64_t* pool_key;
  uint64_t* pool_val[kMaxVals];
  unsigned long long* part_fill;  // rows appended per partition
  const uint64_t* part_off;       // [nparts + 1] region starts (exact: a histogram pass sized them)
  int part_shift;                 // partition of a key = key_hash1(key) >> part_shift
};

// Parameter block of the partitioned strategy's second pass (part_agg_kernel):
// one CTA aggregates one partition's pool rows at a time in a shared-memory
// table and appends its groups, as table rows, to `tails`.
struct PartB {
  const uint64_t* pool_key;
  const uint64_t* pool_val[kMaxVals];
  const uint64_t* part_off;       // [nparts + 1]
  uint32_t nparts;
  int slots;                      // shared-memory table slots (power of two)
  uint64_t* tails;                // row_words words per group
  uint64_t tails_cap;
  unsigned long long* counters;   // [0] groups appended (may pass tails_cap), [1] failed partitions
  uint32_t* failed;               // ids of partitions whose groups did not fit the table
};

// Parameter block of the finalize kernel.
struct FinK {
  void* vals[kMaxKeys + kMaxAggs];
  uint8_t* valid[kMaxKeys + kMaxAggs];
  int32_t rtype[kMaxKeys + kMaxAggs];
  int32_t func[kMaxAggs];
  int32_t vfield[kMaxAggs];
  int32_t nfield[kMaxAggs];
  int naggs;
  unsigned long long* out_count;
  uint64_t out_cap;
  int64_t packed_width;  // > 0: single-key rows hold packed (partition key, bucket index) words
  // Single key: a second table of the same row format (nullptr: none). A row
  // whose key is also there is merged into that row and not emitted; the
  // second table is finalized after this one.
  uint64_t* merge_table;
  uint64_t merge_cap;
};

// Key-column sketch: the estimator's inputs and the heavy-hitter candidates.
constexpr int kSketchFeatures = 80;
struct SketchResult {
  float features[kSketchFeatures];
  double hll_estimate = 0;  // HyperLogLog distinct estimate over the sample
  double sample_rows = 0;
  double total_rows = 0;
  double null_frac = 0;
  double top_share[16] = {};  // share of sampled rows in the top 2^i candidates
  std::vector<uint64_t> heavy;  // candidate heavy-hitter key words, most frequent first
};

// Perfect hash of the first n heavy-hitter key words (qeg_agg.cu): 2^lgT
// slots, 2^lgB buckets, packed into `words` for the partitioned passes.
void hot_phf_build(const uint64_t* keys, int n, int* lgT, int* lgB, std::vector<uint64_t>& words);

// Builds the sketch of one key column (qeg_sketch.cu).
void sketch_key_column(qeg_ctx* ctx, const DevCol& key, const uint32_t* sel, uint64_t nrows, uint64_t len,
                       uint64_t sample_target, int want_heavy, SketchResult& out);
// Sketches every query [offsets[q], offsets[q+1]) of a batch's key column in
// one launch (one CTA per query); `d_offsets` is the device copy of `offsets`.
void batch_sketch(qeg_ctx* ctx, const DevCol& key, const uint64_t* d_offsets, const std::vector<uint64_t>& offsets,
                  uint64_t sample_target, std::vector<SketchResult>& out);
// Classic (non-learned) distinct-count extrapolation from a sketch.
double classic_estimate(const SketchResult& s);
// Learned estimate (qeg_estimator.cu): predicted distinct groups and the share of
// rows covered by the top heavy hitters. Returns false when no trained model
// is loaded in this context.
bool learned_estimate(qeg_ctx* ctx, const SketchResult& s, double* groups, double* hot_share);
// Non-null group count from the network's first output for sketch `s`.
double learned_groups(const SketchResult& s, float out0, double deadband);

struct AggState {
  qeg_ctx* ctx = nullptr;
  qeg_agg_config cfg{};
  std::vector<int32_t> types;
  std::vector<uint32_t> keys;
  std::vector<qeg_agg_spec> aggs;
  int mode = 0;  // 0 global, 1 single key, 2 multi key
  std::vector<uint32_t> val_cols;
  std::vector<uint8_t> fkind;
  std::vector<int> cfirst, cnf, vfield, nfield;
  std::vector<int32_t> rtypes;
  int nfields = 0, row_words = 0;

  DevBuf table;
  uint64_t cap = 0;
  DevBuf counters, spill_rows, spill_parts, hot_keys_dev;
  uint64_t spill_cap = 0, part_cap = 0;
  int smem_slots = 0, smem_insert = 0, nhot = 0;
  int probe_limit = 128;
  uint64_t inserted = 0, rows_seen = 0;
  uint32_t resizes = 0;
  int32_t strategy = QEG_AGG_AUTO;
  double est_groups = 0, hot_share = 0;
  std::vector<uint64_t> heavy_candidates;
  // Tumbling window (qeg_window_create): the last key is the time column, read
  // as its bucket's lower edge with this width; 0 for a plain GROUP BY.
  int64_t bucket_width = 0;
  // A window with one I32 partition key may pack (key, bucket index) into one
  // key word and take the single-key path while every batch allows it (no
  // NULLs in either column, bucket indexes within int32); a batch that does
  // not converts the table to composite rows.
  bool packable = false, packed = false;
  int64_t pack_qmin = 0, pack_qmax = 0;  // bucket-index range of the first packed batch

  // Partitioned strategy (QEG_AGG_PARTITIONED, single key): the first pass
  // aggregates each CTA's first-come keys in its private table and appends
  // every other row to its key-hash partition's region of the pool; the second
  // pass aggregates one partition per CTA in shared memory into `tails`, rows
  // of the table format. The global table holds the private tables' flushes,
  // spilled rows and partitions whose groups did not fit; finish() merges tail
  // rows whose key is also there and emits both.
  int part_bits = 0;
  int pb_slots = 0;
  DevBuf phf_dev;  // the heavy hitters' perfect hash (hot_phf_build)
  int phf_lgT = 6, phf_lgB = 3, phf_words = 0;
  DevBuf pool_key, part_fill, part_off, part_hist, part_failed, tails, part_counters;
  std::vector<DevBuf> pool_vals;
  uint64_t ntails = 0, tails_cap = 0;

  bool finished = false;
  uint64_t nout = 0;
  std::vector<DevBuf> out_vals, out_valid;

  void plan(const int32_t* col_types, int ncols, const uint32_t* key_cols, int nk, const qeg_agg_spec* aggs,
            int na);
  AggK kparams(const std::vector<StagedCol>& staged, const uint32_t* sel, uint64_t nrows, uint64_t len) const;
  AggK kparams_base() const;
  DevCol key_col(const std::vector<StagedCol>& staged, size_t j) const;
  bool can_pack(const std::vector<StagedCol>& staged, uint64_t len);
  void unpack();
  void alloc_table(uint64_t new_cap);
  size_t smem_bytes(int block) const;
  int warp_hot() const;
  int block_threads() const;
  void set_field_columns(AggK& P) const;
  uint32_t field_spec(const AggK& P) const;  // qeg_warpagg.cuh field-set code
  void launch(const AggK& P, uint64_t nrows);
  void launch_private(const AggK& P, uint64_t nrows);  // composite keys, CTA-private tables
  void read_counters(uint64_t out[3]);
  void grow(uint64_t new_cap);
  void first_consume(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len, const uint32_t* dsel);
  double estimate_groups(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len, const uint32_t* dsel);
  void settle(const std::vector<StagedCol>& staged, uint64_t len);
  bool part_eligible(const std::vector<StagedCol>& staged) const;
  int part_table_slots() const;
  void setup_partitioned(uint64_t nrows);
  void consume_partitioned(const std::vector<StagedCol>& staged, uint64_t nrows, uint64_t len, const uint32_t* dsel);
  void part_second_pass();
  void merge_tails();
  void consume(const qeg_column* cols, int ncols, const uint32_t* sel, uint64_t sel_len);
  void finish(uint64_t* nrows_out);
  void fetch(uint64_t first, uint64_t count, const qeg_out_column* outs);
};

}  // namespace qeg
