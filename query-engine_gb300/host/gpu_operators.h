// gpu_operators.h -- GPU-backed operators behind the reference engine's pull
// interface (ops/operator.h:40-47). They are the drop-in replacements of
// qe::Aggregate (ops/aggregate.h:102-144) and qe::HashJoin (ops/join.h:69-123):
// same constructor arguments, same output schema and column order, same
// Batch/Column views; the work runs in libqeg.so (include/qeg.h).
//
//   GpuAggregate  open() drains the child into page-locked host staging
//                 (selection vectors applied, contiguous ranges copied in
//                 bulk, STR codes canonicalised by value through a table built
//                 once per dictionary), hands it to the GPU in chunks of
//                 kChunkRows, finishes and fetches the whole result into
//                 page-locked memory; next() emits <= 2048 groups per batch as
//                 views into it, keys then aggregates (ops/aggregate.cpp:439-493).
//   GpuHashJoin   open() drains the build child into the GPU build store and
//                 builds the table; next() probes kProbeRows staged probe rows
//                 per GPU call, fetches the output kFetchRows at a time into
//                 page-locked memory and emits <= 2048 output rows per batch as
//                 views into it, probe columns then build columns
//                 (ops/join.cpp:260-299).
//   GpuWindow     qe::tsx::Window (tsx/window.h:82-100) in Tumbling mode: a
//                 GpuAggregate over (keys..., bucket start of the time
//                 column), output [keys..., bucket_start, aggregates...].
//   GpuAsofJoin   qe::tsx::AsofJoin (tsx/asof.h:94-150): a GpuHashJoin whose
//                 build side is sorted by (key, time) on the GPU and whose
//                 probe takes the nearest preceding build row per probe row.
//   DeviceTable / GpuScan
//                 qe::Table (ops/table.h:24-47) uploaded once and qe::Scan
//                 (ops/scan.h:13-29) over it. A GpuAggregate or GpuHashJoin
//                 whose child is a GpuScan reads the table's device columns
//                 in place: no host staging, no copy per query.
// A returned Batch's views stay valid until the next next() or close(), as
// ops/operator.h:14-22 requires.
// Errors surface as the reference's exception types: std::invalid_argument,
// std::overflow_error, std::bad_alloc, std::runtime_error otherwise.
#pragma once

#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <optional>
#include <string>
#include <utility>
#include <vector>

#include "../../include/qeg.h"
#include "qe_contract.h"

namespace qe::gpu {

// An owned host column published as a Column view (the OwnedColumn role,
// core/owned_batch.h:28-108).
struct HostColumn {
  Type type = Type::I64;
  std::size_t len = 0;
  std::vector<std::uint8_t> data;
  std::vector<std::uint64_t> validity;  // empty => all valid
  std::shared_ptr<const StringDict> dict;
  Column view() const;
};

// Page-locked host bytes (qeg_host_alloc), grown by doubling with their
// contents kept; ordinary heap memory where page-locked memory is refused.
class PinnedBuf {
 public:
  PinnedBuf() = default;
  ~PinnedBuf();
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  PinnedBuf(PinnedBuf&& o) noexcept { swap(o); }
  PinnedBuf& operator=(PinnedBuf&& o) noexcept {
    swap(o);
    return *this;
  }
  void reserve(std::size_t bytes);  // capacity >= bytes, contents kept
  std::uint8_t* data() const { return p_; }
  std::size_t capacity() const { return cap_; }

 private:
  void swap(PinnedBuf& o) noexcept {
    std::swap(p_, o.p_);
    std::swap(cap_, o.cap_);
    std::swap(pinned_, o.pinned_);
  }
  std::uint8_t* p_ = nullptr;
  std::size_t cap_ = 0;
  bool pinned_ = false;
};

// Host staging of rows pulled from a child, in page-locked memory: contiguous
// values and a packed validity bitmap per column. STR codes become canonical
// ids through a code -> id table built once per source dictionary (extended
// when the dictionary grows), not by interning every row.
struct Staging {
  std::vector<Type> types;
  std::vector<PinnedBuf> vals;
  std::vector<PinnedBuf> valid;  // validity words
  std::vector<bool> any_null;
  std::size_t rows = 0;
  // Per column: source dictionary -> id of each of its codes.
  std::vector<std::map<const StringDict*, std::vector<std::int32_t>>> code_ids;
  void reset(const std::vector<Type>& t);  // empties the rows, keeps buffers and code tables
  // Appends the logical rows of `b`; STR columns go through `ids[c]` (value ->
  // canonical id; nullptr for non-STR columns).
  void append(const Batch& b, const std::vector<StringDict*>& ids);
  std::vector<qeg_column> columns() const;
  std::int32_t* str_ids(std::size_t c) { return reinterpret_cast<std::int32_t*>(vals[c].data()); }
  const std::uint64_t* words(std::size_t c) const { return reinterpret_cast<const std::uint64_t*>(valid[c].data()); }
};

// Output columns fetched from the GPU into page-locked memory; next() hands
// out views of 2048-row slices (slice starts are multiples of 64, so a slice's
// validity is the words from start / 64 on).
struct OutColumns {
  std::vector<Type> types;
  std::vector<PinnedBuf> vals;
  std::vector<PinnedBuf> valid;
  std::vector<std::int32_t> all_valid;
  std::vector<std::shared_ptr<const StringDict>> dicts;
  void reserve(const std::vector<Type>& t, std::size_t rows);
  std::vector<qeg_out_column> outs();
  Column view(std::size_t c, std::size_t first, std::size_t n) const;
};

// One CUDA context per operator instance: operators are single-threaded
// objects and several may live in one process (exec/parallel.h:15-19).
class Device {
 public:
  explicit Device(int device = 0);
  ~Device();
  Device(const Device&) = delete;
  Device& operator=(const Device&) = delete;
  qeg_ctx* ctx() const { return ctx_; }
  void check(qeg_status s) const;  // throws the reference's exception types

 private:
  qeg_ctx* ctx_ = nullptr;
};

// A table resident in device memory: the reference's in-memory Table
// (ops/table.h:24-47) uploaded once, then read in place by every GpuScan over
// it. Each STR column holds codes of one table-owned dictionary (equal
// strings, equal codes); a validity bitmap is kept only for a column that
// holds a NULL.
class DeviceTable {
 public:
  // Drains `src` (open, next until exhausted, close) into device memory.
  static std::shared_ptr<const DeviceTable> upload(Operator& src, int device = 0);
  ~DeviceTable();
  DeviceTable(const DeviceTable&) = delete;
  DeviceTable& operator=(const DeviceTable&) = delete;

  const Schema& schema() const { return schema_; }
  std::size_t num_rows() const { return rows_; }
  const std::shared_ptr<StringDict>& dict(std::size_t c) const { return dicts_[c]; }
  bool all_valid(std::size_t c) const { return valid_[c] == nullptr; }
  // Rows [first, first + n) of every column as device-pointer views (`first`
  // a multiple of 64). A STR column is QEG_STR with code_maps[c] (host memory,
  // one entry per code of its dictionary) as its code map.
  std::vector<qeg_column> columns(std::size_t first, std::size_t n,
                                  const std::vector<std::vector<std::int32_t>>& code_maps) const;
  // Copies rows [first, first + n) of column c (`first` a multiple of 64) to
  // host memory: the values to `vals`, and the validity words to `words` when
  // the column holds a NULL. Safe to call from several threads (the copies
  // share the table's context and take turns).
  void download(std::size_t c, std::size_t first, std::size_t n, void* vals, std::uint64_t* words) const;

 private:
  DeviceTable() = default;
  Schema schema_;
  std::size_t rows_ = 0;
  std::unique_ptr<Device> dev_;
  mutable std::mutex download_mu_;
  std::vector<void*> data_;
  std::vector<std::uint64_t*> valid_;
  std::vector<std::shared_ptr<StringDict>> dicts_;
};

// qe::Scan (ops/scan.h:13-29) over a DeviceTable, with its batch_size check
// and cursor rules. Under an ordinary parent it emits batch_size-row batches
// copied back to page-locked host memory, kFetchRows rows per copy; as the
// child of a GpuAggregate or GpuHashJoin it hands its table to the GPU where
// it lies, with no host staging.
class GpuScan : public Operator {
 public:
  static constexpr std::size_t kDefaultBatchSize = 2048;  // ops/scan.h:15
  static constexpr std::size_t kFetchRows = 1u << 20;

  explicit GpuScan(std::shared_ptr<const DeviceTable> table, std::size_t batch_size = kDefaultBatchSize);

  void open() override;
  std::optional<Batch> next() override;
  void close() override;
  Schema output_schema() const override;
  const std::shared_ptr<const DeviceTable>& table() const { return table_; }

 private:
  std::shared_ptr<const DeviceTable> table_;
  std::size_t batch_size_;
  std::size_t cursor_ = 0;                      // next row to emit
  std::size_t win_first_ = 0, win_rows_ = 0;    // rows held in out_
  OutColumns out_;
};

class GpuAggregate : public Operator {
 public:
  static constexpr std::size_t kOutBatch = 2048;       // ops/aggregate.h:105
  static constexpr std::size_t kChunkRows = 8u << 20;  // rows staged per GPU call
  static constexpr std::size_t kDeviceSliceRows = 1u << 30;  // GpuScan-child rows per GPU call

  GpuAggregate(std::unique_ptr<Operator> child, std::vector<std::uint32_t> key_cols, std::vector<AggSpec> aggs,
               qeg_agg_config cfg = {}, int device = 0);
  ~GpuAggregate() override;

  void open() override;
  std::optional<Batch> next() override;
  void close() override;
  Schema output_schema() const override;

 protected:
  // Tumbling window: GROUP BY (key_cols..., (t / width) * width of time_col),
  // with the Window constructor's checks (tsx/window.cpp:214-241).
  GpuAggregate(std::unique_ptr<Operator> child, std::vector<std::uint32_t> key_cols, std::uint32_t time_col,
               std::int64_t width, std::vector<AggSpec> aggs, qeg_agg_config cfg, int device);

 private:
  void flush();

  bool window_ = false;
  std::uint32_t time_col_ = 0;
  std::int64_t width_ = 0;

  std::unique_ptr<Operator> child_;
  std::vector<std::uint32_t> key_cols_;
  std::vector<AggSpec> aggs_;
  qeg_agg_config cfg_;
  int device_;
  Schema child_schema_;
  std::unique_ptr<Device> dev_;
  qeg_agg* agg_ = nullptr;
  Staging staging_;
  bool has_str_ = false;
  std::vector<std::shared_ptr<StringDict>> str_ids_;  // per child column, STR only
  OutColumns result_;                                  // full result, keys then aggs
  std::size_t nrows_ = 0, cursor_ = 0;
  bool opened_ = false;
};

class GpuHashJoin : public Operator {
 public:
  static constexpr std::size_t kOutBatch = 2048;        // ops/join.h:73
  static constexpr std::size_t kProbeRows = 8u << 20;   // probe rows staged per GPU probe call
  static constexpr std::size_t kFetchRows = 1u << 20;   // output rows fetched per GPU call
  static constexpr std::size_t kBuildSliceRows = 1u << 30;  // GpuScan build rows per GPU call

  GpuHashJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build, std::vector<std::uint32_t> probe_keys,
              std::vector<std::uint32_t> build_keys, JoinType type, qeg_join_config cfg = {}, int device = 0);
  ~GpuHashJoin() override;

  void open() override;
  std::optional<Batch> next() override;
  void close() override;
  Schema output_schema() const override;

 protected:
  // Backward as-of join, with the AsofJoin constructor's checks
  // (tsx/asof.cpp:130-160); key lists may be empty.
  GpuHashJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build, std::vector<std::uint32_t> probe_keys,
              std::vector<std::uint32_t> build_keys, std::uint32_t probe_time, std::uint32_t build_time,
              tsx::AsofType type, std::optional<std::int64_t> tolerance, int device);

 private:
  bool probe_next_chunk();

  bool asof_ = false;
  // A GpuScan probe child read in place: its table, the next row to probe and
  // the STR code maps into the join's value ids.
  const DeviceTable* probe_table_ = nullptr;
  std::size_t probe_row_ = 0;
  std::vector<std::vector<std::int32_t>> probe_maps_;
  std::uint32_t probe_time_ = 0, build_time_ = 0;
  std::optional<std::int64_t> tolerance_;

  std::unique_ptr<Operator> probe_, build_;
  std::vector<std::uint32_t> probe_keys_, build_keys_;
  JoinType type_;
  qeg_join_config cfg_;
  int device_;
  Schema probe_schema_, build_schema_;
  std::unique_ptr<Device> dev_;
  qeg_join* join_ = nullptr;
  std::vector<std::shared_ptr<StringDict>> probe_ids_, build_ids_;  // STR columns
  Staging probe_stage_;
  std::uint64_t pending_ = 0;   // output rows of the last probe call
  std::uint64_t fetched_ = 0;   // of which fetched into out_
  std::uint64_t chunk_ = 0;     // rows in out_
  std::uint64_t cursor_ = 0;    // next row of out_ to emit
  OutColumns out_;
  bool opened_ = false, probe_done_ = false;
};

// qe::tsx::Window on the GPU. WindowMode::Sliding (a sort and a running
// frame, not a hash-table caller) is rejected with std::invalid_argument.
class GpuWindow : public GpuAggregate {
 public:
  static constexpr std::size_t kOutBatch = 2048;  // tsx/window.h:85

  GpuWindow(std::unique_ptr<Operator> child, tsx::WindowMode mode, std::vector<std::uint32_t> keys,
            std::uint32_t time, std::int64_t param, std::vector<AggSpec> aggs, qeg_agg_config cfg = {},
            int device = 0);
};

// qe::tsx::AsofJoin on the GPU: same constructor arguments and output schema
// (all probe columns, then all build columns).
class GpuAsofJoin : public GpuHashJoin {
 public:
  static constexpr std::size_t kOutBatch = 2048;  // tsx/asof.h:97

  GpuAsofJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build, std::vector<std::uint32_t> probe_keys,
              std::vector<std::uint32_t> build_keys, std::uint32_t probe_time, std::uint32_t build_time,
              tsx::AsofType type, std::optional<std::int64_t> tolerance = std::nullopt, int device = 0);
};

}  // namespace qe::gpu
