// gpu_operators.h -- GPU-backed operators behind the reference engine's pull
// interface (ops/operator.h:40-47). They are the drop-in replacements of
// qe::Aggregate (ops/aggregate.h:102-144) and qe::HashJoin (ops/join.h:69-123):
// same constructor arguments, same output schema and column order, same
// Batch/Column views; the work runs in libqeg.so (include/qeg.h).
//
//   GpuAggregate  open() drains the child into pinned host staging (selection
//                 vectors applied, STR canonicalised by value), hands it to
//                 the GPU in chunks, finishes; next() emits <= 2048 groups per
//                 batch, keys then aggregates (ops/aggregate.cpp:439-493).
//   GpuHashJoin   open() drains the build child into the GPU build store and
//                 builds the table; next() probes one probe batch at a time
//                 and emits <= 2048 output rows per batch, probe columns then
//                 build columns (ops/join.cpp:260-299).
//   GpuWindow     qe::tsx::Window (tsx/window.h:82-100) in Tumbling mode: a
//                 GpuAggregate over (keys..., bucket start of the time
//                 column), output [keys..., bucket_start, aggregates...].
//   GpuAsofJoin   qe::tsx::AsofJoin (tsx/asof.h:94-150): a GpuHashJoin whose
//                 build side is sorted by (key, time) on the GPU and whose
//                 probe takes the nearest preceding build row per probe row.
// Errors surface as the reference's exception types: std::invalid_argument,
// std::overflow_error, std::bad_alloc, std::runtime_error otherwise.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <string>
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

// Host staging of rows pulled from a child: contiguous values and a packed
// validity bitmap per column, STR values canonicalised by value into ids.
struct Staging {
  std::vector<Type> types;
  std::vector<std::vector<std::uint8_t>> vals;
  std::vector<std::vector<std::uint64_t>> valid;
  std::vector<bool> any_null;
  std::size_t rows = 0;
  void reset(const std::vector<Type>& t);
  // Appends the logical rows of `b`; STR columns go through `ids[c]` (value ->
  // canonical id; nullptr for non-STR columns).
  void append(const Batch& b, const std::vector<StringDict*>& ids);
  std::vector<qeg_column> columns() const;
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

class GpuAggregate : public Operator {
 public:
  static constexpr std::size_t kOutBatch = 2048;       // ops/aggregate.h:105
  static constexpr std::size_t kChunkRows = 8u << 20;  // rows staged per GPU call

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
  std::vector<HostColumn> result_;                    // full result, keys then aggs
  std::vector<std::shared_ptr<StringDict>> out_dicts_;
  std::size_t nrows_ = 0, cursor_ = 0;
  std::vector<HostColumn> current_;
  bool opened_ = false;
};

class GpuHashJoin : public Operator {
 public:
  static constexpr std::size_t kOutBatch = 2048;  // ops/join.h:73

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
  bool probe_next_batch();

  bool asof_ = false;
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
  std::uint64_t pending_ = 0, cursor_ = 0;
  std::vector<HostColumn> current_;
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
