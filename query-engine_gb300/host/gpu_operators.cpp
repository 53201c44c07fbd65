// gpu_operators.cpp -- GpuAggregate / GpuHashJoin (see gpu_operators.h).
#include "gpu_operators.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>

namespace qe::gpu {

namespace {

int32_t to_qeg(Type t) { return static_cast<int32_t>(t); }

int32_t agg_func(AggFunc f) { return static_cast<int32_t>(f); }

Type result_type(AggFunc f, Type in) {  // ops/aggregate.cpp:78-97
  switch (f) {
    case AggFunc::CountStar:
    case AggFunc::Count: return Type::I64;
    case AggFunc::Sum:
      if (in == Type::STR) throw std::invalid_argument("SUM is not defined on STR (VARCHAR)");
      return in == Type::F64 ? Type::F64 : Type::I64;
    case AggFunc::Avg:
      if (in == Type::STR) throw std::invalid_argument("AVG is not defined on STR (VARCHAR)");
      return Type::F64;
    default: return in;
  }
}

inline uint32_t sel_at(const SelectionVector* sel, std::size_t k) {
  return sel ? sel->idx[k] : static_cast<uint32_t>(k);
}

}  // namespace

Column HostColumn::view() const {
  Column c;
  c.type = type;
  c.len = len;
  c.data = reinterpret_cast<const std::byte*>(data.data());
  const bool av = validity.empty();
  c.all_valid = av;
  c.validity = av ? nullptr : validity.data();
  c.dict = dict.get();
  return c;
}

PinnedBuf::~PinnedBuf() {
  if (pinned_) qeg_host_free(p_);
  else std::free(p_);
}

void PinnedBuf::reserve(std::size_t bytes) {
  if (bytes <= cap_) return;
  const std::size_t want = std::max<std::size_t>({bytes, cap_ * 2, 4096});
  void* q = nullptr;
  bool pinned = qeg_host_alloc(want, &q) == QEG_OK && q != nullptr;
  if (!pinned) {
    q = std::malloc(want);
    if (!q) throw std::bad_alloc();
  }
  if (cap_) std::memcpy(q, p_, cap_);
  if (pinned_) qeg_host_free(p_);
  else std::free(p_);
  p_ = static_cast<std::uint8_t*>(q);
  cap_ = want;
  pinned_ = pinned;
}

void Staging::reset(const std::vector<Type>& t) {
  if (types != t) {
    types = t;
    vals.clear();
    valid.clear();
    vals.resize(t.size());
    valid.resize(t.size());
    code_ids.assign(t.size(), {});
  }
  any_null.assign(t.size(), false);
  rows = 0;
}

void Staging::append(const Batch& b, const std::vector<StringDict*>& ids) {
  const std::size_t n = b.row_count;
  if (n == 0) return;
  const std::size_t new_rows = rows + n;
  const std::size_t old_words = validity::words(rows), new_words = validity::words(new_rows);
  for (std::size_t c = 0; c < types.size(); ++c) {
    const Column& col = b.cols[c];
    const std::size_t w = byte_width(types[c]);
    vals[c].reserve(new_rows * w);
    valid[c].reserve(new_words * 8);
    auto* bits = reinterpret_cast<std::uint64_t*>(valid[c].data());
    // Words this batch starts: all valid until a NULL clears a bit.
    for (std::size_t k = old_words; k < new_words; ++k) bits[k] = ~0ull;
    std::uint8_t* dst = vals[c].data() + rows * w;
    if (types[c] == Type::STR) {
      // Codes -> canonical ids through the dictionary's table.
      std::vector<std::int32_t>& tab = code_ids[c][col.dict];
      for (std::size_t code = tab.size(); code < col.dict->size(); ++code)
        tab.push_back(ids[c]->intern(col.dict->at(static_cast<std::int32_t>(code))));
      const auto* codes = reinterpret_cast<const std::int32_t*>(col.data);
      auto* out = reinterpret_cast<std::int32_t*>(dst);
      for (std::size_t k = 0; k < n; ++k) {
        const uint32_t p = sel_at(b.sel, k);
        const bool ok = col.all_valid || validity::get_bit(col.validity, p);
        const std::int32_t code = ok ? codes[p] : 0;
        if (ok && (code < 0 || static_cast<std::size_t>(code) >= tab.size()))
          throw std::invalid_argument("STR code outside its dictionary");
        out[k] = ok ? tab[code] : 0;
      }
    } else if (b.sel == nullptr) {
      std::memcpy(dst, col.data, n * w);  // a contiguous range: one copy
    } else {
      for (std::size_t k = 0; k < n; ++k)
        std::memcpy(dst + k * w, col.data + static_cast<std::size_t>(b.sel->idx[k]) * w, w);
    }
    if (col.all_valid) continue;
    if (b.sel == nullptr && rows % 64 == 0) {
      // Word-aligned destination: copy the batch's validity words.
      const std::size_t nw = validity::words(n);
      std::uint64_t any = ~0ull;
      for (std::size_t k = 0; k < nw; ++k) {
        std::uint64_t v = col.validity[k];
        if (k + 1 == nw && (n & 63u)) v |= ~0ull << (n & 63u);  // rows past the batch stay valid
        bits[rows / 64 + k] = v;
        any &= v;
      }
      if (any != ~0ull) any_null[c] = true;
    } else {
      for (std::size_t k = 0; k < n; ++k)
        if (!validity::get_bit(col.validity, sel_at(b.sel, k))) {
          validity::set_bit(bits, rows + k, false);
          any_null[c] = true;
        }
    }
  }
  rows = new_rows;
}

std::vector<qeg_column> Staging::columns() const {
  std::vector<qeg_column> out(types.size());
  for (std::size_t c = 0; c < types.size(); ++c) {
    qeg_column q{};
    // STR values are already canonical ids: hand them over as I32.
    q.type = types[c] == Type::STR ? QEG_I32 : to_qeg(types[c]);
    q.len = rows;
    q.data = vals[c].data();
    q.all_valid = any_null[c] ? 0 : 1;
    q.validity = any_null[c] ? words(c) : nullptr;
    out[c] = q;
  }
  return out;
}

void OutColumns::reserve(const std::vector<Type>& t, std::size_t rows) {
  if (types != t) {
    types = t;
    vals.clear();
    valid.clear();
    vals.resize(t.size());
    valid.resize(t.size());
    dicts.assign(t.size(), nullptr);
  }
  all_valid.assign(t.size(), 1);
  for (std::size_t c = 0; c < t.size(); ++c) {
    vals[c].reserve(std::max<std::size_t>(1, rows) * byte_width(t[c]));
    valid[c].reserve(std::max<std::size_t>(1, validity::words(rows)) * 8);
  }
}

std::vector<qeg_out_column> OutColumns::outs() {
  std::vector<qeg_out_column> o(types.size());
  for (std::size_t c = 0; c < types.size(); ++c)
    o[c] = {vals[c].data(), reinterpret_cast<std::uint64_t*>(valid[c].data()), &all_valid[c]};
  return o;
}

Column OutColumns::view(std::size_t c, std::size_t first, std::size_t n) const {
  Column v;
  v.type = types[c];
  v.len = n;
  v.data = reinterpret_cast<const std::byte*>(vals[c].data() + first * byte_width(types[c]));
  v.all_valid = all_valid[c] != 0;
  v.validity = v.all_valid ? nullptr : reinterpret_cast<const std::uint64_t*>(valid[c].data()) + first / 64;
  v.dict = dicts[c].get();
  return v;
}

Device::Device(int device) {
  const qeg_status s = qeg_ctx_create(device, &ctx_);
  if (s != QEG_OK) throw std::runtime_error(std::string("GPU context: ") + qeg_last_error(nullptr));
}

Device::~Device() { qeg_ctx_destroy(ctx_); }

void Device::check(qeg_status s) const {
  if (s == QEG_OK) return;
  const std::string m = qeg_last_error(ctx_);
  if (s == QEG_ERR_INVALID) throw std::invalid_argument(m);
  if (s == QEG_ERR_OVERFLOW) throw std::overflow_error(m);
  if (s == QEG_ERR_OOM) throw std::bad_alloc();
  throw std::runtime_error(m);
}

// ---------------------------------------------------------------------------
// DeviceTable / GpuScan
// ---------------------------------------------------------------------------
std::shared_ptr<const DeviceTable> DeviceTable::upload(Operator& src, int device) {
  std::shared_ptr<DeviceTable> t(new DeviceTable());
  t->schema_ = src.output_schema();
  t->dev_ = std::make_unique<Device>(device);
  const std::size_t nc = t->schema_.fields.size();
  std::vector<Type> types;
  for (const auto& f : t->schema_.fields) types.push_back(f.second);
  t->dicts_.assign(nc, nullptr);
  std::vector<StringDict*> ids(nc, nullptr);
  for (std::size_t c = 0; c < nc; ++c)
    if (types[c] == Type::STR) {
      t->dicts_[c] = std::make_shared<StringDict>();
      ids[c] = t->dicts_[c].get();
    }
  // The source's rows into page-locked staging (selections applied, STR codes
  // made the table dictionary's), then one copy per column.
  Staging st;
  st.reset(types);
  src.open();
  while (std::optional<Batch> b = src.next()) st.append(*b, ids);
  src.close();
  t->rows_ = st.rows;
  t->data_.assign(nc, nullptr);
  t->valid_.assign(nc, nullptr);
  for (std::size_t c = 0; c < nc; ++c) {
    const std::size_t bytes = st.rows * byte_width(types[c]);
    t->dev_->check(qeg_dev_alloc(t->dev_->ctx(), bytes, &t->data_[c]));
    t->dev_->check(qeg_dev_upload(t->dev_->ctx(), t->data_[c], st.vals[c].data(), bytes));
    if (!st.any_null[c]) continue;
    const std::size_t wbytes = validity::words(st.rows) * 8;
    void* w = nullptr;
    t->dev_->check(qeg_dev_alloc(t->dev_->ctx(), wbytes, &w));
    t->valid_[c] = static_cast<std::uint64_t*>(w);
    t->dev_->check(qeg_dev_upload(t->dev_->ctx(), w, st.valid[c].data(), wbytes));
  }
  return t;
}

DeviceTable::~DeviceTable() {
  for (void* p : data_) qeg_dev_free(p);
  for (std::uint64_t* p : valid_) qeg_dev_free(p);
}

std::vector<qeg_column> DeviceTable::columns(std::size_t first, std::size_t n,
                                             const std::vector<std::vector<std::int32_t>>& code_maps) const {
  if (first % 64 != 0 || first + n > rows_) throw std::invalid_argument("DeviceTable: slice out of range");
  std::vector<qeg_column> out(schema_.fields.size());
  for (std::size_t c = 0; c < out.size(); ++c) {
    const Type t = schema_.fields[c].second;
    qeg_column q{};
    q.type = to_qeg(t);
    q.len = n;
    q.data = n ? static_cast<const std::uint8_t*>(data_[c]) + first * byte_width(t) : nullptr;
    q.all_valid = valid_[c] ? 0 : 1;
    q.validity = valid_[c] && n ? valid_[c] + first / 64 : nullptr;
    if (t == Type::STR && c < code_maps.size() && !code_maps[c].empty()) {
      q.code_map = code_maps[c].data();
      q.code_map_len = code_maps[c].size();
    }
    out[c] = q;
  }
  return out;
}

void DeviceTable::download(std::size_t c, std::size_t first, std::size_t n, void* vals,
                           std::uint64_t* words) const {
  if (first % 64 != 0 || first + n > rows_) throw std::invalid_argument("DeviceTable: slice out of range");
  if (n == 0) return;
  const std::size_t w = byte_width(schema_.fields[c].second);
  std::lock_guard<std::mutex> lock(download_mu_);
  dev_->check(qeg_dev_download(dev_->ctx(), vals, static_cast<const std::uint8_t*>(data_[c]) + first * w, n * w));
  if (valid_[c])
    dev_->check(qeg_dev_download(dev_->ctx(), words, valid_[c] + first / 64, validity::words(n) * 8));
}

GpuScan::GpuScan(std::shared_ptr<const DeviceTable> table, std::size_t batch_size)
    : table_(std::move(table)), batch_size_(batch_size) {
  if (!table_) throw std::invalid_argument("GpuScan: table is NULL");
  if (batch_size_ == 0 || batch_size_ % 64 != 0)  // ops/scan.cpp:11-19
    throw std::invalid_argument("Scan batch_size must be a positive multiple of 64 (validity word alignment)");
}

void GpuScan::open() {
  cursor_ = 0;
  win_first_ = win_rows_ = 0;
}

void GpuScan::close() { cursor_ = table_->num_rows(); }

Schema GpuScan::output_schema() const { return table_->schema(); }

std::optional<Batch> GpuScan::next() {
  const std::size_t total = table_->num_rows();
  if (cursor_ >= total) return std::nullopt;
  if (cursor_ < win_first_ || cursor_ >= win_first_ + win_rows_) {
    // The next kFetchRows rows (a multiple of batch_size) into page-locked memory.
    const std::size_t span = std::max(batch_size_, kFetchRows - kFetchRows % batch_size_);
    win_first_ = cursor_;
    win_rows_ = std::min(span, total - cursor_);
    std::vector<Type> types;
    for (const auto& f : table_->schema().fields) types.push_back(f.second);
    out_.reserve(types, win_rows_);
    for (std::size_t c = 0; c < types.size(); ++c) {
      table_->download(c, win_first_, win_rows_, out_.vals[c].data(),
                       reinterpret_cast<std::uint64_t*>(out_.valid[c].data()));
      out_.all_valid[c] = table_->all_valid(c) ? 1 : 0;
      out_.dicts[c] = table_->dict(c);
    }
  }
  const std::size_t n = std::min(batch_size_, total - cursor_);
  Batch b;
  for (std::size_t c = 0; c < out_.types.size(); ++c) b.cols.push_back(out_.view(c, cursor_ - win_first_, n));
  b.sel = nullptr;
  b.row_count = n;
  cursor_ += n;
  return b;
}

// ---------------------------------------------------------------------------
// GpuAggregate
// ---------------------------------------------------------------------------
GpuAggregate::GpuAggregate(std::unique_ptr<Operator> child, std::vector<std::uint32_t> key_cols,
                           std::vector<AggSpec> aggs, qeg_agg_config cfg, int device)
    : child_(std::move(child)), key_cols_(std::move(key_cols)), aggs_(std::move(aggs)), cfg_(cfg), device_(device) {
  if (aggs_.empty()) throw std::invalid_argument("Aggregate needs >=1 aggregate");
  child_schema_ = child_->output_schema();
}

GpuAggregate::GpuAggregate(std::unique_ptr<Operator> child, std::vector<std::uint32_t> key_cols,
                           std::uint32_t time_col, std::int64_t width, std::vector<AggSpec> aggs, qeg_agg_config cfg,
                           int device)
    : window_(true),
      time_col_(time_col),
      width_(width),
      child_(std::move(child)),
      key_cols_(std::move(key_cols)),
      aggs_(std::move(aggs)),
      cfg_(cfg),
      device_(device) {
  if (aggs_.empty()) throw std::invalid_argument("Window needs >=1 aggregate");
  child_schema_ = child_->output_schema();
  const std::size_t nc = child_schema_.fields.size();
  for (std::uint32_t k : key_cols_) {
    if (k >= nc) throw std::invalid_argument("Window: partition key column out of range");
    if (child_schema_.fields[k].second == Type::STR)
      throw std::invalid_argument("Window: STR partition keys are not supported (out of grammar)");
  }
  for (const AggSpec& a : aggs_)
    if (a.func != AggFunc::CountStar && a.input_col < nc && child_schema_.fields[a.input_col].second == Type::STR)
      throw std::invalid_argument("Window: STR aggregate inputs are not supported (out of grammar)");
  if (time_col_ >= nc) throw std::invalid_argument("Window: time column out of range");
  const Type tt = child_schema_.fields[time_col_].second;
  if (tt != Type::I32 && tt != Type::I64 && tt != Type::TS)
    throw std::invalid_argument("Window: time column must be I32/I64/TS");
  if (width_ <= 0) throw std::invalid_argument("Window: tumbling width W must be > 0");
}

GpuAggregate::~GpuAggregate() { close(); }

Schema GpuAggregate::output_schema() const {
  Schema s;
  for (std::uint32_t k : key_cols_) s.fields.push_back(child_schema_.fields[k]);
  if (window_) s.fields.push_back(child_schema_.fields[time_col_]);  // bucket_start
  for (const AggSpec& a : aggs_) {
    const Type in = a.func == AggFunc::CountStar ? Type::I64 : child_schema_.fields[a.input_col].second;
    s.fields.emplace_back(a.out_name, result_type(a.func, in));
  }
  return s;
}

void GpuAggregate::flush() {
  if (staging_.rows == 0) return;
  const auto cols = staging_.columns();
  dev_->check(qeg_agg_consume(agg_, cols.data(), static_cast<int>(cols.size()), nullptr, 0));
  staging_.reset(staging_.types);
}

void GpuAggregate::open() {
  if (opened_) return;
  opened_ = true;
  dev_ = std::make_unique<Device>(device_);
  // A GpuScan child: its device columns are consumed where they lie, STR
  // columns as codes with a code map; otherwise rows are staged on the host
  // and STR columns arrive as canonical ids.
  const auto* scan = dynamic_cast<const GpuScan*>(child_.get());
  const DeviceTable* table = scan ? scan->table().get() : nullptr;
  std::vector<Type> types;
  std::vector<int32_t> qtypes;
  for (const auto& f : child_schema_.fields) {
    types.push_back(f.second);
    qtypes.push_back(f.second == Type::STR && !table ? QEG_I32 : to_qeg(f.second));
    if (f.second == Type::STR) has_str_ = true;
  }
  std::vector<qeg_agg_spec> specs;
  for (const AggSpec& a : aggs_) {
    const Type in = a.func == AggFunc::CountStar ? Type::I64 : child_schema_.fields[a.input_col].second;
    result_type(a.func, in);  // raises the reference's errors (SUM/AVG on STR)
    specs.push_back({agg_func(a.func), a.input_col});
  }
  if (window_)
    dev_->check(qeg_window_create(dev_->ctx(), qtypes.data(), static_cast<int>(qtypes.size()), key_cols_.data(),
                                  static_cast<int>(key_cols_.size()), time_col_, width_, specs.data(),
                                  static_cast<int>(specs.size()), &cfg_, &agg_));
  else
    dev_->check(qeg_agg_create(dev_->ctx(), qtypes.data(), static_cast<int>(qtypes.size()), key_cols_.data(),
                               static_cast<int>(key_cols_.size()), specs.data(), static_cast<int>(specs.size()),
                               &cfg_, &agg_));
  staging_.reset(types);
  str_ids_.assign(types.size(), nullptr);
  std::vector<StringDict*> ids(types.size(), nullptr);
  for (std::size_t c = 0; c < types.size(); ++c)
    if (types[c] == Type::STR) {
      str_ids_[c] = std::make_shared<StringDict>();
      ids[c] = str_ids_[c].get();
    }

  // STR ids must be order-preserving for MIN/MAX by value: a STR value goes
  // to the GPU as its rank in string order, and rank_to_id[c] maps it back.
  std::vector<std::vector<int32_t>> rank_to_id(types.size());
  if (table) {
    std::vector<std::vector<int32_t>> ranks(types.size());
    for (std::size_t c = 0; c < types.size(); ++c) {
      if (types[c] != Type::STR) continue;
      str_ids_[c] = table->dict(c);
      const StringDict& d = *str_ids_[c];
      std::vector<int32_t> order(d.size());
      for (std::size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int32_t>(i);
      std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return d.at(a) < d.at(b); });
      ranks[c].resize(d.size());
      for (std::size_t r = 0; r < order.size(); ++r) ranks[c][order[r]] = static_cast<int32_t>(r);
      rank_to_id[c] = std::move(order);
    }
    child_->open();
    const std::size_t rows = table->num_rows();
    for (std::size_t first = 0; first < rows; first += kDeviceSliceRows) {
      const auto cols = table->columns(first, std::min(kDeviceSliceRows, rows - first), ranks);
      dev_->check(qeg_agg_consume(agg_, cols.data(), static_cast<int>(cols.size()), nullptr, 0));
    }
    child_->close();
  } else {
    child_->open();
    while (std::optional<Batch> b = child_->next()) {
      staging_.append(*b, ids);
      if (!has_str_ && staging_.rows >= kChunkRows) flush();
    }
    child_->close();
  }
  if (has_str_ && !table) {
    for (std::size_t c = 0; c < types.size(); ++c) {
      if (!str_ids_[c]) continue;
      const StringDict& d = *str_ids_[c];
      std::vector<int32_t> order(d.size());
      for (std::size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int32_t>(i);
      std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return d.at(a) < d.at(b); });
      std::vector<int32_t> rank(d.size());
      for (std::size_t r = 0; r < order.size(); ++r) rank[order[r]] = static_cast<int32_t>(r);
      std::int32_t* v = staging_.str_ids(c);
      const std::uint64_t* ok = staging_.words(c);
      for (std::size_t r = 0; r < staging_.rows; ++r)
        if (validity::get_bit(ok, r)) v[r] = rank[v[r]];
      rank_to_id[c] = std::move(order);
    }
  }
  flush();
  uint64_t n = 0;
  dev_->check(qeg_agg_finish(agg_, &n));
  nrows_ = n;
  const Schema out = output_schema();
  std::vector<Type> otypes;
  for (const auto& f : out.fields) otypes.push_back(f.second);
  result_.reserve(otypes, nrows_);
  std::vector<qeg_out_column> outs = result_.outs();
  dev_->check(qeg_agg_fetch(agg_, 0, nrows_, outs.data()));
  // STR results: ranks back to strings, published through an owned dict.
  for (std::size_t c = 0; c < out.fields.size(); ++c) {
    if (out.fields[c].second != Type::STR) continue;  // (a window has no STR outputs)
    const std::uint32_t src = c < key_cols_.size() ? key_cols_[c] : aggs_[c - key_cols_.size()].input_col;
    const StringDict& d = *str_ids_[src];
    auto dict = std::make_shared<StringDict>();
    auto* v = reinterpret_cast<std::int32_t*>(result_.vals[c].data());
    const auto* ok = reinterpret_cast<const std::uint64_t*>(result_.valid[c].data());
    for (std::size_t r = 0; r < nrows_; ++r) {
      if (!result_.all_valid[c] && !validity::get_bit(ok, r)) continue;
      v[r] = dict->intern(d.at(rank_to_id[src][v[r]]));
    }
    result_.dicts[c] = dict;
  }
  cursor_ = 0;
}

std::optional<Batch> GpuAggregate::next() {
  if (cursor_ >= nrows_) return std::nullopt;
  const std::size_t m = std::min(kOutBatch, nrows_ - cursor_);
  Batch b;
  for (std::size_t c = 0; c < result_.types.size(); ++c) b.cols.push_back(result_.view(c, cursor_, m));
  b.sel = nullptr;
  b.row_count = m;
  cursor_ += m;
  return b;
}

void GpuAggregate::close() {
  if (agg_) qeg_agg_destroy(agg_);
  agg_ = nullptr;
  dev_.reset();
  opened_ = false;
}

// ---------------------------------------------------------------------------
// GpuHashJoin
// ---------------------------------------------------------------------------
GpuHashJoin::GpuHashJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build,
                         std::vector<std::uint32_t> probe_keys, std::vector<std::uint32_t> build_keys, JoinType type,
                         qeg_join_config cfg, int device)
    : probe_(std::move(probe)),
      build_(std::move(build)),
      probe_keys_(std::move(probe_keys)),
      build_keys_(std::move(build_keys)),
      type_(type),
      cfg_(cfg),
      device_(device) {
  if (probe_keys_.size() != build_keys_.size() || probe_keys_.empty())
    throw std::invalid_argument("join needs equal-length, non-empty key lists");
  probe_schema_ = probe_->output_schema();
  build_schema_ = build_->output_schema();
  for (std::size_t i = 0; i < probe_keys_.size(); ++i)
    if (probe_schema_.fields[probe_keys_[i]].second != build_schema_.fields[build_keys_[i]].second)
      throw std::invalid_argument("HashJoin: join key column types must match positionally");
}

GpuHashJoin::GpuHashJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build,
                         std::vector<std::uint32_t> probe_keys, std::vector<std::uint32_t> build_keys,
                         std::uint32_t probe_time, std::uint32_t build_time, tsx::AsofType type,
                         std::optional<std::int64_t> tolerance, int device)
    : asof_(true),
      probe_time_(probe_time),
      build_time_(build_time),
      tolerance_(tolerance),
      probe_(std::move(probe)),
      build_(std::move(build)),
      probe_keys_(std::move(probe_keys)),
      build_keys_(std::move(build_keys)),
      type_(type == tsx::AsofType::Left ? JoinType::Left : JoinType::Inner),
      cfg_{},
      device_(device) {
  if (probe_keys_.size() != build_keys_.size()) throw std::invalid_argument("asof needs equal-length key lists");
  probe_schema_ = probe_->output_schema();
  build_schema_ = build_->output_schema();
  if (probe_time_ >= probe_schema_.fields.size() || build_time_ >= build_schema_.fields.size())
    throw std::invalid_argument("AsofJoin: time column out of range");
  auto ts_ok = [](Type t) { return t == Type::I32 || t == Type::I64 || t == Type::TS; };
  if (!ts_ok(probe_schema_.fields[probe_time_].second) || !ts_ok(build_schema_.fields[build_time_].second))
    throw std::invalid_argument("AsofJoin: time columns must be I32/I64/TS");
  for (std::size_t i = 0; i < probe_keys_.size(); ++i)
    if (probe_schema_.fields[probe_keys_[i]].second != build_schema_.fields[build_keys_[i]].second)
      throw std::invalid_argument("AsofJoin: key column types must match positionally");
}

GpuHashJoin::~GpuHashJoin() { close(); }

Schema GpuHashJoin::output_schema() const {
  Schema s;
  for (const auto& f : probe_schema_.fields) s.fields.push_back(f);
  for (const auto& f : build_schema_.fields) s.fields.push_back(f);
  return s;
}

void GpuHashJoin::open() {
  if (opened_) return;
  opened_ = true;
  probe_done_ = false;
  pending_ = cursor_ = 0;
  dev_ = std::make_unique<Device>(device_);
  // A GpuScan child is read in place, its STR columns as codes with a code map
  // into the join's value ids. Key columns pair up by type, so a STR key read
  // in place needs the other side's in place too; otherwise that GpuScan runs
  // as an ordinary child through host staging.
  auto in_place = [](const std::unique_ptr<Operator>& op) -> const DeviceTable* {
    const auto* scan = dynamic_cast<const GpuScan*>(op.get());
    return scan ? scan->table().get() : nullptr;
  };
  const DeviceTable* build_table = in_place(build_);
  probe_table_ = in_place(probe_);
  probe_row_ = 0;
  if ((build_table == nullptr) != (probe_table_ == nullptr))
    for (std::size_t i = 0; i < build_keys_.size(); ++i)
      if (build_schema_.fields[build_keys_[i]].second == Type::STR) build_table = probe_table_ = nullptr;
  std::vector<Type> ptypes, btypes;
  std::vector<int32_t> qp, qb;
  for (const auto& f : probe_schema_.fields) {
    ptypes.push_back(f.second);
    qp.push_back(f.second == Type::STR && !probe_table_ ? QEG_I32 : to_qeg(f.second));
  }
  for (const auto& f : build_schema_.fields) {
    btypes.push_back(f.second);
    qb.push_back(f.second == Type::STR && !build_table ? QEG_I32 : to_qeg(f.second));
  }
  if (asof_)
    dev_->check(qeg_asof_create(dev_->ctx(), qp.data(), static_cast<int>(qp.size()), qb.data(),
                                static_cast<int>(qb.size()), probe_keys_.data(), build_keys_.data(),
                                static_cast<int>(probe_keys_.size()), probe_time_, build_time_,
                                type_ == JoinType::Left ? QEG_LEFT : QEG_INNER, tolerance_ ? 1 : 0,
                                tolerance_.value_or(0), &join_));
  else
    dev_->check(qeg_join_create(dev_->ctx(), qp.data(), static_cast<int>(qp.size()), qb.data(),
                                static_cast<int>(qb.size()), probe_keys_.data(), build_keys_.data(),
                                static_cast<int>(probe_keys_.size()), type_ == JoinType::Left ? QEG_LEFT : QEG_INNER,
                                &cfg_, &join_));
  // STR: key positions share one value-id space between the sides
  // (ops/join.cpp:48-71); other STR columns get their own dict.
  probe_ids_.assign(ptypes.size(), nullptr);
  build_ids_.assign(btypes.size(), nullptr);
  for (std::size_t i = 0; i < build_keys_.size(); ++i)
    if (btypes[build_keys_[i]] == Type::STR) {
      auto d = std::make_shared<StringDict>();
      build_ids_[build_keys_[i]] = d;
      probe_ids_[probe_keys_[i]] = d;
    }
  for (std::size_t c = 0; c < btypes.size(); ++c)
    if (btypes[c] == Type::STR && !build_ids_[c]) build_ids_[c] = std::make_shared<StringDict>();
  for (std::size_t c = 0; c < ptypes.size(); ++c)
    if (ptypes[c] == Type::STR && !probe_ids_[c]) probe_ids_[c] = std::make_shared<StringDict>();
  // Code maps of an in-place table: each code of its dictionary -> value id.
  auto value_ids = [](const DeviceTable& t, const std::vector<std::shared_ptr<StringDict>>& ids) {
    std::vector<std::vector<int32_t>> maps(ids.size());
    for (std::size_t c = 0; c < ids.size(); ++c) {
      if (!ids[c]) continue;
      const StringDict& d = *t.dict(c);
      for (std::size_t code = 0; code < d.size(); ++code)
        maps[c].push_back(ids[c]->intern(d.at(static_cast<int32_t>(code))));
    }
    return maps;
  };
  build_->open();
  if (build_table) {
    const auto maps = value_ids(*build_table, build_ids_);
    const std::size_t rows = build_table->num_rows();
    for (std::size_t first = 0; first < rows; first += kBuildSliceRows) {
      const auto cols = build_table->columns(first, std::min(kBuildSliceRows, rows - first), maps);
      dev_->check(qeg_join_build(join_, cols.data(), static_cast<int>(cols.size())));
    }
  } else {
    std::vector<StringDict*> bids(btypes.size(), nullptr);
    for (std::size_t c = 0; c < btypes.size(); ++c) bids[c] = build_ids_[c].get();
    Staging bs;
    bs.reset(btypes);
    while (std::optional<Batch> b = build_->next()) {
      bs.append(*b, bids);
      if (bs.rows >= (8u << 20)) {
        const auto cols = bs.columns();
        dev_->check(qeg_join_build(join_, cols.data(), static_cast<int>(cols.size())));
        bs.reset(btypes);
      }
    }
    if (bs.rows) {
      const auto cols = bs.columns();
      dev_->check(qeg_join_build(join_, cols.data(), static_cast<int>(cols.size())));
    }
  }
  build_->close();
  dev_->check(qeg_join_build_finish(join_));
  probe_maps_.clear();
  if (probe_table_) probe_maps_ = value_ids(*probe_table_, probe_ids_);
  probe_stage_.reset(ptypes);
  probe_->open();
  const Schema out = output_schema();
  std::vector<Type> otypes;
  for (const auto& f : out.fields) otypes.push_back(f.second);
  out_.reserve(otypes, 0);
  const std::size_t np = probe_schema_.fields.size();
  for (std::size_t c = 0; c < otypes.size(); ++c)
    if (otypes[c] == Type::STR) out_.dicts[c] = c < np ? probe_ids_[c] : build_ids_[c - np];
  pending_ = fetched_ = chunk_ = cursor_ = 0;
}

// Stages up to kProbeRows probe rows (whole batches) and probes them in one
// call. False when the probe child is exhausted.
bool GpuHashJoin::probe_next_chunk() {
  if (probe_table_) {  // the next kProbeRows rows of the in-place table
    const std::size_t rows = probe_table_->num_rows();
    if (probe_row_ >= rows) return false;
    const std::size_t n = std::min(kProbeRows, rows - probe_row_);
    const auto cols = probe_table_->columns(probe_row_, n, probe_maps_);
    probe_row_ += n;
    uint64_t out = 0;
    dev_->check(qeg_join_probe(join_, cols.data(), static_cast<int>(cols.size()), &out));
    pending_ = out;
    fetched_ = chunk_ = cursor_ = 0;
    return true;
  }
  std::vector<StringDict*> pids(probe_stage_.types.size(), nullptr);
  for (std::size_t c = 0; c < pids.size(); ++c) pids[c] = probe_ids_[c].get();
  probe_stage_.reset(probe_stage_.types);
  while (probe_stage_.rows < kProbeRows) {
    std::optional<Batch> b = probe_->next();
    if (!b) break;
    probe_stage_.append(*b, pids);
  }
  if (probe_stage_.rows == 0) return false;
  const auto cols = probe_stage_.columns();
  uint64_t n = 0;
  dev_->check(qeg_join_probe(join_, cols.data(), static_cast<int>(cols.size()), &n));
  pending_ = n;
  fetched_ = chunk_ = cursor_ = 0;
  return true;
}

std::optional<Batch> GpuHashJoin::next() {
  while (cursor_ >= chunk_) {
    if (fetched_ < pending_) {
      // The next kFetchRows output rows into the page-locked chunk.
      const std::uint64_t cnt = std::min<std::uint64_t>(kFetchRows, pending_ - fetched_);
      out_.reserve(out_.types, cnt);
      std::vector<qeg_out_column> outs = out_.outs();
      dev_->check(qeg_join_fetch(join_, fetched_, cnt, outs.data()));
      fetched_ += cnt;
      chunk_ = cnt;
      cursor_ = 0;
      continue;
    }
    if (probe_done_ || !probe_next_chunk()) {
      probe_done_ = true;
      return std::nullopt;
    }
  }
  const std::size_t m = std::min<std::uint64_t>(kOutBatch, chunk_ - cursor_);
  Batch b;
  for (std::size_t c = 0; c < out_.types.size(); ++c) b.cols.push_back(out_.view(c, cursor_, m));
  b.sel = nullptr;
  b.row_count = m;
  cursor_ += m;
  return b;
}

void GpuHashJoin::close() {
  if (opened_ && probe_) probe_->close();
  if (join_) qeg_join_destroy(join_);
  join_ = nullptr;
  dev_.reset();
  opened_ = false;
}

// ---------------------------------------------------------------------------
// GpuWindow / GpuAsofJoin
// ---------------------------------------------------------------------------
namespace {
std::int64_t tumbling_width(tsx::WindowMode mode, std::int64_t param) {
  if (mode != tsx::WindowMode::Tumbling)
    throw std::invalid_argument("GPU window: only WindowMode::Tumbling runs on the GPU (sliding uses qe::tsx::Window)");
  return param;
}
}  // namespace

GpuWindow::GpuWindow(std::unique_ptr<Operator> child, tsx::WindowMode mode, std::vector<std::uint32_t> keys,
                     std::uint32_t time, std::int64_t param, std::vector<AggSpec> aggs, qeg_agg_config cfg,
                     int device)
    : GpuAggregate(std::move(child), std::move(keys), time, tumbling_width(mode, param), std::move(aggs), cfg,
                   device) {}

GpuAsofJoin::GpuAsofJoin(std::unique_ptr<Operator> probe, std::unique_ptr<Operator> build,
                         std::vector<std::uint32_t> probe_keys, std::vector<std::uint32_t> build_keys,
                         std::uint32_t probe_time, std::uint32_t build_time, tsx::AsofType type,
                         std::optional<std::int64_t> tolerance, int device)
    : GpuHashJoin(std::move(probe), std::move(build), std::move(probe_keys), std::move(build_keys), probe_time,
                  build_time, type, tolerance, device) {}

}  // namespace qe::gpu
