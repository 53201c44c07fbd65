// qe_contract.h -- the reference engine's frozen operator contract, restated so
// the GPU operators in this directory build standalone.
//
// The GPU operators must be drop-in replacements inside the reference's plan
// trees, so these declarations are kept layout- and signature-identical to the
// reference's frozen headers:
//   Type / byte_width          core/types.h:18-48
//   Column, SelectionVector,
//   Batch, Schema              core/column.h:55-90
//   validity word helpers      core/validity.h:21-63
//   Operator                   ops/operator.h:40-47
//   StringDict (interface)     core/string_dict.h:34-72
//   AggFunc / AggSpec          ops/aggregate.h:61-89
//   JoinType                   ops/join.h:59
//   tsx::WindowMode            tsx/window.h:79
//   tsx::AsofType              tsx/asof.h:90
// When compiled inside the reference tree, define QEG_WITH_REFERENCE_HEADERS
// and the reference's own headers are used instead of these.
#pragma once

#ifdef QEG_WITH_REFERENCE_HEADERS
#include "core/column.h"
#include "core/string_dict.h"
#include "core/types.h"
#include "core/validity.h"
#include "ops/aggregate.h"
#include "ops/join.h"
#include "ops/operator.h"
#include "tsx/asof.h"
#include "tsx/window.h"
#else

#include <cstddef>
#include <cstdint>
#include <deque>
#include <optional>
#include <string>
#include <string_view>
#include <unordered_map>
#include <utility>
#include <vector>

namespace qe {

enum class Type { I32, I64, F64, BOOL, TS, STR };

inline constexpr std::size_t byte_width(Type t) {
  switch (t) {
    case Type::I32: return 4;
    case Type::I64: return 8;
    case Type::F64: return 8;
    case Type::BOOL: return 1;
    case Type::TS: return 8;
    case Type::STR: return 4;
  }
  return 0;
}

// A string dictionary with the reference's interface (intern / at / size):
// codes are dense and handed out in first-seen order. The strings live in a
// deque (stable addresses), and the lookup map's keys are views of them.
class StringDict {
 public:
  StringDict() = default;
  StringDict(const StringDict& o) : values_(o.values_) { reindex(); }
  StringDict& operator=(const StringDict& o) {
    if (this != &o) {
      values_ = o.values_;
      reindex();
    }
    return *this;
  }
  // (A moved deque keeps its elements where they are, so the views stay valid.)
  StringDict(StringDict&&) noexcept = default;
  StringDict& operator=(StringDict&&) noexcept = default;

  std::int32_t intern(std::string_view s) {
    const auto found = codes_.find(s);
    if (found != codes_.end()) return found->second;
    const auto code = static_cast<std::int32_t>(values_.size());
    values_.emplace_back(s);
    codes_.emplace(std::string_view(values_.back()), code);
    return code;
  }
  std::string_view at(std::int32_t code) const { return values_[static_cast<std::size_t>(code)]; }
  std::size_t size() const noexcept { return values_.size(); }

 private:
  void reindex() {
    codes_.clear();
    for (std::size_t i = 0; i < values_.size(); ++i)
      codes_.emplace(std::string_view(values_[i]), static_cast<std::int32_t>(i));
  }
  std::deque<std::string> values_;
  std::unordered_map<std::string_view, std::int32_t> codes_;
};

struct Column {
  Type type;
  size_t len;
  const std::byte* data;
  const uint64_t* validity;
  bool all_valid;
  const StringDict* dict;
};

struct SelectionVector {
  const uint32_t* idx;
  size_t len;
};

struct Batch {
  std::vector<Column> cols;
  const SelectionVector* sel;
  size_t row_count;
};

struct Schema {
  std::vector<std::pair<std::string, Type>> fields;
};

namespace validity {
inline constexpr std::size_t words(std::size_t nbits) { return (nbits + 63) / 64; }
inline bool get_bit(const std::uint64_t* w, std::size_t i) { return (w[i >> 6] >> (i & 63u)) & 1ull; }
inline void set_bit(std::uint64_t* w, std::size_t i, bool valid) {
  const std::uint64_t bit = std::uint64_t{1} << (i & 63u);
  if (valid) w[i >> 6] |= bit;
  else w[i >> 6] &= ~bit;
}
}  // namespace validity

class Operator {
 public:
  virtual void open() = 0;
  virtual std::optional<Batch> next() = 0;
  virtual void close() = 0;
  virtual Schema output_schema() const = 0;
  virtual ~Operator() = default;
};

enum class AggFunc { CountStar, Count, Sum, Min, Max, Avg };

struct AggSpec {
  AggFunc func = AggFunc::CountStar;
  std::uint32_t input_col = 0;
  std::string out_name;
  static AggSpec count_star(std::string name) { return {AggFunc::CountStar, 0, std::move(name)}; }
  static AggSpec count(std::uint32_t col, std::string name) { return {AggFunc::Count, col, std::move(name)}; }
  static AggSpec sum(std::uint32_t col, std::string name) { return {AggFunc::Sum, col, std::move(name)}; }
  static AggSpec min(std::uint32_t col, std::string name) { return {AggFunc::Min, col, std::move(name)}; }
  static AggSpec max(std::uint32_t col, std::string name) { return {AggFunc::Max, col, std::move(name)}; }
  static AggSpec avg(std::uint32_t col, std::string name) { return {AggFunc::Avg, col, std::move(name)}; }
};

enum class JoinType { Inner, Left };

namespace tsx {
enum class WindowMode { Tumbling, Sliding };
enum class AsofType { Inner, Left };
}  // namespace tsx

}  // namespace qe

#endif  // QEG_WITH_REFERENCE_HEADERS
