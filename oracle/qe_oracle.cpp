// qe_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU restatement of the reference engine's hash GROUP BY / hash join semantics
// (explorer-skp/query-engine). It is the parity checker for the GPU kernels and
// the timed CPU baseline; the product never links it. See qe_oracle.h for the
// list of reference files and lines each part follows.
//
// Written from the reference's documented behaviour: this is not a copy of its
// sources (the data structures here are plain std:: containers keyed the way the
// reference's contract requires; the order of group ids and output rows, the NULL
// rules, the canonicalisation and the result types are what must agree).

#include "qe_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <string_view>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

enum class T : int32_t { I32 = 0, I64 = 1, F64 = 2, BOOL = 3, TS = 4, STR = 5 };
enum class Fn : int32_t { CountStar = 0, Count = 1, Sum = 2, Min = 3, Max = 4, Avg = 5 };

constexpr uint32_t kNoGroup = UINT32_MAX;                      // ops/hashtable.h:52
constexpr uint64_t kSeed = 0x51E57A11AB1E5EEDull;              // ops/hashtable.h:56
constexpr uint64_t kNullWord = 0x9E3779B97F4A7C15ull;          // ops/hash_internal.h:35
constexpr uint64_t kCanonNaN = 0x7ff8000000000000ull;          // ops/hash_internal.cpp:16

// A string dictionary: code -> bytes, plus a value -> code index (core/string_dict.h).
struct Dict {
  std::vector<std::string> vals;
  std::unordered_map<std::string, int32_t> index;
  int32_t intern(std::string_view s) {
    auto it = index.find(std::string(s));
    if (it != index.end()) return it->second;
    const int32_t c = static_cast<int32_t>(vals.size());
    vals.emplace_back(s);
    index.emplace(vals.back(), c);
    return c;
  }
};

struct Col {
  T type;
  uint64_t len;
  const uint8_t* data;
  const uint64_t* validity;
  bool all_valid;
  const uint32_t* dict_off;
  const char* dict_bytes;
  uint32_t dict_size;

  bool valid(uint64_t p) const {
    return all_valid || validity == nullptr || ((validity[p >> 6] >> (p & 63)) & 1ull);
  }
  int64_t ival(uint64_t p) const {
    switch (type) {
      case T::I32:
      case T::STR: {
        int32_t v;
        std::memcpy(&v, data + p * 4, 4);
        return v;
      }
      case T::I64:
      case T::TS: {
        int64_t v;
        std::memcpy(&v, data + p * 8, 8);
        return v;
      }
      case T::BOOL: return data[p];
      case T::F64: return 0;
    }
    return 0;
  }
  double fval(uint64_t p) const {
    double v;
    std::memcpy(&v, data + p * 8, 8);
    return v;
  }
  std::string_view str(int64_t code) const {
    if (code < 0 || static_cast<uint64_t>(code) >= dict_size)
      throw std::invalid_argument("STR code out of dictionary range");
    return std::string_view(dict_bytes + dict_off[code], dict_off[code + 1] - dict_off[code]);
  }
};

Col to_col(const orc_column& c) {
  Col r;
  r.type = static_cast<T>(c.type);
  r.len = c.len;
  r.data = static_cast<const uint8_t*>(c.data);
  r.validity = c.validity;
  r.all_valid = c.all_valid != 0 || c.validity == nullptr;
  r.dict_off = c.dict_offsets;
  r.dict_bytes = c.dict_bytes;
  r.dict_size = c.dict_size;
  if (r.type == T::STR && (r.dict_off == nullptr || r.dict_bytes == nullptr) && r.len > 0)
    throw std::invalid_argument("STR column without a dictionary");
  return r;
}

// ---------------------------------------------------------------------------
// Hash and normalisation (ops/hash_kernels.h:7-12, ops/hash_internal.cpp:29-97)
// ---------------------------------------------------------------------------
inline uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}
inline uint64_t fold(uint64_t acc, uint64_t w) { return mix64(acc ^ mix64(w)); }

uint64_t canon_word(const Col& c, uint64_t p) {
  switch (c.type) {
    case T::I32:
    case T::STR: return static_cast<uint32_t>(static_cast<int32_t>(c.ival(p)));
    case T::I64:
    case T::TS: return static_cast<uint64_t>(c.ival(p));
    case T::BOOL: return c.data[p];
    case T::F64: {
      const double d = c.fval(p);
      if (std::isnan(d)) return kCanonNaN;
      if (d == 0.0) return 0ull;
      uint64_t b;
      std::memcpy(&b, &d, 8);
      return b;
    }
  }
  return 0;
}

// One normalised key tuple.
struct KeyRow {
  std::vector<uint64_t> w;
  uint64_t nullmask = 0;
  uint64_t hash = kSeed;
};

// ---------------------------------------------------------------------------
// HashTable: open addressing, linear probing, power-of-two capacity, dense
// first-seen ids, growth x2 when occupancy exceeds 0.7 (ops/hashtable.cpp:60-163).
// ---------------------------------------------------------------------------
class HashTable {
 public:
  HashTable(size_t ncols, bool never_match) : ncols_(ncols), never_match_(never_match) {
    cap_ = 1024;
    slots_.assign(cap_, kNoGroup);
    words_.resize(ncols);
  }

  uint32_t insert_or_find(const KeyRow& k) {
    if (never_match_ && k.nullmask != 0) return new_group(k);  // dead, unfindable id
    size_t s = k.hash & (cap_ - 1);
    while (slots_[s] != kNoGroup) {
      const uint32_t g = slots_[s];
      if (hash_[g] == k.hash && equal(k, g)) return g;
      s = (s + 1) & (cap_ - 1);
    }
    const uint32_t g = new_group(k);
    slots_[s] = g;
    ++occupied_;
    if (occupied_ > static_cast<size_t>(static_cast<double>(cap_) * 0.7)) grow();
    return g;
  }

  uint32_t find(const KeyRow& k) const {
    if (never_match_ && k.nullmask != 0) return kNoGroup;
    size_t s = k.hash & (cap_ - 1);
    while (slots_[s] != kNoGroup) {
      const uint32_t g = slots_[s];
      if (hash_[g] == k.hash && equal(k, g)) return g;
      s = (s + 1) & (cap_ - 1);
    }
    return kNoGroup;
  }

  size_t groups() const { return hash_.size(); }
  bool is_null(uint32_t g, size_t c) const { return (null_[g] >> c) & 1ull; }
  uint64_t word(uint32_t g, size_t c) const { return words_[c][g]; }

 private:
  bool equal(const KeyRow& k, uint32_t g) const {
    if (k.nullmask != null_[g]) return false;
    for (size_t j = 0; j < ncols_; ++j) {
      if ((k.nullmask >> j) & 1ull) continue;
      if (k.w[j] != words_[j][g]) return false;
    }
    return true;
  }
  uint32_t new_group(const KeyRow& k) {
    if (hash_.size() >= kNoGroup) throw std::overflow_error("group id space exhausted");
    const uint32_t g = static_cast<uint32_t>(hash_.size());
    for (size_t j = 0; j < ncols_; ++j) words_[j].push_back(k.w[j]);
    null_.push_back(k.nullmask);
    hash_.push_back(k.hash);
    return g;
  }
  void grow() {
    const size_t nc = cap_ * 2;
    std::vector<uint32_t> ns(nc, kNoGroup);
    for (size_t s = 0; s < cap_; ++s) {
      const uint32_t g = slots_[s];
      if (g == kNoGroup) continue;
      size_t t = hash_[g] & (nc - 1);
      while (ns[t] != kNoGroup) t = (t + 1) & (nc - 1);
      ns[t] = g;
    }
    slots_.swap(ns);
    cap_ = nc;
  }

  size_t ncols_;
  bool never_match_;
  size_t cap_;
  size_t occupied_ = 0;
  std::vector<uint32_t> slots_;
  std::vector<std::vector<uint64_t>> words_;
  std::vector<uint64_t> null_;
  std::vector<uint64_t> hash_;
};

// ---------------------------------------------------------------------------
// Results
// ---------------------------------------------------------------------------
struct ResCol {
  T type;
  std::vector<int64_t> i;
  std::vector<double> f;
  std::vector<uint8_t> valid;
  std::shared_ptr<Dict> dict;  // STR only
};

}  // namespace

struct orc_result {
  std::vector<ResCol> cols;
  uint64_t rows = 0;
};

namespace {

// ---------------------------------------------------------------------------
// Aggregation (ops/aggregate.cpp, ops/agg_internal.h)
// ---------------------------------------------------------------------------
struct Cell {  // AggCell, ops/agg_internal.h:47-51
  int64_t i = 0;
  double d = 0.0;
  int64_t cnt = 0;
};

// NaN-greatest total order (ops/agg_internal.h:34-40).
inline bool less_total(double a, double b) {
  if (std::isnan(b)) return !std::isnan(a);
  if (std::isnan(a)) return false;
  return a < b;
}
inline double min_total(double a, double b) { return less_total(b, a) ? b : a; }
inline double max_total(double a, double b) { return less_total(a, b) ? b : a; }

Cell init_cell(Fn f) {  // ops/agg_internal.h:65-81
  Cell c;
  if (f == Fn::Min) {
    c.i = std::numeric_limits<int64_t>::max();
    c.d = std::numeric_limits<double>::quiet_NaN();
  } else if (f == Fn::Max) {
    c.i = std::numeric_limits<int64_t>::min();
    c.d = -std::numeric_limits<double>::infinity();
  }
  return c;
}

T result_type(Fn f, T in) {  // ops/aggregate.cpp:78-97
  switch (f) {
    case Fn::CountStar:
    case Fn::Count: return T::I64;
    case Fn::Sum:
      if (in == T::STR) throw std::invalid_argument("SUM is not defined on STR (VARCHAR)");
      return in == T::F64 ? T::F64 : T::I64;
    case Fn::Avg:
      if (in == T::STR) throw std::invalid_argument("AVG is not defined on STR (VARCHAR)");
      return T::F64;
    case Fn::Min:
    case Fn::Max: return in;
  }
  return T::I64;
}

struct AggSpecX {
  Fn f;
  uint32_t col;
};

// Fold one value into a cell (ops/aggregate.cpp:118-155). STR MIN/MAX compare
// by VALUE through the owned dict (ops/aggregate.cpp:191-202).
void scatter(Cell& c, Fn f, const Col* col, uint64_t p, Dict* owned) {
  if (f == Fn::CountStar) {
    ++c.cnt;
    return;
  }
  const bool v = col->valid(p);
  if (f == Fn::Count) {
    if (v) ++c.cnt;
    return;
  }
  if (!v) return;
  if (col->type == T::STR) {  // MIN/MAX(str)
    const std::string_view s = col->str(col->ival(p));
    if (c.cnt == 0) {
      c.i = owned->intern(s);
    } else {
      const std::string& cur = owned->vals[static_cast<size_t>(c.i)];
      const bool take = (f == Fn::Min) ? (s < std::string_view(cur)) : (s > std::string_view(cur));
      if (take) c.i = owned->intern(s);
    }
    ++c.cnt;
    return;
  }
  const bool isf = col->type == T::F64;
  switch (f) {
    case Fn::Sum:
    case Fn::Avg:
      if (isf) c.d += col->fval(p);
      else c.i += col->ival(p);
      ++c.cnt;
      return;
    case Fn::Min:
      if (isf) c.d = min_total(c.d, col->fval(p));
      else c.i = std::min(c.i, col->ival(p));
      ++c.cnt;
      return;
    case Fn::Max:
      if (isf) c.d = max_total(c.d, col->fval(p));
      else c.i = std::max(c.i, col->ival(p));
      ++c.cnt;
      return;
    default: return;
  }
}

// Finalise one cell into a result column (ops/agg_internal.h:169-229).
void write_cell(ResCol& out, Fn f, T in, const Cell& c) {
  const T rt = out.type;
  switch (f) {
    case Fn::CountStar:
    case Fn::Count:
      out.i.push_back(c.cnt);
      out.f.push_back(0);
      out.valid.push_back(1);
      return;
    case Fn::Sum:
    case Fn::Min:
    case Fn::Max:
      if (c.cnt == 0) {
        out.i.push_back(0);
        out.f.push_back(0);
        out.valid.push_back(0);
        return;
      }
      if (rt == T::F64) {
        out.i.push_back(0);
        out.f.push_back(c.d);
      } else if (rt == T::I32 || rt == T::STR) {
        out.i.push_back(static_cast<int32_t>(c.i));
        out.f.push_back(0);
      } else if (rt == T::BOOL) {
        out.i.push_back(c.i & 1);
        out.f.push_back(0);
      } else {
        out.i.push_back(c.i);
        out.f.push_back(0);
      }
      out.valid.push_back(1);
      return;
    case Fn::Avg:
      if (c.cnt == 0) {
        out.i.push_back(0);
        out.f.push_back(0);
        out.valid.push_back(0);
        return;
      }
      out.i.push_back(0);
      out.f.push_back((in == T::F64 ? c.d : static_cast<double>(c.i)) / static_cast<double>(c.cnt));
      out.valid.push_back(1);
      return;
  }
}

// The single-thread Aggregate operator over rows [lo, hi) of `cols`, fed in
// batches of `batch` rows. Returns a result with keys then aggregates.
std::unique_ptr<orc_result> run_aggregate(const std::vector<Col>& cols,
                                          const std::vector<uint32_t>& keys,
                                          const std::vector<AggSpecX>& aggs, uint64_t lo,
                                          uint64_t hi, uint64_t batch) {
  const size_t nk = keys.size();
  const size_t na = aggs.size();
  std::vector<T> in_types(na);
  for (size_t a = 0; a < na; ++a)
    in_types[a] = aggs[a].f == Fn::CountStar ? T::I64 : cols[aggs[a].col].type;
  auto res = std::make_unique<orc_result>();
  auto owned = std::make_shared<Dict>();

  if (nk == 0) {
    // Global path: exactly one row, even over empty input (ops/aggregate.cpp:439-458).
    std::vector<Cell> cells(na);
    for (size_t a = 0; a < na; ++a) cells[a] = init_cell(aggs[a].f);
    for (uint64_t p = lo; p < hi; ++p)
      for (size_t a = 0; a < na; ++a)
        scatter(cells[a], aggs[a].f, aggs[a].f == Fn::CountStar ? nullptr : &cols[aggs[a].col], p,
                owned.get());
    for (size_t a = 0; a < na; ++a) {
      ResCol rc;
      rc.type = result_type(aggs[a].f, in_types[a]);
      if (rc.type == T::STR) rc.dict = owned;
      write_cell(rc, aggs[a].f, in_types[a], cells[a]);
      res->cols.push_back(std::move(rc));
    }
    res->rows = 1;
    return res;
  }

  (void)batch;  // batches only bound the hash/normalise scratch in the reference
  HashTable ht(nk, /*never_match=*/false);
  std::vector<std::vector<Cell>> cells(na);
  KeyRow kr;
  kr.w.resize(nk);
  for (uint64_t p = lo; p < hi; ++p) {
    kr.nullmask = 0;
    kr.hash = kSeed;
    for (size_t j = 0; j < nk; ++j) {
      const Col& c = cols[keys[j]];
      if (!c.valid(p)) {
        kr.w[j] = kNullWord;
        kr.nullmask |= 1ull << j;
      } else if (c.type == T::STR) {
        kr.w[j] = static_cast<uint32_t>(owned->intern(c.str(c.ival(p))));
      } else {
        kr.w[j] = canon_word(c, p);
      }
      kr.hash = fold(kr.hash, kr.w[j]);
    }
    const uint32_t g = ht.insert_or_find(kr);
    if (g >= cells[0].size() || cells[0].empty()) {
      for (size_t a = 0; a < na; ++a)
        while (cells[a].size() <= g) cells[a].push_back(init_cell(aggs[a].f));
    }
    for (size_t a = 0; a < na; ++a)
      scatter(cells[a][g], aggs[a].f, aggs[a].f == Fn::CountStar ? nullptr : &cols[aggs[a].col], p,
              owned.get());
  }
  const size_t G = ht.groups();
  for (size_t j = 0; j < nk; ++j) {
    ResCol rc;
    rc.type = cols[keys[j]].type;
    if (rc.type == T::STR) rc.dict = owned;
    for (size_t g = 0; g < G; ++g) {
      const bool isnull = ht.is_null(static_cast<uint32_t>(g), j);
      const uint64_t w = ht.word(static_cast<uint32_t>(g), j);
      rc.valid.push_back(isnull ? 0 : 1);
      int64_t iv = 0;
      double fv = 0;
      if (!isnull) {  // ops/agg_internal.h:123-161
        switch (rc.type) {
          case T::I32:
          case T::STR: iv = static_cast<int32_t>(static_cast<uint32_t>(w)); break;
          case T::I64:
          case T::TS: iv = static_cast<int64_t>(w); break;
          case T::BOOL: iv = static_cast<int64_t>(w & 1ull); break;
          case T::F64: std::memcpy(&fv, &w, 8); break;
        }
      }
      rc.i.push_back(iv);
      rc.f.push_back(fv);
    }
    res->cols.push_back(std::move(rc));
  }
  for (size_t a = 0; a < na; ++a) {
    ResCol rc;
    rc.type = result_type(aggs[a].f, in_types[a]);
    if (rc.type == T::STR) rc.dict = owned;
    for (size_t g = 0; g < G; ++g) write_cell(rc, aggs[a].f, in_types[a], cells[a][g]);
    res->cols.push_back(std::move(rc));
  }
  res->rows = G;
  return res;
}

// ---------------------------------------------------------------------------
// Join (ops/join.cpp:133-299, ops/join_internal.h)
// ---------------------------------------------------------------------------
struct JoinBuild {
  std::unique_ptr<HashTable> ht;
  std::vector<std::vector<uint32_t>> group_rows;  // group id -> build rows
  std::vector<std::shared_ptr<Dict>> idmaps;      // per key position, STR only
};

KeyRow key_row(const std::vector<Col>& cols, const std::vector<uint32_t>& keys,
               const std::vector<std::shared_ptr<Dict>>& idmaps, uint64_t p, bool insert_ids) {
  KeyRow kr;
  kr.w.resize(keys.size());
  for (size_t j = 0; j < keys.size(); ++j) {
    const Col& c = cols[keys[j]];
    if (!c.valid(p)) {
      kr.w[j] = kNullWord;
      kr.nullmask |= 1ull << j;
    } else if (c.type == T::STR) {
      // STR join keys map to a value-id space shared by both sides (ops/join.cpp:48-71).
      (void)insert_ids;
      kr.w[j] = static_cast<uint32_t>(idmaps[j]->intern(c.str(c.ival(p))));
    } else {
      kr.w[j] = canon_word(c, p);
    }
    kr.hash = fold(kr.hash, kr.w[j]);
  }
  return kr;
}

JoinBuild build_join(const std::vector<Col>& build, const std::vector<uint32_t>& bkeys) {
  JoinBuild jb;
  jb.ht = std::make_unique<HashTable>(bkeys.size(), /*never_match=*/true);
  jb.idmaps.resize(bkeys.size());
  for (size_t j = 0; j < bkeys.size(); ++j)
    if (build[bkeys[j]].type == T::STR) jb.idmaps[j] = std::make_shared<Dict>();
  const uint64_t n = build.empty() ? 0 : build[0].len;
  for (uint64_t p = 0; p < n; ++p) {
    const KeyRow kr = key_row(build, bkeys, jb.idmaps, p, true);
    const uint32_t g = jb.ht->insert_or_find(kr);
    if (g >= jb.group_rows.size()) jb.group_rows.resize(g + 1);
    jb.group_rows[g].push_back(static_cast<uint32_t>(p));
  }
  return jb;
}

void push_value(ResCol& rc, const Col& c, uint64_t p, bool null_out) {
  if (null_out || !c.valid(p)) {
    rc.i.push_back(0);
    rc.f.push_back(0);
    rc.valid.push_back(0);
    return;
  }
  if (c.type == T::F64) {
    rc.i.push_back(0);
    rc.f.push_back(c.fval(p));
  } else {
    rc.i.push_back(c.ival(p));
    rc.f.push_back(0);
  }
  rc.valid.push_back(1);
}

std::shared_ptr<Dict> dict_of(const Col& c) {
  auto d = std::make_shared<Dict>();
  for (uint32_t k = 0; k < c.dict_size; ++k) {
    d->vals.emplace_back(c.dict_bytes + c.dict_off[k], c.dict_off[k + 1] - c.dict_off[k]);
  }
  return d;
}

std::vector<Col> to_cols(const orc_column* c, int n) {
  std::vector<Col> v;
  for (int i = 0; i < n; ++i) v.push_back(to_col(c[i]));
  if (!v.empty())
    for (const Col& x : v)
      if (x.len != v[0].len) throw std::invalid_argument("columns of unequal length");
  return v;
}

std::vector<AggSpecX> to_aggs(const int32_t* f, const uint32_t* c, int n, int ncols) {
  if (n <= 0) throw std::invalid_argument("aggregate needs >=1 aggregate");
  std::vector<AggSpecX> v;
  for (int i = 0; i < n; ++i) {
    if (f[i] < 0 || f[i] > 5) throw std::invalid_argument("unknown aggregate function");
    AggSpecX s{static_cast<Fn>(f[i]), c[i]};
    if (s.f != Fn::CountStar && s.col >= static_cast<uint32_t>(ncols))
      throw std::invalid_argument("aggregate input column out of range");
    v.push_back(s);
  }
  return v;
}

template <class F>
int guarded(F&& fn) {
  try {
    fn();
    return 0;
  } catch (const std::invalid_argument& e) {
    g_err = e.what();
    return -1;
  } catch (const std::overflow_error& e) {
    g_err = e.what();
    return -2;
  } catch (const std::bad_alloc&) {
    g_err = "out of memory";
    return -3;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -4;
  }
}

// ---------------------------------------------------------------------------
// Morsel-parallel CPU baseline (exec/parallel.cpp:189-599 restated).
// ---------------------------------------------------------------------------
enum class PK { CountStar, Count, SumI, SumF, MinI, MinF, MaxI, MaxF };

struct Acc {
  bool seen = false;
  int64_t i = 0;
  double f = 0;
};

struct PGroup {
  std::vector<int64_t> ki;
  std::vector<double> kf;
  std::vector<uint8_t> kvalid;
  std::vector<Acc> acc;
};

std::string key_string(const orc_result& r, size_t row, size_t nk) {
  std::string s;
  s.reserve(nk * 9);
  for (size_t k = 0; k < nk; ++k) {
    const ResCol& c = r.cols[k];
    const bool nul = !c.valid[row];
    s.push_back(nul ? char(1) : char(0));
    uint64_t bits = 0;
    if (!nul) {
      if (c.type == T::F64) {
        double d = c.f[row];
        if (d == 0.0) d = 0.0;
        std::memcpy(&bits, &d, 8);
      } else {
        bits = static_cast<uint64_t>(c.i[row]);
      }
    }
    char b[8];
    std::memcpy(b, &bits, 8);
    s.append(b, 8);
  }
  return s;
}

void fold_partial(Acc& a, const ResCol& c, size_t row, PK k) {
  const bool nul = !c.valid[row];
  switch (k) {
    case PK::CountStar:
    case PK::Count:
      a.i += c.i[row];
      a.seen = true;
      break;
    case PK::SumI:
      if (!nul) { a.i += c.i[row]; a.seen = true; }
      break;
    case PK::SumF:
      if (!nul) { a.f += c.f[row]; a.seen = true; }
      break;
    case PK::MinI:
      if (!nul) { a.i = a.seen ? std::min(a.i, c.i[row]) : c.i[row]; a.seen = true; }
      break;
    case PK::MinF:
      if (!nul) { a.f = a.seen ? min_total(a.f, c.f[row]) : c.f[row]; a.seen = true; }
      break;
    case PK::MaxI:
      if (!nul) { a.i = a.seen ? std::max(a.i, c.i[row]) : c.i[row]; a.seen = true; }
      break;
    case PK::MaxF:
      if (!nul) { a.f = a.seen ? max_total(a.f, c.f[row]) : c.f[row]; a.seen = true; }
      break;
  }
}

void merge_acc(Acc& a, const Acc& b, PK k) {
  switch (k) {
    case PK::CountStar:
    case PK::Count:
      a.i += b.i;
      a.seen = a.seen || b.seen;
      break;
    case PK::SumI:
      if (b.seen) { a.i = a.seen ? a.i + b.i : b.i; a.seen = true; }
      break;
    case PK::SumF:
      if (b.seen) { a.f = a.seen ? a.f + b.f : b.f; a.seen = true; }
      break;
    case PK::MinI:
      if (b.seen) { a.i = a.seen ? std::min(a.i, b.i) : b.i; a.seen = true; }
      break;
    case PK::MinF:
      if (b.seen) { a.f = a.seen ? std::min(a.f, b.f) : b.f; a.seen = true; }
      break;
    case PK::MaxI:
      if (b.seen) { a.i = a.seen ? std::max(a.i, b.i) : b.i; a.seen = true; }
      break;
    case PK::MaxF:
      if (b.seen) { a.f = a.seen ? std::max(a.f, b.f) : b.f; a.seen = true; }
      break;
  }
}

unsigned resolve_threads(unsigned t) {
  if (t == 0) t = std::thread::hardware_concurrency();
  return t == 0 ? 1 : t;
}

template <class Work>
void run_workers(unsigned threads, Work&& work) {
  std::vector<std::thread> pool;
  for (unsigned w = 1; w < threads; ++w) pool.emplace_back(work, w);
  work(0u);
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

uint64_t orc_hash_combine(uint64_t acc, uint64_t word) { return fold(acc, word); }

int orc_groupby(const orc_column* cols_in, int ncols, const uint32_t* key_cols, int nkeys,
                const int32_t* agg_funcs, const uint32_t* agg_cols, int naggs,
                uint64_t batch_rows, orc_result** out) {
  return guarded([&] {
    if (batch_rows == 0 || batch_rows % 64 != 0)
      throw std::invalid_argument(
          "Scan batch_size must be a positive multiple of 64 (validity word alignment)");
    if (nkeys < 0 || nkeys > 63) throw std::invalid_argument("key column count must be in [0, 63]");
    const std::vector<Col> cols = to_cols(cols_in, ncols);
    std::vector<uint32_t> keys(key_cols, key_cols + nkeys);
    for (uint32_t k : keys)
      if (k >= static_cast<uint32_t>(ncols)) throw std::invalid_argument("key column out of range");
    const std::vector<AggSpecX> aggs = to_aggs(agg_funcs, agg_cols, naggs, ncols);
    const uint64_t n = cols.empty() ? 0 : cols[0].len;
    *out = run_aggregate(cols, keys, aggs, 0, n, batch_rows).release();
  });
}

int orc_join(const orc_column* probe_in, int nprobe, const orc_column* build_in, int nbuild,
             const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
             int32_t join_type, uint64_t batch_rows, orc_result** out) {
  return guarded([&] {
    if (batch_rows == 0 || batch_rows % 64 != 0)
      throw std::invalid_argument(
          "Scan batch_size must be a positive multiple of 64 (validity word alignment)");
    if (nkeys <= 0) throw std::invalid_argument("equi-join needs >=1 key");
    const std::vector<Col> probe = to_cols(probe_in, nprobe);
    const std::vector<Col> build = to_cols(build_in, nbuild);
    std::vector<uint32_t> pk(probe_keys, probe_keys + nkeys), bk(build_keys, build_keys + nkeys);
    for (int j = 0; j < nkeys; ++j) {
      if (pk[j] >= static_cast<uint32_t>(nprobe) || bk[j] >= static_cast<uint32_t>(nbuild))
        throw std::invalid_argument("join key column out of range");
      if (probe[pk[j]].type != build[bk[j]].type)
        throw std::invalid_argument("HashJoin: join key column types must match positionally");
    }
    JoinBuild jb = build_join(build, bk);
    auto res = std::make_unique<orc_result>();
    res->cols.resize(probe.size() + build.size());
    for (size_t c = 0; c < probe.size(); ++c) {
      res->cols[c].type = probe[c].type;
      if (probe[c].type == T::STR) res->cols[c].dict = dict_of(probe[c]);
    }
    for (size_t c = 0; c < build.size(); ++c) {
      res->cols[probe.size() + c].type = build[c].type;
      if (build[c].type == T::STR) res->cols[probe.size() + c].dict = dict_of(build[c]);
    }
    const uint64_t n = probe.empty() ? 0 : probe[0].len;
    const bool left = join_type == ORC_LEFT;
    uint64_t rows = 0;
    for (uint64_t p = 0; p < n; ++p) {
      const KeyRow kr = key_row(probe, pk, jb.idmaps, p, false);
      const uint32_t g = jb.ht->find(kr);
      auto emit = [&](uint64_t brow, bool bnull) {
        for (size_t c = 0; c < probe.size(); ++c) push_value(res->cols[c], probe[c], p, false);
        for (size_t c = 0; c < build.size(); ++c)
          push_value(res->cols[probe.size() + c], build[c], bnull ? 0 : brow, bnull);
        ++rows;
      };
      if (g != kNoGroup) {
        for (uint32_t br : jb.group_rows[g]) emit(br, false);
      } else if (left) {
        emit(0, true);
      }
    }
    res->rows = rows;
    *out = res.release();
  });
}

// Tumbling window (tsx/window.cpp:305-394): the bucket lower edge
// (t / W) * W of every row (C++ truncating division, typed as the time column,
// NULL when t is NULL) becomes one more key column of an ordinary GROUP BY
// (keys..., bucket) with NULL keys grouping together -- the same table, cells
// and first-seen group order as the reference's Window.
int orc_window_tumbling(const orc_column* cols_in, int ncols, const uint32_t* key_cols, int nkeys,
                        uint32_t time_col, int64_t width, const int32_t* agg_funcs,
                        const uint32_t* agg_cols, int naggs, uint64_t batch_rows, orc_result** out) {
  return guarded([&] {
    if (batch_rows == 0 || batch_rows % 64 != 0)
      throw std::invalid_argument(
          "Scan batch_size must be a positive multiple of 64 (validity word alignment)");
    std::vector<Col> cols = to_cols(cols_in, ncols);
    if (time_col >= static_cast<uint32_t>(ncols)) throw std::invalid_argument("time column out of range");
    const T tt = cols[time_col].type;
    if (tt != T::I32 && tt != T::I64 && tt != T::TS)
      throw std::invalid_argument("Window: time column must be I32/I64/TS");
    if (width <= 0) throw std::invalid_argument("Window: tumbling width W must be > 0");
    std::vector<uint32_t> keys(key_cols, key_cols + nkeys);
    for (uint32_t k : keys) {
      if (k >= static_cast<uint32_t>(ncols)) throw std::invalid_argument("key column out of range");
      if (cols[k].type == T::STR)
        throw std::invalid_argument("Window: STR partition keys are not supported (out of grammar)");
    }
    const std::vector<AggSpecX> aggs = to_aggs(agg_funcs, agg_cols, naggs, ncols);
    for (const AggSpecX& a : aggs)
      if (a.f != Fn::CountStar && cols[a.col].type == T::STR)
        throw std::invalid_argument("Window: STR aggregate inputs are not supported (out of grammar)");
    const Col& tc = cols[time_col];
    const uint64_t n = tc.len;
    const size_t w = (tt == T::I32) ? 4 : 8;
    std::vector<uint8_t> bdata(std::max<uint64_t>(n, 1) * w, 0);
    std::vector<uint64_t> bvalid((n + 63) / 64 + 1, ~0ull);
    for (uint64_t p = 0; p < n; ++p) {
      if (!tc.valid(p)) {
        bvalid[p >> 6] &= ~(1ull << (p & 63));
        continue;
      }
      const int64_t t = tc.ival(p);
      const int64_t b = (t / width) * width;
      if (w == 4) {
        const int32_t v = static_cast<int32_t>(b);
        std::memcpy(bdata.data() + p * 4, &v, 4);
      } else {
        std::memcpy(bdata.data() + p * 8, &b, 8);
      }
    }
    Col bc = tc;
    bc.data = bdata.data();
    bc.validity = bvalid.data();
    bc.all_valid = false;
    cols.push_back(bc);
    keys.push_back(static_cast<uint32_t>(ncols));
    *out = run_aggregate(cols, keys, aggs, 0, n, batch_rows).release();
  });
}

// Backward as-of join (tsx/asof.cpp): build rows with non-NULL keys and a
// non-NULL time are grouped by key (kNeverMatch; STR keys by value, as the
// hash join) and ordered by time stably (tsx/asof.cpp:158-219, the sorted
// build lists); each probe row with non-NULL keys and time t takes the last
// build row of its key whose time is <= t (tsx/asof.cpp:269-296), kept only
// when t - tb <= tolerance in uint64 arithmetic if a tolerance is set
// (tsx/asof.cpp:283-293). INNER drops unmatched probe rows, LEFT emits them
// with NULL build columns. Rows are emitted in probe order.
int orc_asof_join(const orc_column* probe_in, int nprobe, const orc_column* build_in, int nbuild,
                  const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
                  uint32_t probe_time, uint32_t build_time, int32_t asof_type, int32_t has_tol,
                  int64_t tol, orc_result** out) {
  return guarded([&] {
    const std::vector<Col> probe = to_cols(probe_in, nprobe);
    const std::vector<Col> build = to_cols(build_in, nbuild);
    if (probe_time >= static_cast<uint32_t>(nprobe) || build_time >= static_cast<uint32_t>(nbuild))
      throw std::invalid_argument("time column out of range");
    auto ts_ok = [](T t) { return t == T::I32 || t == T::I64 || t == T::TS; };
    if (!ts_ok(probe[probe_time].type) || !ts_ok(build[build_time].type))
      throw std::invalid_argument("AsofJoin: time columns must be I32/I64/TS");
    std::vector<uint32_t> pk(probe_keys, probe_keys + nkeys), bk(build_keys, build_keys + nkeys);
    for (int j = 0; j < nkeys; ++j) {
      if (pk[j] >= static_cast<uint32_t>(nprobe) || bk[j] >= static_cast<uint32_t>(nbuild))
        throw std::invalid_argument("join key column out of range");
      if (probe[pk[j]].type != build[bk[j]].type)
        throw std::invalid_argument("AsofJoin: key column types must match positionally");
    }
    const Col& ptc = probe[probe_time];
    const Col& btc = build[build_time];
    // Build: group id per key tuple, rows per group as (time, row) by time.
    HashTable ht(bk.size(), /*never_match=*/true);
    std::vector<std::shared_ptr<Dict>> idmaps(bk.size());
    for (size_t j = 0; j < bk.size(); ++j)
      if (build[bk[j]].type == T::STR) idmaps[j] = std::make_shared<Dict>();
    std::vector<std::vector<std::pair<int64_t, uint32_t>>> groups(nkeys == 0 ? 1 : 0);
    const uint64_t nb = build.empty() ? 0 : build[0].len;
    for (uint64_t r = 0; r < nb; ++r) {
      if (!btc.valid(r)) continue;
      uint32_t g = 0;
      if (nkeys > 0) {
        const KeyRow kr = key_row(build, bk, idmaps, r, true);
        if (kr.nullmask) continue;
        g = ht.insert_or_find(kr);
        if (g >= groups.size()) groups.resize(g + 1);
      }
      groups[g].emplace_back(btc.ival(r), static_cast<uint32_t>(r));
    }
    for (auto& v : groups)
      std::stable_sort(v.begin(), v.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    auto res = std::make_unique<orc_result>();
    res->cols.resize(probe.size() + build.size());
    for (size_t c = 0; c < probe.size(); ++c) {
      res->cols[c].type = probe[c].type;
      if (probe[c].type == T::STR) res->cols[c].dict = dict_of(probe[c]);
    }
    for (size_t c = 0; c < build.size(); ++c) {
      res->cols[probe.size() + c].type = build[c].type;
      if (build[c].type == T::STR) res->cols[probe.size() + c].dict = dict_of(build[c]);
    }
    const uint64_t np = probe.empty() ? 0 : probe[0].len;
    const bool left = asof_type == ORC_LEFT;
    uint64_t rows = 0;
    for (uint64_t p = 0; p < np; ++p) {
      int64_t match = -1;
      if (ptc.valid(p)) {
        uint32_t g = 0;
        bool ok = true;
        if (nkeys > 0) {
          const KeyRow kr = key_row(probe, pk, idmaps, p, false);
          g = kr.nullmask ? kNoGroup : ht.find(kr);
          ok = g != kNoGroup && g < groups.size();
        }
        if (ok) {
          const auto& v = groups[g];
          const int64_t t = ptc.ival(p);
          auto it = std::upper_bound(v.begin(), v.end(), t,
                                     [](int64_t x, const std::pair<int64_t, uint32_t>& e) { return x < e.first; });
          if (it != v.begin()) {
            --it;
            if (!has_tol || static_cast<uint64_t>(t) - static_cast<uint64_t>(it->first) <=
                                static_cast<uint64_t>(tol))
              match = it->second;
          }
        }
      }
      if (match < 0 && !left) continue;
      for (size_t c = 0; c < probe.size(); ++c) push_value(res->cols[c], probe[c], p, false);
      for (size_t c = 0; c < build.size(); ++c)
        push_value(res->cols[probe.size() + c], build[c], match < 0 ? 0 : static_cast<uint64_t>(match), match < 0);
      ++rows;
    }
    res->rows = rows;
    *out = res.release();
  });
}

int orc_join_count_sum(const orc_column* probe_key, const orc_column* probe_val,
                       const orc_column* build_key, uint64_t batch_rows, int64_t* out_count,
                       int64_t* out_sum, int32_t* sum_valid) {
  return guarded([&] {
    (void)batch_rows;
    const Col pk = to_col(*probe_key), pv = to_col(*probe_val), bk = to_col(*build_key);
    if (pk.type != bk.type) throw std::invalid_argument("join key column types must match");
    if (pk.len != pv.len) throw std::invalid_argument("columns of unequal length");
    // Multiplicity per distinct build key; NULL build keys never match.
    HashTable ht(1, /*never_match=*/true);
    std::vector<int64_t> mult;
    std::vector<Col> bcols{bk};
    std::vector<uint32_t> keys{0};
    std::vector<std::shared_ptr<Dict>> idm(1);
    for (uint64_t p = 0; p < bk.len; ++p) {
      const KeyRow kr = key_row(bcols, keys, idm, p, true);
      if (kr.nullmask) continue;  // a dead group: never probeable
      const uint32_t g = ht.insert_or_find(kr);
      if (g >= mult.size()) mult.resize(g + 1, 0);
      ++mult[g];
    }
    std::vector<Col> pcols{pk};
    int64_t cnt = 0, sum = 0;
    bool seen = false;
    for (uint64_t p = 0; p < pk.len; ++p) {
      const KeyRow kr = key_row(pcols, keys, idm, p, false);
      const uint32_t g = ht.find(kr);
      if (g == kNoGroup) continue;
      cnt += mult[g];
      if (pv.valid(p)) {
        sum += pv.ival(p) * mult[g];
        seen = true;
      }
    }
    *out_count = cnt;
    *out_sum = sum;
    *sum_valid = seen ? 1 : 0;
  });
}

int orc_parallel_groupby(const orc_column* cols_in, int ncols, const uint32_t* key_cols,
                         int nkeys, const int32_t* agg_funcs, const uint32_t* agg_cols, int naggs,
                         unsigned threads, uint64_t morsel_rows, orc_result** out) {
  return guarded([&] {
    if (morsel_rows == 0 || morsel_rows % 64 != 0)
      throw std::invalid_argument("ParallelConfig.morsel_rows must be a multiple of 64");
    const std::vector<Col> cols = to_cols(cols_in, ncols);
    const std::vector<uint32_t> keys(key_cols, key_cols + nkeys);
    const std::vector<AggSpecX> aggs = to_aggs(agg_funcs, agg_cols, naggs, ncols);
    for (const Col& c : cols)
      if (c.type == T::STR) throw std::invalid_argument("parallel baseline: STR not supported");
    // Partial specs: AVG -> SUM + COUNT (exec/parallel.cpp:189-246).
    std::vector<AggSpecX> specs;
    std::vector<PK> kinds;
    struct OMap { Fn f; int v; int c; T rt; };
    std::vector<OMap> omap;
    for (const AggSpecX& a : aggs) {
      const T in = a.f == Fn::CountStar ? T::I64 : cols[a.col].type;
      const bool fl = in == T::F64;
      switch (a.f) {
        case Fn::CountStar:
          specs.push_back(a); kinds.push_back(PK::CountStar);
          omap.push_back({a.f, (int)specs.size() - 1, -1, T::I64}); break;
        case Fn::Count:
          specs.push_back(a); kinds.push_back(PK::Count);
          omap.push_back({a.f, (int)specs.size() - 1, -1, T::I64}); break;
        case Fn::Sum:
          specs.push_back(a); kinds.push_back(fl ? PK::SumF : PK::SumI);
          omap.push_back({a.f, (int)specs.size() - 1, -1, fl ? T::F64 : T::I64}); break;
        case Fn::Min:
          specs.push_back(a); kinds.push_back(fl ? PK::MinF : PK::MinI);
          omap.push_back({a.f, (int)specs.size() - 1, -1, in}); break;
        case Fn::Max:
          specs.push_back(a); kinds.push_back(fl ? PK::MaxF : PK::MaxI);
          omap.push_back({a.f, (int)specs.size() - 1, -1, in}); break;
        case Fn::Avg: {
          specs.push_back({Fn::Sum, a.col}); kinds.push_back(fl ? PK::SumF : PK::SumI);
          const int s = (int)specs.size() - 1;
          specs.push_back({Fn::Count, a.col}); kinds.push_back(PK::Count);
          omap.push_back({a.f, s, (int)specs.size() - 1, T::F64}); break;
        }
      }
    }
    const size_t nk = keys.size();
    const uint64_t total = cols.empty() ? 0 : cols[0].len;
    std::vector<std::pair<uint64_t, uint64_t>> morsels;
    for (uint64_t s = 0; s < total; s += morsel_rows) morsels.push_back({s, std::min(s + morsel_rows, total)});
    if (morsels.empty()) morsels.push_back({0, 0});
    const unsigned T_ = resolve_threads(threads);
    std::vector<std::unordered_map<std::string, PGroup>> per(T_);
    std::atomic<size_t> cursor{0};
    std::mutex err_mu;
    std::string err;
    run_workers(T_, [&](unsigned w) {
      try {
        auto& map = per[w];
        size_t mi;
        while ((mi = cursor.fetch_add(1)) < morsels.size()) {
          auto pr = run_aggregate(cols, keys, specs, morsels[mi].first, morsels[mi].second, 2048);
          for (size_t row = 0; row < pr->rows; ++row) {
            const std::string key = key_string(*pr, row, nk);
            auto it = map.find(key);
            if (it == map.end()) {
              PGroup g;
              for (size_t k = 0; k < nk; ++k) {
                g.ki.push_back(pr->cols[k].i[row]);
                g.kf.push_back(pr->cols[k].f[row]);
                g.kvalid.push_back(pr->cols[k].valid[row]);
              }
              g.acc.resize(kinds.size());
              it = map.emplace(key, std::move(g)).first;
            }
            for (size_t j = 0; j < kinds.size(); ++j)
              fold_partial(it->second.acc[j], pr->cols[nk + j], row, kinds[j]);
          }
        }
      } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(err_mu);
        err = e.what();
      }
    });
    if (!err.empty()) throw std::runtime_error(err);
    std::unordered_map<std::string, PGroup> merged;
    for (auto& wm : per)
      for (auto& kv : wm) {
        auto it = merged.find(kv.first);
        if (it == merged.end()) {
          merged.emplace(kv.first, std::move(kv.second));
          continue;
        }
        for (size_t j = 0; j < kinds.size(); ++j) merge_acc(it->second.acc[j], kv.second.acc[j], kinds[j]);
      }
    auto res = std::make_unique<orc_result>();
    for (size_t k = 0; k < nk; ++k) res->cols.push_back(ResCol{cols[keys[k]].type, {}, {}, {}, nullptr});
    for (const OMap& om : omap) res->cols.push_back(ResCol{om.rt, {}, {}, {}, nullptr});
    for (auto& kv : merged) {
      const PGroup& g = kv.second;
      for (size_t k = 0; k < nk; ++k) {
        res->cols[k].i.push_back(g.ki[k]);
        res->cols[k].f.push_back(g.kf[k]);
        res->cols[k].valid.push_back(g.kvalid[k]);
      }
      for (size_t o = 0; o < omap.size(); ++o) {
        ResCol& rc = res->cols[nk + o];
        const Acc& a = g.acc[omap[o].v];
        int64_t iv = 0;
        double fv = 0;
        uint8_t ok = 1;
        switch (omap[o].f) {
          case Fn::CountStar:
          case Fn::Count: iv = a.i; break;
          case Fn::Sum:
          case Fn::Min:
          case Fn::Max:
            if (!a.seen) ok = 0;
            else if (omap[o].rt == T::F64) fv = a.f;
            else iv = a.i;
            break;
          case Fn::Avg: {
            const Acc& c = g.acc[omap[o].c];
            if (c.i > 0)
              fv = (kinds[omap[o].v] == PK::SumF ? a.f : static_cast<double>(a.i)) / static_cast<double>(c.i);
            else ok = 0;
            break;
          }
        }
        rc.i.push_back(iv);
        rc.f.push_back(fv);
        rc.valid.push_back(ok);
      }
    }
    res->rows = merged.size();
    *out = res.release();
  });
}

int orc_parallel_join_count_sum(const orc_column* probe_key, const orc_column* probe_val,
                                const orc_column* build_key, const orc_column* build_val,
                                unsigned threads, uint64_t morsel_rows, int64_t* out_count,
                                int64_t* out_sum, int32_t* sum_valid) {
  return guarded([&] {
    if (morsel_rows == 0 || morsel_rows % 64 != 0)
      throw std::invalid_argument("ParallelConfig.morsel_rows must be a multiple of 64");
    const std::vector<Col> probe{to_col(*probe_key), to_col(*probe_val)};
    const std::vector<Col> build{to_col(*build_key), to_col(*build_val)};
    if (probe[0].type != build[0].type) throw std::invalid_argument("join key column types must match");
    const uint64_t total = probe[0].len;
    std::vector<std::pair<uint64_t, uint64_t>> morsels;
    for (uint64_t s = 0; s < total; s += morsel_rows) morsels.push_back({s, std::min(s + morsel_rows, total)});
    if (morsels.empty()) morsels.push_back({0, 0});
    const unsigned T_ = resolve_threads(threads);
    std::vector<Acc> cnt(T_), sum(T_);
    std::atomic<size_t> cursor{0};
    std::mutex err_mu;
    std::string err;
    const std::vector<uint32_t> pk{0}, bk{0};
    run_workers(T_, [&](unsigned w) {
      try {
        size_t mi;
        while ((mi = cursor.fetch_add(1)) < morsels.size()) {
          // Each morsel's private tree rebuilds the whole build side
          // (exec/parallel.cpp:101-105), then probes its morsel and feeds the
          // joined rows (probe cols then build cols, ops/join.cpp:260-299) to
          // the global COUNT(*)/SUM aggregate.
          JoinBuild jb = build_join(build, bk);
          std::vector<int64_t> out_pv, out_bk, out_bv;
          std::vector<uint8_t> out_pvv;
          auto flush = [&]() {
            for (size_t r = 0; r < out_pv.size(); ++r) {
              cnt[w].i += 1;
              cnt[w].seen = true;
              if (out_pvv[r]) {
                sum[w].i += out_pv[r];
                sum[w].seen = true;
              }
            }
            out_pv.clear(); out_pvv.clear(); out_bk.clear(); out_bv.clear();
          };
          for (uint64_t p = morsels[mi].first; p < morsels[mi].second; ++p) {
            const KeyRow kr = key_row(probe, pk, jb.idmaps, p, false);
            const uint32_t g = jb.ht->find(kr);
            if (g == kNoGroup) continue;
            for (uint32_t br : jb.group_rows[g]) {
              out_pv.push_back(probe[1].valid(p) ? probe[1].ival(p) : 0);
              out_pvv.push_back(probe[1].valid(p) ? 1 : 0);
              out_bk.push_back(build[0].ival(br));
              out_bv.push_back(build[1].valid(br) ? build[1].ival(br) : 0);
              if (out_pv.size() == 2048) flush();
            }
          }
          flush();
        }
      } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(err_mu);
        err = e.what();
      }
    });
    if (!err.empty()) throw std::runtime_error(err);
    int64_t c = 0, s = 0;
    bool seen = false;
    for (unsigned w = 0; w < T_; ++w) {
      c += cnt[w].i;
      if (sum[w].seen) { s += sum[w].i; seen = true; }
    }
    *out_count = c;
    *out_sum = s;
    *sum_valid = seen ? 1 : 0;
  });
}

uint64_t orc_result_rows(const orc_result* r) { return r ? r->rows : 0; }
int orc_result_cols(const orc_result* r) { return r ? static_cast<int>(r->cols.size()) : 0; }
int32_t orc_result_type(const orc_result* r, int col) {
  if (!r || col < 0 || col >= static_cast<int>(r->cols.size())) return -1;
  return static_cast<int32_t>(r->cols[col].type);
}
int orc_result_fetch(const orc_result* r, int col, int64_t* ivals, double* fvals, uint8_t* valid) {
  if (!r || col < 0 || col >= static_cast<int>(r->cols.size())) {
    g_err = "result column out of range";
    return -1;
  }
  const ResCol& c = r->cols[col];
  if (ivals && !c.i.empty()) std::memcpy(ivals, c.i.data(), c.i.size() * 8);
  if (fvals && !c.f.empty()) std::memcpy(fvals, c.f.data(), c.f.size() * 8);
  if (valid && !c.valid.empty()) std::memcpy(valid, c.valid.data(), c.valid.size());
  return 0;
}
int orc_result_str(const orc_result* r, int col, int64_t code, const char** s, uint64_t* len) {
  if (!r || col < 0 || col >= static_cast<int>(r->cols.size()) || !r->cols[col].dict) {
    g_err = "not a STR result column";
    return -1;
  }
  const Dict& d = *r->cols[col].dict;
  if (code < 0 || static_cast<size_t>(code) >= d.vals.size()) {
    g_err = "STR code out of range";
    return -1;
  }
  *s = d.vals[static_cast<size_t>(code)].data();
  *len = d.vals[static_cast<size_t>(code)].size();
  return 0;
}
void orc_result_free(orc_result* r) { delete r; }

}  // extern "C"
