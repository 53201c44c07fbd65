// Drives qe::gpu::GpuAggregate / GpuHashJoin / GpuWindow / GpuAsofJoin through the reference's pull
// interface (Operator::open/next/close, Batch/Column views) exactly as a plan
// tree would, and checks the drained results against values computed here on
// the CPU and against expectations written in the reference's own tests.
// Exit code 0 = all checks passed.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../query-engine_gb300/host/gpu_operators.h"

using namespace qe;

static std::atomic<int> g_fail{0};  // checks may fail on several threads
#define CHECK(c)                                                        \
  do {                                                                  \
    if (!(c)) {                                                         \
      std::fprintf(stderr, "CHECK failed at line %d: %s\n", __LINE__, #c); \
      ++g_fail;                                                         \
    }                                                                   \
  } while (0)

// A columnar table and a Scan over it: zero-copy windows of `batch` rows
// (a multiple of 64), validity re-based by whole words (ops/scan.cpp:27-64).
struct TestTable {
  Schema schema;
  std::vector<gpu::HostColumn> cols;
};

class TestScan : public Operator {
 public:
  TestScan(const TestTable& t, std::size_t batch) : t_(t), batch_(batch) {}
  void open() override { cur_ = 0; }
  std::optional<Batch> next() override {
    const std::size_t n = t_.cols.empty() ? 0 : t_.cols[0].len;
    if (cur_ >= n) return std::nullopt;
    const std::size_t m = std::min(batch_, n - cur_);
    Batch b;
    for (const auto& c : t_.cols) {
      Column v = c.view();
      v.len = m;
      v.data += cur_ * byte_width(c.type);
      if (!v.all_valid) v.validity += cur_ / 64;
      b.cols.push_back(v);
    }
    b.sel = nullptr;
    b.row_count = m;
    cur_ += m;
    return b;
  }
  void close() override {}
  Schema output_schema() const override { return t_.schema; }

 private:
  const TestTable& t_;
  std::size_t batch_, cur_ = 0;
};

// Emits prepared batches that carry selection vectors and their own dicts.
class BatchSource : public Operator {
 public:
  Schema schema;
  std::vector<std::vector<gpu::HostColumn>> batches;
  std::vector<std::vector<uint32_t>> sels;  // empty => dense
  void open() override { i_ = 0; }
  std::optional<Batch> next() override {
    if (i_ >= batches.size()) return std::nullopt;
    Batch b;
    for (const auto& c : batches[i_]) b.cols.push_back(c.view());
    if (!sels[i_].empty()) {
      sv_ = {sels[i_].data(), sels[i_].size()};
      b.sel = &sv_;
      b.row_count = sels[i_].size();
    } else {
      b.sel = nullptr;
      b.row_count = batches[i_][0].len;
    }
    ++i_;
    return b;
  }
  void close() override {}
  Schema output_schema() const override { return schema; }

 private:
  std::size_t i_ = 0;
  SelectionVector sv_{nullptr, 0};
};

template <class T>
gpu::HostColumn make_col(Type t, const std::vector<T>& v, const std::vector<std::size_t>& nulls = {}) {
  gpu::HostColumn c;
  c.type = t;
  c.len = v.size();
  c.data.resize(std::max<std::size_t>(1, v.size() * sizeof(T)));
  if (!v.empty()) std::memcpy(c.data.data(), v.data(), v.size() * sizeof(T));
  if (!nulls.empty()) {
    c.validity.assign(validity::words(v.size()), ~0ull);
    for (auto k : nulls) validity::set_bit(c.validity.data(), k, false);
  }
  return c;
}

gpu::HostColumn str_col(const std::vector<std::string>& dict, const std::vector<int32_t>& codes) {
  gpu::HostColumn c = make_col(Type::STR, codes);
  auto d = std::make_shared<StringDict>();
  for (const auto& s : dict) d->intern(s);
  c.dict = d;
  return c;
}

struct Cell {
  bool null = true;
  int64_t i = 0;
  double f = 0;
  std::string s;
  bool operator<(const Cell& o) const { return std::tie(null, i, f, s) < std::tie(o.null, o.i, o.f, o.s); }
};
using Row = std::vector<Cell>;

std::vector<Row> drain(Operator& op) {
  std::vector<Row> rows;
  const Schema sch = op.output_schema();
  op.open();
  while (auto b = op.next()) {
    CHECK(b->row_count >= 1 && b->row_count <= 2048);
    CHECK(b->cols.size() == sch.fields.size());
    for (std::size_t k = 0; k < b->row_count; ++k) {
      const uint32_t p = b->sel ? b->sel->idx[k] : static_cast<uint32_t>(k);
      Row r;
      for (const Column& c : b->cols) {
        Cell x;
        x.null = !(c.all_valid || validity::get_bit(c.validity, p));
        if (!x.null) {
          switch (c.type) {
            case Type::I32: x.i = reinterpret_cast<const int32_t*>(c.data)[p]; break;
            case Type::I64:
            case Type::TS: x.i = reinterpret_cast<const int64_t*>(c.data)[p]; break;
            case Type::BOOL: x.i = reinterpret_cast<const uint8_t*>(c.data)[p]; break;
            case Type::F64: x.f = reinterpret_cast<const double*>(c.data)[p]; break;
            case Type::STR: x.s = std::string(c.dict->at(reinterpret_cast<const int32_t*>(c.data)[p])); break;
          }
        }
        r.push_back(x);
      }
      rows.push_back(r);
    }
  }
  CHECK(!op.next().has_value());  // stays exhausted
  op.close();
  return rows;
}

void test_aggregate_edge_table() {
  // tests/aggregate_differential_test.cpp edge table of the reference.
  TestTable t;
  t.schema.fields = {{"c0", Type::I32}, {"c1", Type::I32}, {"c2", Type::F64}};
  t.cols.push_back(make_col<int32_t>(Type::I32, {1, 1, 2, 2, 3, 1, 2, 3, 0, 0}, {8, 9}));
  t.cols.push_back(make_col<int32_t>(Type::I32, {10, 20, 30, 40, 50, 60, 70, 80, 90, 100}, {0}));
  t.cols.push_back(make_col<double>(Type::F64, {1.5, 2.5, 3.5, 4.5, 5.5, 6.5, 7.5, 8.5, 9.5, 10.5}, {2}));
  for (std::size_t bs : {64, 256, 2048}) {
    gpu::GpuAggregate agg(std::make_unique<TestScan>(t, bs), {0},
                          {AggSpec::count_star("cs"), AggSpec::count(1, "c1"), AggSpec::sum(1, "s1"),
                           AggSpec::min(1, "mn"), AggSpec::max(1, "mx"), AggSpec::avg(1, "av"),
                           AggSpec::sum(2, "s2"), AggSpec::avg(2, "a2")});
    const Schema s = agg.output_schema();
    CHECK(s.fields.size() == 9 && s.fields[0].second == Type::I32 && s.fields[3].second == Type::I64 &&
          s.fields[4].second == Type::I32 && s.fields[6].second == Type::F64);
    std::map<int64_t, Row> by;
    Row null_group;
    for (Row& r : drain(agg)) {
      if (r[0].null) null_group = r;
      else by[r[0].i] = r;
    }
    CHECK(by.size() == 3 && !null_group.empty());
    // key 1: rows 0 (c1 NULL), 1, 5 -> COUNT(*)=3, COUNT(c1)=2, SUM=80, MIN=20, MAX=60, AVG=40
    CHECK(by[1][1].i == 3 && by[1][2].i == 2 && by[1][3].i == 80 && by[1][4].i == 20 && by[1][5].i == 60);
    CHECK(std::fabs(by[1][6].f - 40.0) < 1e-12);
    // key 2: rows 2 (c2 NULL), 3, 6 -> SUM(c2) = 4.5 + 7.5
    CHECK(by[2][1].i == 3 && std::fabs(by[2][7].f - 12.0) < 1e-12 && std::fabs(by[2][8].f - 6.0) < 1e-12);
    // NULL key group: rows 8, 9
    CHECK(null_group[1].i == 2 && null_group[3].i == 190);
  }
}

void test_aggregate_random_vs_cpu() {
  std::mt19937_64 rng(42);
  const std::size_t n = 100000;
  std::vector<int64_t> k(n);
  std::vector<double> v(n);
  std::vector<std::size_t> nulls;
  for (std::size_t i = 0; i < n; ++i) {
    k[i] = static_cast<int64_t>(rng() % 5000) - 2500;
    v[i] = static_cast<double>(rng() % 100000) / 7.0;
    if (rng() % 20 == 0) nulls.push_back(i);
  }
  TestTable t;
  t.schema.fields = {{"k", Type::I64}, {"v", Type::F64}};
  t.cols.push_back(make_col(Type::I64, k));
  t.cols.push_back(make_col(Type::F64, v, nulls));
  std::vector<bool> isnull(n, false);
  for (auto i : nulls) isnull[i] = true;
  std::map<int64_t, std::tuple<int64_t, double, double, int64_t>> exp;  // count, sum, max, nn
  for (std::size_t i = 0; i < n; ++i) {
    auto& e = exp[k[i]];
    std::get<0>(e)++;
    if (!isnull[i]) {
      std::get<1>(e) += v[i];
      std::get<2>(e) = std::get<3>(e) ? std::max(std::get<2>(e), v[i]) : v[i];
      std::get<3>(e)++;
    }
  }
  gpu::GpuAggregate agg(std::make_unique<TestScan>(t, 2048), {0},
                        {AggSpec::count_star("n"), AggSpec::sum(1, "s"), AggSpec::max(1, "m")});
  std::size_t groups = 0;
  for (Row& r : drain(agg)) {
    ++groups;
    const auto& e = exp[r[0].i];
    CHECK(r[1].i == std::get<0>(e));
    CHECK(std::fabs(r[2].f - std::get<1>(e)) <= 1e-9 + 1e-9 * std::fabs(std::get<1>(e)));
    CHECK(r[3].f == std::get<2>(e));
  }
  CHECK(groups == exp.size());
}

void test_aggregate_str_by_value_and_selection() {
  // Two batches with different dictionaries and a selection vector.
  BatchSource* src = new BatchSource();
  src->schema.fields = {{"sym", Type::STR}, {"q", Type::I64}};
  src->batches.push_back({str_col({"AAPL", "MSFT", "GOOG"}, {0, 1, 2, 0}), make_col<int64_t>(Type::I64, {1, 2, 3, 4})});
  src->sels.push_back({});
  src->batches.push_back(
      {str_col({"GOOG", "AAPL", "IBM", "MSFT"}, {1, 0, 2, 3, 3}), make_col<int64_t>(Type::I64, {10, 30, 7, 20, 99})});
  src->sels.push_back({0, 1, 2, 3});  // row 4 (MSFT 99) is filtered out
  gpu::GpuAggregate agg(std::unique_ptr<Operator>(src), {0},
                        {AggSpec::count_star("n"), AggSpec::sum(1, "s"), AggSpec::min(0, "mn"), AggSpec::max(0, "mx")});
  std::map<std::string, Row> by;
  for (Row& r : drain(agg)) by[r[0].s] = r;
  CHECK(by.size() == 4);
  CHECK(by["AAPL"][1].i == 3 && by["AAPL"][2].i == 15);
  CHECK(by["MSFT"][1].i == 2 && by["MSFT"][2].i == 22);
  CHECK(by["GOOG"][1].i == 2 && by["GOOG"][2].i == 33);
  CHECK(by["IBM"][1].i == 1 && by["IBM"][2].i == 7 && by["IBM"][3].s == "IBM" && by["IBM"][4].s == "IBM");
}

void test_aggregate_errors_and_global_empty() {
  TestTable t;
  t.schema.fields = {{"s", Type::STR}};
  t.cols.push_back(str_col({"a"}, {}));
  bool threw = false;
  try {
    gpu::GpuAggregate agg(std::make_unique<TestScan>(t, 64), {}, {AggSpec::sum(0, "x")});
    agg.output_schema();
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);  // SUM(STR) is a type error (ops/aggregate.cpp:85-90)
  TestTable e;
  e.schema.fields = {{"v", Type::I64}};
  e.cols.push_back(make_col<int64_t>(Type::I64, {}));
  gpu::GpuAggregate g(std::make_unique<TestScan>(e, 64), {}, {AggSpec::count_star("n"), AggSpec::sum(0, "s")});
  auto rows = drain(g);
  CHECK(rows.size() == 1 && rows[0][0].i == 0 && rows[0][1].null);
}

void test_join_edge_cases() {
  // tests/join_differential_test.cpp one-key case of the reference.
  TestTable b, p;
  b.schema.fields = {{"c0", Type::I32}, {"c1", Type::I64}};
  b.cols.push_back(make_col<int32_t>(Type::I32, {1, 1, 2, 5, 5, 5}));
  b.cols.push_back(make_col<int64_t>(Type::I64, {10, 11, 20, 50, 51, 52}));
  p.schema.fields = {{"c0", Type::I32}, {"c1", Type::I64}};
  p.cols.push_back(make_col<int32_t>(Type::I32, {1, 2, 3, 5, 0}, {4}));
  p.cols.push_back(make_col<int64_t>(Type::I64, {100, 200, 300, 500, 999}));
  for (JoinType jt : {JoinType::Inner, JoinType::Left}) {
    gpu::GpuHashJoin j(std::make_unique<TestScan>(p, 64), std::make_unique<TestScan>(b, 64), {0}, {0}, jt);
    auto rows = drain(j);
    std::multiset<std::tuple<int64_t, int64_t, bool, int64_t>> got;
    for (Row& r : rows) got.insert({r[1].i, r[0].null ? -1 : r[0].i, r[3].null, r[3].null ? 0 : r[3].i});
    std::multiset<std::tuple<int64_t, int64_t, bool, int64_t>> exp = {
        {100, 1, false, 10}, {100, 1, false, 11}, {200, 2, false, 20},
        {500, 5, false, 50}, {500, 5, false, 51}, {500, 5, false, 52}};
    if (jt == JoinType::Left) {
      exp.insert({300, 3, true, 0});
      exp.insert({999, -1, true, 0});
    }
    CHECK(got == exp);
  }
  // 3000-row fan-out crosses the 2048-row output batch.
  TestTable fb, fp;
  fb.schema.fields = {{"k", Type::I32}, {"v", Type::I64}};
  std::vector<int32_t> fk(3000, 7);
  std::vector<int64_t> fv(3000);
  for (int i = 0; i < 3000; ++i) fv[i] = i;
  fb.cols.push_back(make_col(Type::I32, fk));
  fb.cols.push_back(make_col(Type::I64, fv));
  fp.schema.fields = {{"k", Type::I32}};
  fp.cols.push_back(make_col<int32_t>(Type::I32, {7, 9, 7}));
  gpu::GpuHashJoin fj(std::make_unique<TestScan>(fp, 64), std::make_unique<TestScan>(fb, 2048), {0}, {0},
                      JoinType::Inner);
  auto rows = drain(fj);
  CHECK(rows.size() == 6000);
  int64_t s = 0;
  for (Row& r : rows) s += r[2].i;
  CHECK(s == 2 * (2999LL * 3000 / 2));
  // key type mismatch is rejected like the reference (ops/join.cpp:118-122)
  TestTable m;
  m.schema.fields = {{"k", Type::I64}};
  m.cols.push_back(make_col<int64_t>(Type::I64, {1}));
  bool threw = false;
  try {
    gpu::GpuHashJoin bad(std::make_unique<TestScan>(m, 64), std::make_unique<TestScan>(fp, 64), {0}, {0},
                         JoinType::Inner);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);
}

void test_join_str_keys() {
  BatchSource* build = new BatchSource();
  build->schema.fields = {{"sym", Type::STR}, {"sector", Type::I32}};
  build->batches.push_back({str_col({"IBM", "AAPL", "MSFT"}, {0, 1, 2}), make_col<int32_t>(Type::I32, {1, 2, 3})});
  build->sels.push_back({});
  BatchSource* probe = new BatchSource();
  probe->schema.fields = {{"sym", Type::STR}};
  probe->batches.push_back({str_col({"MSFT", "GOOG", "AAPL"}, {0, 1, 2, 2})});
  probe->sels.push_back({});
  gpu::GpuHashJoin j(std::unique_ptr<Operator>(probe), std::unique_ptr<Operator>(build), {0}, {0}, JoinType::Inner);
  auto rows = drain(j);
  std::multiset<std::pair<std::string, int64_t>> got;
  for (Row& r : rows) {
    CHECK(r[0].s == r[1].s);
    got.insert({r[0].s, r[2].i});
  }
  CHECK((got == std::multiset<std::pair<std::string, int64_t>>{{"MSFT", 3}, {"AAPL", 2}, {"AAPL", 2}}));
}

void test_window_tumbling() {
  // tests/window_differential_test.cpp make_input of the reference, width 10.
  TestTable t;
  t.schema.fields = {{"c0", Type::I32}, {"c1", Type::TS}, {"c2", Type::I64}, {"c3", Type::F64}};
  t.cols.push_back(make_col<int32_t>(Type::I32, {1, 1, 1, 2, 2, 1}));
  t.cols.push_back(make_col<int64_t>(Type::TS, {0, 5, 12, 3, 21, 30}));
  t.cols.push_back(make_col<int64_t>(Type::I64, {10, 20, 30, 40, 50, 60}, {2}));
  t.cols.push_back(make_col<double>(Type::F64, {1.5, 2.5, 3.5, 4.5, 5.5, 6.5}));
  gpu::GpuWindow w(std::make_unique<TestScan>(t, 64), tsx::WindowMode::Tumbling, {0}, 1, 10,
                   {AggSpec::count_star("n"), AggSpec::sum(2, "s"), AggSpec::avg(3, "a")});
  const Schema sch = w.output_schema();
  CHECK(sch.fields.size() == 5 && sch.fields[1].first == "c1" && sch.fields[1].second == Type::TS);
  auto rows = drain(w);
  std::set<std::tuple<int64_t, int64_t, int64_t, bool, int64_t>> got;
  for (Row& r : rows) got.insert({r[0].i, r[1].i, r[2].i, r[3].null, r[3].null ? 0 : r[3].i});
  // (key, bucket, n, sum null?, sum): t 0,5 -> 0; 12 -> 10 (NULL value); 30 -> 30; key 2: 3 -> 0, 21 -> 20
  CHECK((got == std::set<std::tuple<int64_t, int64_t, int64_t, bool, int64_t>>{
                    {1, 0, 2, false, 30}, {1, 10, 1, true, 0}, {1, 30, 1, false, 60}, {2, 0, 1, false, 40},
                    {2, 20, 1, false, 50}}));
  // 5000 one-row buckets cross the 2048-row output batch; zero partition keys.
  TestTable big;
  big.schema.fields = {{"t", Type::I64}};
  std::vector<int64_t> tv(10000);
  for (int i = 0; i < 10000; ++i) tv[i] = i;
  big.cols.push_back(make_col(Type::I64, tv));
  gpu::GpuWindow wb(std::make_unique<TestScan>(big, 2048), tsx::WindowMode::Tumbling, {}, 0, 2,
                    {AggSpec::count_star("n")});
  auto brows = drain(wb);
  CHECK(brows.size() == 5000);
  int64_t total = 0;
  for (Row& r : brows) total += r[1].i;
  CHECK(total == 10000);
  // Sliding mode and bad widths / time types are rejected.
  for (int bad = 0; bad < 3; ++bad) {
    bool threw = false;
    try {
      if (bad == 0)
        gpu::GpuWindow x(std::make_unique<TestScan>(t, 64), tsx::WindowMode::Sliding, {0}, 1, 2,
                         {AggSpec::count_star("n")});
      else if (bad == 1)
        gpu::GpuWindow x(std::make_unique<TestScan>(t, 64), tsx::WindowMode::Tumbling, {0}, 1, 0,
                         {AggSpec::count_star("n")});
      else
        gpu::GpuWindow x(std::make_unique<TestScan>(t, 64), tsx::WindowMode::Tumbling, {0}, 3, 10,
                         {AggSpec::count_star("n")});
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    CHECK(threw);
  }
}

void test_asof_join() {
  // tests/asof_differential_test.cpp make_build / make_probe of the reference.
  TestTable b, p;
  b.schema.fields = {{"c0", Type::I32}, {"c1", Type::TS}, {"c2", Type::I64}};
  b.cols.push_back(make_col<int32_t>(Type::I32, {1, 1, 1, 2}));
  b.cols.push_back(make_col<int64_t>(Type::TS, {10, 20, 30, 15}));
  b.cols.push_back(make_col<int64_t>(Type::I64, {100, 200, 300, 150}));
  p.schema.fields = {{"c0", Type::I32}, {"c1", Type::TS}};
  p.cols.push_back(make_col<int32_t>(Type::I32, {1, 1, 1, 2, 3, 1}));
  p.cols.push_back(make_col<int64_t>(Type::TS, {5, 10, 25, 15, 99, 50}));
  using R = std::tuple<int64_t, int64_t, bool, int64_t>;
  for (auto type : {tsx::AsofType::Inner, tsx::AsofType::Left}) {
    for (int tol = 0; tol < 2; ++tol) {
      std::optional<int64_t> t;
      if (tol) t = 10;
      gpu::GpuAsofJoin j(std::make_unique<TestScan>(p, 64), std::make_unique<TestScan>(b, 64), {0}, {0}, 1, 1, type,
                         t);
      CHECK(j.output_schema().fields.size() == 5);
      auto rows = drain(j);
      std::multiset<R> got;
      for (Row& r : rows) got.insert({r[0].i, r[1].i, r[4].null, r[4].null ? 0 : r[4].i});
      // (1,5) precedes every build row; (1,10) takes the equal time; with
      // tolerance 10, (1,50) -> t30 is 20 back and is dropped.
      std::multiset<R> exp = {{1, 10, false, 100}, {2, 15, false, 150}, {1, 25, false, 200}};
      if (!tol) exp.insert({1, 50, false, 300});
      if (type == tsx::AsofType::Left) {
        exp.insert({1, 5, true, 0});
        exp.insert({3, 99, true, 0});
        if (tol) exp.insert({1, 50, true, 0});
      }
      CHECK(got == exp);
    }
  }
  // Zero partition keys, and a probe side of 5000 rows crossing output batches.
  TestTable gb, gp;
  gb.schema.fields = {{"t", Type::TS}, {"v", Type::I64}};
  gb.cols.push_back(make_col<int64_t>(Type::TS, {10, 20, 30}));
  gb.cols.push_back(make_col<int64_t>(Type::I64, {100, 200, 300}));
  gp.schema.fields = {{"t", Type::TS}};
  std::vector<int64_t> pt(5000);
  for (int i = 0; i < 5000; ++i) pt[i] = i % 40;
  gp.cols.push_back(make_col(Type::TS, pt));
  gpu::GpuAsofJoin g(std::make_unique<TestScan>(gp, 2048), std::make_unique<TestScan>(gb, 64), {}, {}, 0, 0,
                     tsx::AsofType::Inner);
  auto rows = drain(g);
  int64_t s = 0;
  for (Row& r : rows) s += r[2].i;
  // per 40 probe times: 10 match t10 (100), 10 t20 (200), 10 t30 (300), 10 none
  CHECK(rows.size() == 3750);
  CHECK(s == 125 * (10 * 100 + 10 * 200 + 10 * 300));
  bool threw = false;
  try {
    TestTable f;
    f.schema.fields = {{"k", Type::I32}, {"t", Type::F64}};
    f.cols.push_back(make_col<int32_t>(Type::I32, {1}));
    f.cols.push_back(make_col<double>(Type::F64, {1.0}));
    gpu::GpuAsofJoin bad(std::make_unique<TestScan>(f, 64), std::make_unique<TestScan>(b, 64), {0}, {0}, 1, 1,
                         tsx::AsofType::Inner);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);
}

// A deterministic multi-batch source: dictionaries that differ per batch, a
// selection vector, NULLs in every column type.
std::unique_ptr<BatchSource> mixed_source(std::size_t batches, std::size_t rows_per_batch) {
  auto src = std::make_unique<BatchSource>();
  src->schema.fields = {{"sym", Type::STR}, {"k", Type::I64}, {"v", Type::F64}, {"q", Type::I32}};
  std::mt19937_64 rng(7);
  const std::vector<std::string> names = {"AAPL", "MSFT", "GOOG", "IBM", "ORCL", "NVDA", "AMD", "INTC"};
  for (std::size_t b = 0; b < batches; ++b) {
    std::vector<std::string> dict(names.begin() + static_cast<long>(b % 3), names.end());
    std::vector<int32_t> codes(rows_per_batch), q(rows_per_batch);
    std::vector<int64_t> k(rows_per_batch);
    std::vector<double> v(rows_per_batch);
    std::vector<std::size_t> nk, nv, ns;
    for (std::size_t i = 0; i < rows_per_batch; ++i) {
      codes[i] = static_cast<int32_t>(rng() % dict.size());
      k[i] = static_cast<int64_t>(rng() % 3000) - 1000;
      v[i] = static_cast<double>(rng() % 100000) / 8.0;
      q[i] = static_cast<int32_t>(rng() % 1000);
      if (rng() % 31 == 0) nk.push_back(i);
      if (rng() % 17 == 0) nv.push_back(i);
      if (rng() % 23 == 0) ns.push_back(i);
    }
    gpu::HostColumn sc = str_col(dict, codes);
    if (!ns.empty()) {
      sc.validity.assign(validity::words(rows_per_batch), ~0ull);
      for (auto i : ns) validity::set_bit(sc.validity.data(), i, false);
    }
    src->batches.push_back({sc, make_col(Type::I64, k, nk), make_col(Type::F64, v, nv), make_col(Type::I32, q)});
    std::vector<uint32_t> sel;
    if (b % 2 == 1)
      for (uint32_t i = 0; i < rows_per_batch; ++i)
        if (i % 5 != 2) sel.push_back(i);
    src->sels.push_back(sel);
  }
  return src;
}

// A small dimension table: STR key with a repeated value, an I64 key.
std::unique_ptr<BatchSource> dims_source() {
  auto d = std::make_unique<BatchSource>();
  d->schema.fields = {{"sym", Type::STR}, {"sector", Type::I32}, {"k", Type::I64}};
  d->batches.push_back({str_col({"IBM", "AAPL", "NVDA", "XOM"}, {0, 1, 2, 3, 1}),
                        make_col<int32_t>(Type::I32, {1, 2, 3, 4, 5}),
                        make_col<int64_t>(Type::I64, {-1000, 5, 17, 1999, 5})});
  d->sels.push_back({});
  return d;
}

std::vector<Row> sorted(std::vector<Row> r) {
  std::sort(r.begin(), r.end());
  return r;
}

// Equal row multisets; F64 cells within a relative 1e-12 (summation order).
bool same_rows(std::vector<Row> a, std::vector<Row> b) {
  a = sorted(std::move(a));
  b = sorted(std::move(b));
  if (a.size() != b.size()) return false;
  for (std::size_t i = 0; i < a.size(); ++i) {
    if (a[i].size() != b[i].size()) return false;
    for (std::size_t c = 0; c < a[i].size(); ++c) {
      const Cell &x = a[i][c], &y = b[i][c];
      if (x.null != y.null || x.i != y.i || x.s != y.s) return false;
      if (std::fabs(x.f - y.f) > 1e-12 * std::max(1.0, std::fabs(y.f))) return false;
    }
  }
  return true;
}

void test_device_table_scan() {
  // 90 batches of 2000 rows (odd batches filtered by a selection vector):
  // 162000 logical rows, not a multiple of 64.
  auto up_src = mixed_source(90, 2000);
  auto table = gpu::DeviceTable::upload(*up_src);
  CHECK(table->num_rows() == 162000);
  CHECK(table->schema().fields.size() == 4);
  // Scanned back through host memory: the source's rows in the source's order.
  {
    auto host = mixed_source(90, 2000);
    const auto want = drain(*host);
    for (std::size_t batch : {std::size_t{2048}, std::size_t{192}}) {
      gpu::GpuScan scan(table, batch);
      const auto got = drain(scan);
      CHECK(got.size() == want.size());
      bool eq = got.size() == want.size();
      for (std::size_t i = 0; eq && i < got.size(); ++i)
        for (std::size_t c = 0; eq && c < got[i].size(); ++c)
          eq = !(got[i][c] < want[i][c]) && !(want[i][c] < got[i][c]);
      CHECK(eq);
    }
  }
  bool threw = false;
  try {
    gpu::GpuScan bad(table, 100);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);  // ops/scan.cpp:14-18
  // GROUP BY read in place == GROUP BY through host staging.
  const std::vector<AggSpec> by_sym = {AggSpec::count_star("n"), AggSpec::sum(1, "s"), AggSpec::avg(2, "a"),
                                       AggSpec::min(0, "mn"), AggSpec::max(0, "mx"), AggSpec::count(1, "c")};
  {
    gpu::GpuAggregate dev(std::make_unique<gpu::GpuScan>(table), {0}, by_sym);
    gpu::GpuAggregate host(mixed_source(90, 2000), {0}, by_sym);
    const auto a = drain(dev), b = drain(host);
    CHECK(a.size() == 9);  // 8 symbols and NULL
    CHECK(same_rows(a, b));
  }
  {
    const std::vector<AggSpec> by_k = {AggSpec::count_star("n"), AggSpec::sum(3, "q"), AggSpec::max(2, "m")};
    gpu::GpuAggregate dev(std::make_unique<gpu::GpuScan>(table), {1, 3}, by_k);
    gpu::GpuAggregate host(mixed_source(90, 2000), {1, 3}, by_k);
    CHECK(same_rows(drain(dev), drain(host)));
  }
  // Joins: both sides in place (STR key), in-place probe with a host build
  // (I64 key), and a STR key with only one side in place (staged).
  auto dims = dims_source();
  auto dims_table = gpu::DeviceTable::upload(*dims);
  auto host_dims = [] { return dims_source(); };
  for (JoinType jt : {JoinType::Inner, JoinType::Left}) {
    gpu::GpuHashJoin dev(std::make_unique<gpu::GpuScan>(table), std::make_unique<gpu::GpuScan>(dims_table), {0}, {0},
                         jt);
    gpu::GpuHashJoin host(mixed_source(90, 2000), host_dims(), {0}, {0}, jt);
    const auto a = drain(dev), b = drain(host);
    CHECK(!a.empty());
    CHECK(same_rows(a, b));
    gpu::GpuHashJoin dev_k(std::make_unique<gpu::GpuScan>(table), host_dims(), {1}, {2}, jt);
    gpu::GpuHashJoin host_k(mixed_source(90, 2000), host_dims(), {1}, {2}, jt);
    CHECK(same_rows(drain(dev_k), drain(host_k)));
    gpu::GpuHashJoin mixed(std::make_unique<gpu::GpuScan>(table), host_dims(), {0}, {0}, jt);
    CHECK(same_rows(drain(mixed), b));
  }
  // An empty table: no batches, and a global aggregate of zero rows.
  auto none = mixed_source(0, 0);
  auto empty = gpu::DeviceTable::upload(*none);
  CHECK(empty->num_rows() == 0);
  gpu::GpuScan es(empty);
  CHECK(drain(es).empty());
  gpu::GpuAggregate g(std::make_unique<gpu::GpuScan>(empty), {}, {AggSpec::count_star("n"), AggSpec::sum(1, "s")});
  const auto rows = drain(g);
  CHECK(rows.size() == 1 && rows[0][0].i == 0 && rows[0][1].null);
}

void test_concurrent_instances() {
  // Several operator instances in one process, one per thread, as the
  // reference's morsel workers run them (exec/parallel.h:15-19): each owns its
  // context, stream and buffers; two of them read one DeviceTable at a time.
  auto up = mixed_source(90, 2000);
  auto table = gpu::DeviceTable::upload(*up);
  const std::vector<AggSpec> by_sym = {AggSpec::count_star("n"), AggSpec::sum(1, "s"), AggSpec::avg(2, "a"),
                                       AggSpec::min(0, "mn"), AggSpec::max(0, "mx")};
  const std::vector<AggSpec> by_k = {AggSpec::count_star("n"), AggSpec::sum(3, "q"), AggSpec::max(2, "m")};
  auto run = [&](int kind) {
    switch (kind) {
      case 0: {
        gpu::GpuAggregate a(std::make_unique<gpu::GpuScan>(table), {0}, by_sym);
        return drain(a);
      }
      case 1: {
        gpu::GpuAggregate a(mixed_source(90, 2000), {1, 3}, by_k);
        return drain(a);
      }
      case 2: {
        gpu::GpuHashJoin j(std::make_unique<gpu::GpuScan>(table), std::make_unique<gpu::GpuScan>(
                               gpu::DeviceTable::upload(*dims_source())), {0}, {0}, JoinType::Left);
        return drain(j);
      }
      default: {
        gpu::GpuHashJoin j(mixed_source(90, 2000), dims_source(), {1}, {2}, JoinType::Inner);
        return drain(j);
      }
    }
  };
  std::vector<std::vector<Row>> want;
  for (int k = 0; k < 4; ++k) want.push_back(run(k));
  std::atomic<int> mismatches{0}, errors{0};
  std::vector<std::thread> workers;
  for (int w = 0; w < 4; ++w)
    workers.emplace_back([&, w] {
      try {
        for (int it = 0; it < 4; ++it) {
          const int k = (w + it) % 4;
          if (!same_rows(run(k), want[k])) ++mismatches;
        }
      } catch (const std::exception& e) {
        std::fprintf(stderr, "worker %d: %s\n", w, e.what());
        ++errors;
      }
    });
  for (auto& t : workers) t.join();
  CHECK(errors.load() == 0);
  CHECK(mismatches.load() == 0);
}

int main() {
  try {
    test_aggregate_edge_table();
    test_aggregate_random_vs_cpu();
    test_aggregate_str_by_value_and_selection();
    test_aggregate_errors_and_global_empty();
    test_join_edge_cases();
    test_join_str_keys();
    test_window_tumbling();
    test_asof_join();
    test_device_table_scan();
    test_concurrent_instances();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "exception: %s\n", e.what());
    return 2;
  }
  if (g_fail) {
    std::fprintf(stderr, "%d check(s) failed\n", g_fail.load());
    return 1;
  }
  std::printf("all operator checks passed\n");
  return 0;
}
