// bench_operators.cpp -- end-to-end throughput of the GPU operators through the
// reference's pull interface: host tables, a Scan of 2048-row Batch views
// (ops/scan.cpp:27-64), the GPU operator, and a drain of its <= 2048-row output
// batches on the host, exactly as a plan tree runs them.
//
//   bench_operators agg  <rows> <steps>   GROUP BY of the 1M-row plain aggregate
//                                         workload: I64 key uniform over 1024
//                                         values, F64 value U[0,1000) with 5%
//                                         NULLs; COUNT(*), SUM, AVG, MIN, MAX.
//   bench_operators agg_resident <rows> <steps>
//                                         the same GROUP BY over a DeviceTable
//                                         uploaded once: GpuAggregate over a
//                                         GpuScan reads the columns in place.
//   bench_operators join <build> <probe> <steps>
//                                         inner join of the 16M x 256M workload:
//                                         build keys a permutation of
//                                         0..build-1, probe keys half from the
//                                         build range and half from [build,
//                                         2*build), 2% NULL keys on both sides,
//                                         probe payload U[0,2^20); the drain
//                                         counts the output rows and sums the
//                                         probe payload.
//   bench_operators join_resident <build> <probe> <steps>
//                                         the same join with both sides in
//                                         DeviceTables uploaded once.
//
// Prints one JSON object: rows/s over the input rows (build + probe for the
// join) of the median step, each step's seconds, and a check of the drained
// result against the same result computed here on the host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "gpu_operators.h"

using namespace qe;

namespace {

// splitmix64: the seeded generator of the synthetic columns.
struct Rng {
  std::uint64_t s;
  std::uint64_t next() {
    std::uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Table {
  Schema schema;
  std::vector<gpu::HostColumn> cols;
  std::size_t rows = 0;
};

gpu::HostColumn column(Type t, std::size_t n) {
  gpu::HostColumn c;
  c.type = t;
  c.len = n;
  c.data.resize(n * byte_width(t));
  return c;
}

void set_nulls(gpu::HostColumn& c, Rng& r, double p) {
  c.validity.assign(validity::words(c.len), ~0ull);
  for (std::size_t i = 0; i < c.len; ++i)
    if (r.uniform() < p) validity::set_bit(c.validity.data(), i, false);
}

// Zero-copy 2048-row windows of a table (validity re-based by whole words).
class Scan : public Operator {
 public:
  explicit Scan(const Table& t) : t_(t) {}
  void open() override { cur_ = 0; }
  std::optional<Batch> next() override {
    if (cur_ >= t_.rows) return std::nullopt;
    const std::size_t m = std::min<std::size_t>(2048, t_.rows - cur_);
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
  const Table& t_;
  std::size_t cur_ = 0;
};

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool valid_at(const Column& c, std::size_t i) { return c.all_valid || validity::get_bit(c.validity, i); }

void print_steps(const std::vector<double>& t) {
  std::printf("\"step_s\": [");
  for (std::size_t i = 0; i < t.size(); ++i) std::printf("%s%.4f", i ? ", " : "", t[i]);
  std::printf("]");
}

double median(std::vector<double> t) {
  std::sort(t.begin(), t.end());
  return t[t.size() / 2];
}

// Uploads a table once (the upload is not part of a step).
std::shared_ptr<const gpu::DeviceTable> resident(const Table& t, double* seconds) {
  const double t0 = now();
  Scan s(t);
  auto dt = gpu::DeviceTable::upload(s);
  *seconds = now() - t0;
  return dt;
}

std::unique_ptr<Operator> source(const Table& t, const std::shared_ptr<const gpu::DeviceTable>& dt) {
  if (dt) return std::make_unique<gpu::GpuScan>(dt);
  return std::make_unique<Scan>(t);
}

int run_agg(std::size_t n, int steps, bool in_place) {
  Rng r{20260616};
  Table t;
  t.schema.fields = {{"k", Type::I64}, {"v", Type::F64}};
  t.rows = n;
  t.cols.push_back(column(Type::I64, n));
  t.cols.push_back(column(Type::F64, n));
  auto* k = reinterpret_cast<std::int64_t*>(t.cols[0].data.data());
  auto* v = reinterpret_cast<double*>(t.cols[1].data.data());
  for (std::size_t i = 0; i < n; ++i) {
    k[i] = static_cast<std::int64_t>(r.next() % 1024);
    v[i] = r.uniform() * 1000.0;
  }
  set_nulls(t.cols[1], r, 0.05);
  // Host check: per key COUNT(*) and COUNT(v).
  std::vector<std::int64_t> cnt(1024, 0), cntv(1024, 0);
  for (std::size_t i = 0; i < n; ++i) {
    ++cnt[k[i]];
    if (validity::get_bit(t.cols[1].validity.data(), i)) ++cntv[k[i]];
  }
  double upload_s = 0;
  const auto dt = in_place ? resident(t, &upload_s) : nullptr;
  std::vector<double> times;
  bool ok = true;
  std::size_t groups = 0, batches = 0;
  for (int s = 0; s < steps + 1; ++s) {
    const double t0 = now();
    gpu::GpuAggregate agg(source(t, dt), {0},
                          {AggSpec::count_star("n"), AggSpec::sum(1, "s"), AggSpec::avg(1, "a"),
                           AggSpec::min(1, "lo"), AggSpec::max(1, "hi")});
    agg.open();
    std::vector<std::int64_t> seen(1024, -1);
    groups = batches = 0;
    while (std::optional<Batch> b = agg.next()) {
      ++batches;
      const auto* kk = reinterpret_cast<const std::int64_t*>(b->cols[0].data);
      const auto* nn = reinterpret_cast<const std::int64_t*>(b->cols[1].data);
      for (std::size_t i = 0; i < b->row_count; ++i, ++groups)
        if (kk[i] >= 0 && kk[i] < 1024) seen[kk[i]] = nn[i];
    }
    agg.close();
    const double dt = now() - t0;
    if (s > 0) times.push_back(dt);  // the first step is the warm-up
    for (int g = 0; g < 1024; ++g) ok = ok && seen[g] == cnt[g];
    ok = ok && groups == 1024;
  }
  const double med = median(times);
  std::printf("{\"workload\": \"plain_agg_1M_1024keys through GpuAggregate::open/next/close%s\", \"rows\": %zu, "
              "\"value\": %.6g, \"unit\": \"rows/s\", \"groups\": %zu, \"output_batches\": %zu, "
              "\"check_counts_vs_host\": %s, \"upload_s\": %.4f, ",
              in_place ? " over a GpuScan of a DeviceTable" : "", n, n / med, groups, batches, ok ? "true" : "false",
              upload_s);
  print_steps(times);
  std::printf("}\n");
  return ok ? 0 : 1;
}

int run_join(std::size_t nb, std::size_t np, int steps, bool in_place) {
  Rng r{20260617};
  Table b, p;
  b.schema.fields = {{"bk", Type::I64}, {"bv", Type::I64}};
  p.schema.fields = {{"pk", Type::I64}, {"pv", Type::I64}};
  b.rows = nb;
  p.rows = np;
  b.cols.push_back(column(Type::I64, nb));
  b.cols.push_back(column(Type::I64, nb));
  p.cols.push_back(column(Type::I64, np));
  p.cols.push_back(column(Type::I64, np));
  auto* bk = reinterpret_cast<std::int64_t*>(b.cols[0].data.data());
  auto* bv = reinterpret_cast<std::int64_t*>(b.cols[1].data.data());
  for (std::size_t i = 0; i < nb; ++i) {
    bk[i] = static_cast<std::int64_t>(i);
    bv[i] = static_cast<std::int64_t>(i);
  }
  for (std::size_t i = nb; i > 1; --i) std::swap(bk[i - 1], bk[r.next() % i]);  // Fisher-Yates
  set_nulls(b.cols[0], r, 0.02);
  auto* pk = reinterpret_cast<std::int64_t*>(p.cols[0].data.data());
  auto* pv = reinterpret_cast<std::int64_t*>(p.cols[1].data.data());
  for (std::size_t i = 0; i < np; ++i) {
    const bool hit = r.uniform() < 0.5;
    pk[i] = static_cast<std::int64_t>(hit ? r.next() % nb : nb + r.next() % nb);
    pv[i] = static_cast<std::int64_t>(r.next() & ((1u << 20) - 1));
  }
  set_nulls(p.cols[0], r, 0.02);
  // Host check: the matched count and payload sum.
  std::vector<std::uint8_t> present(nb, 0);
  for (std::size_t i = 0; i < nb; ++i)
    if (validity::get_bit(b.cols[0].validity.data(), i)) present[bk[i]] = 1;
  std::int64_t want_n = 0, want_s = 0;
  for (std::size_t i = 0; i < np; ++i)
    if (validity::get_bit(p.cols[0].validity.data(), i) && pk[i] < static_cast<std::int64_t>(nb) && present[pk[i]]) {
      ++want_n;
      want_s += pv[i];
    }
  double up_b = 0, up_p = 0;
  const auto dtb = in_place ? resident(b, &up_b) : nullptr;
  const auto dtp = in_place ? resident(p, &up_p) : nullptr;
  std::vector<double> times;
  bool ok = true;
  std::int64_t got_n = 0, got_s = 0;
  std::size_t batches = 0;
  for (int s = 0; s < steps + 1; ++s) {
    const double t0 = now();
    gpu::GpuHashJoin j(source(p, dtp), source(b, dtb), {0}, {0}, JoinType::Inner);
    j.open();
    got_n = got_s = 0;
    batches = 0;
    while (std::optional<Batch> o = j.next()) {
      ++batches;
      const Column& c = o->cols[1];
      const auto* x = reinterpret_cast<const std::int64_t*>(c.data);
      std::int64_t acc = 0;
      for (std::size_t i = 0; i < o->row_count; ++i) acc += valid_at(c, i) ? x[i] : 0;
      got_s += acc;
      got_n += static_cast<std::int64_t>(o->row_count);
    }
    j.close();
    const double dt = now() - t0;
    if (s > 0) times.push_back(dt);
    ok = ok && got_n == want_n && got_s == want_s;
  }
  const double med = median(times);
  std::printf("{\"workload\": \"join_%zuMx%zuM through GpuHashJoin::open/next/close%s, output drained on the "
              "host\", \"build_rows\": %zu, \"probe_rows\": %zu, \"value\": %.6g, \"unit\": \"rows/s\", "
              "\"output_rows\": %lld, \"output_batches\": %zu, \"check_count_sum_vs_host\": %s, "
              "\"upload_s\": %.4f, ",
              nb >> 20, np >> 20, in_place ? " over GpuScans of DeviceTables" : "", nb, np, (nb + np) / med,
              static_cast<long long>(got_n), batches, ok ? "true" : "false", up_b + up_p);
  print_steps(times);
  std::printf("}\n");
  return ok ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string w = argc > 1 ? argv[1] : "agg";
  try {
    if (w == "agg" || w == "agg_resident")
      return run_agg(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : (1u << 20), argc > 3 ? std::atoi(argv[3]) : 5,
                     w == "agg_resident");
    if (w == "join" || w == "join_resident")
      return run_join(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : (1u << 24),
                      argc > 3 ? std::strtoull(argv[3], nullptr, 10) : (1ull << 28), argc > 4 ? std::atoi(argv[4]) : 3,
                      w == "join_resident");
  } catch (const std::exception& e) {
    std::printf("{\"error\": \"%s\"}\n", e.what());
    return 2;
  }
  std::fprintf(stderr,
               "usage: bench_operators agg|agg_resident <rows> <steps> | join|join_resident <build> <probe> <steps>\n");
  return 2;
}
