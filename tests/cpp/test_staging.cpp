// Host-side staging of the GPU operators, checked without a GPU: Staging
// (rows pulled from a child into contiguous values and packed validity words,
// selection vectors applied, STR codes made canonical ids by value) and
// OutColumns views. Page-locked allocation falls back to ordinary heap memory
// where no device is present, so this runs on any host.
// Exit code 0 = all checks passed.
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../query-engine_gb300/host/gpu_operators.h"

using namespace qe;

static int g_fail = 0;
#define CHECK(c)                                                        \
  do {                                                                  \
    if (!(c)) {                                                         \
      std::fprintf(stderr, "CHECK failed at line %d: %s\n", __LINE__, #c); \
      ++g_fail;                                                         \
    }                                                                   \
  } while (0)

namespace {

template <class T>
gpu::HostColumn col(Type t, const std::vector<T>& v, const std::vector<bool>& valid = {}) {
  gpu::HostColumn c;
  c.type = t;
  c.len = v.size();
  c.data.resize(std::max<std::size_t>(1, v.size() * sizeof(T)));
  if (!v.empty()) std::memcpy(c.data.data(), v.data(), v.size() * sizeof(T));
  if (!valid.empty()) {
    c.validity.assign(validity::words(v.size()), ~0ull);
    for (std::size_t i = 0; i < valid.size(); ++i)
      if (!valid[i]) validity::set_bit(c.validity.data(), i, false);
  }
  return c;
}

gpu::HostColumn strs(const std::vector<std::string>& dict, const std::vector<int32_t>& codes,
                     const std::vector<bool>& valid = {}) {
  gpu::HostColumn c = col(Type::STR, codes, valid);
  auto d = std::make_shared<StringDict>();
  for (const auto& s : dict) d->intern(s);
  c.dict = d;
  return c;
}

Batch batch(const std::vector<gpu::HostColumn>& cols, const SelectionVector* sel) {
  Batch b;
  for (const auto& c : cols) b.cols.push_back(c.view());
  b.sel = sel;
  b.row_count = sel ? sel->len : cols[0].len;
  return b;
}

// Random batches of random lengths (some with selection vectors) against a
// row-by-row model of what staging must produce.
void test_values_and_validity_across_batches() {
  std::mt19937_64 rng(11);
  gpu::Staging st;
  st.reset({Type::I64, Type::F64, Type::BOOL});
  std::vector<int64_t> want_k;
  std::vector<double> want_v;
  std::vector<uint8_t> want_b;
  std::vector<bool> want_kv, want_vv;
  const std::vector<StringDict*> ids(3, nullptr);
  for (int b = 0; b < 60; ++b) {
    const std::size_t n = 1 + rng() % 300;
    std::vector<int64_t> k(n);
    std::vector<double> v(n);
    std::vector<uint8_t> bo(n);
    std::vector<bool> kv(n), vv(n);
    const bool k_nulls = rng() % 2, v_nulls = rng() % 3 == 0;
    for (std::size_t i = 0; i < n; ++i) {
      k[i] = static_cast<int64_t>(rng());
      v[i] = static_cast<double>(rng() % 1000) / 3.0;
      bo[i] = rng() % 2;
      kv[i] = !k_nulls || rng() % 5 != 0;
      vv[i] = !v_nulls || rng() % 7 != 0;
    }
    std::vector<gpu::HostColumn> cols = {col(Type::I64, k, k_nulls ? kv : std::vector<bool>{}),
                                         col(Type::F64, v, v_nulls ? vv : std::vector<bool>{}),
                                         col(Type::BOOL, bo)};
    std::vector<uint32_t> idx;
    const bool use_sel = rng() % 3 == 0;
    if (use_sel)
      for (uint32_t i = 0; i < n; ++i)
        if (rng() % 3) idx.push_back(i);
    SelectionVector sv{idx.data(), idx.size()};
    if (use_sel && idx.empty()) continue;
    st.append(batch(cols, use_sel ? &sv : nullptr), ids);
    const std::size_t m = use_sel ? idx.size() : n;
    for (std::size_t j = 0; j < m; ++j) {
      const std::size_t r = use_sel ? idx[j] : j;
      want_k.push_back(k[r]);
      want_v.push_back(v[r]);
      want_b.push_back(bo[r]);
      want_kv.push_back(kv[r]);
      want_vv.push_back(vv[r]);
    }
  }
  CHECK(st.rows == want_k.size());
  const auto* gk = reinterpret_cast<const int64_t*>(st.vals[0].data());
  const auto* gv = reinterpret_cast<const double*>(st.vals[1].data());
  const auto* gb = st.vals[2].data();
  bool vals_ok = true, bits_ok = true;
  bool any_k = false, any_v = false;
  for (std::size_t r = 0; r < st.rows; ++r) {
    vals_ok = vals_ok && gk[r] == want_k[r] && gv[r] == want_v[r] && gb[r] == want_b[r];
    bits_ok = bits_ok && validity::get_bit(st.words(0), r) == want_kv[r] &&
              validity::get_bit(st.words(1), r) == want_vv[r] && validity::get_bit(st.words(2), r);
    any_k = any_k || !want_kv[r];
    any_v = any_v || !want_vv[r];
  }
  CHECK(vals_ok);
  CHECK(bits_ok);
  CHECK(st.any_null[0] == any_k && st.any_null[1] == any_v && !st.any_null[2]);
  const auto qc = st.columns();
  CHECK(qc.size() == 3);
  CHECK(qc[0].type == QEG_I64 && qc[1].type == QEG_F64 && qc[2].type == QEG_BOOL);
  CHECK(qc[0].len == st.rows && qc[2].all_valid == 1 && qc[2].validity == nullptr);
  CHECK(qc[0].all_valid == (any_k ? 0 : 1));
  // reset: no rows, the same columns, no NULL flags.
  st.reset(st.types);
  CHECK(st.rows == 0 && st.columns()[0].len == 0 && !st.any_null[0]);
}

// STR codes of several dictionaries become one id per distinct string, with
// the code -> id table of each dictionary kept across resets.
void test_str_canonical_ids() {
  gpu::Staging st;
  st.reset({Type::STR});
  StringDict ids;
  const std::vector<StringDict*> idp = {&ids};
  auto a = strs({"AAPL", "MSFT", "GOOG"}, {0, 1, 2, 0, 1}, {true, true, false, true, true});
  auto b = strs({"GOOG", "IBM", "AAPL"}, {0, 1, 2, 2});
  st.append(batch({a}, nullptr), idp);
  uint32_t pick[] = {3, 1};
  SelectionVector sv{pick, 2};
  st.append(batch({b}, &sv), idp);
  CHECK(st.rows == 7);
  const int32_t* v = st.str_ids(0);
  auto name = [&](std::size_t r) { return std::string(ids.at(v[r])); };
  CHECK(name(0) == "AAPL" && name(1) == "MSFT" && name(3) == "AAPL" && name(4) == "MSFT");
  CHECK(!validity::get_bit(st.words(0), 2) && v[2] == 0);  // a NULL row carries id 0
  CHECK(name(5) == "AAPL" && name(6) == "IBM");
  CHECK(v[0] == v[3] && v[3] == v[5]);                     // equal strings, equal ids
  CHECK(ids.size() == 4);                                  // AAPL MSFT GOOG IBM
  CHECK(st.columns()[0].type == QEG_I32 && st.any_null[0]);
  CHECK(st.code_ids[0].size() == 2);
  st.reset(st.types);
  CHECK(st.code_ids[0].size() == 2);  // the per-dictionary tables survive a reset
  // A code outside its dictionary is the reference's invalid input.
  auto bad = strs({"X"}, {0, 5});
  bool threw = false;
  try {
    st.append(batch({bad}, nullptr), idp);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  CHECK(threw);
}

// OutColumns: views of 2048-row slices at multiples of 64 re-base the
// validity words, carry the column's dictionary and its all-valid flag.
void test_out_column_views() {
  gpu::OutColumns o;
  o.reserve({Type::I32, Type::STR}, 5000);
  auto* x = reinterpret_cast<int32_t*>(o.vals[0].data());
  auto* w = reinterpret_cast<uint64_t*>(o.valid[0].data());
  for (int i = 0; i < 5000; ++i) x[i] = i * 3;
  for (std::size_t k = 0; k < validity::words(5000); ++k) w[k] = 0x5555555555555555ull;
  o.all_valid[0] = 0;
  auto d = std::make_shared<StringDict>();
  d->intern("s");
  o.dicts[1] = d;
  const Column c = o.view(0, 2048, 2048);
  CHECK(c.type == Type::I32 && c.len == 2048 && !c.all_valid);
  CHECK(reinterpret_cast<const int32_t*>(c.data)[0] == 2048 * 3);
  CHECK(c.validity == w + 32);
  CHECK(validity::get_bit(c.validity, 0) && !validity::get_bit(c.validity, 1));
  const Column s = o.view(1, 4096, 904);
  CHECK(s.all_valid && s.validity == nullptr && s.dict == d.get() && s.len == 904);
  // A reserve with the same types keeps the buffers and resets the flags.
  o.reserve({Type::I32, Type::STR}, 100);
  CHECK(o.all_valid[0] == 1 && o.dicts[1] == d);
}

}  // namespace

int main() {
  try {
    test_values_and_validity_across_batches();
    test_str_canonical_ids();
    test_out_column_views();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "exception: %s\n", e.what());
    return 2;
  }
  if (g_fail) {
    std::fprintf(stderr, "%d check(s) failed\n", g_fail);
    return 1;
  }
  std::printf("all staging checks passed\n");
  return 0;
}
