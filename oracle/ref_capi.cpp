// ref_capi.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// A thin C API over the REFERENCE engine itself (explorer-skp/query-engine),
// compiled from the reference's own sources by `make -C oracle ref` into
// oracle/_ref/libqe_ref.so. It exists only in a checkout that has the reference
// tree; it is used to pin the restatement in qe_oracle.cpp and to generate the
// golden vectors under tests/golden/. It calls the reference's public API:
//   plan::scan(t).aggregate(...) / .join(...)      plan/plan.h:218-262
//   oracle::drain_operator                          oracle/result_set.h:64
//   oracle::run_reference / run_join_reference      oracle/reference_oracle.h:30-56
//   exec::ParallelEngine::run                       exec/parallel.h:72-111
//   plan window_tumbling / asof_join                plan/plan.h:215-243
//   oracle::run_window_reference / run_asof_reference oracle/reference_oracle.h:65-87
//   ops::hash_combine_scalar                        ops/hash_kernels.h:56-58
// The result accessor functions mirror the orc_result_* ones.

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "core/owned_batch.h"
#include "core/string_dict.h"
#include "exec/parallel.h"
#include "ops/hash_kernels.h"
#include "ops/table.h"
#include "oracle/logical_query.h"
#include "oracle/reference_oracle.h"
#include "oracle/result_set.h"
#include "plan/plan.h"
#include "qe_oracle.h"

namespace {
thread_local std::string g_err;

qe::Table make_table(const orc_column* cols, int n) {
    qe::Schema s;
    std::vector<qe::OwnedColumn> oc;
    for (int c = 0; c < n; ++c) {
        const orc_column& x = cols[c];
        const qe::Type t = static_cast<qe::Type>(x.type);
        s.fields.emplace_back("c" + std::to_string(c), t);
        qe::OwnedColumn col;
        if (t == qe::Type::STR) {
            auto d = std::make_shared<qe::StringDict>();
            for (uint32_t k = 0; k < x.dict_size; ++k)
                d->intern(std::string_view(x.dict_bytes + x.dict_offsets[k],
                                           x.dict_offsets[k + 1] - x.dict_offsets[k]));
            col = qe::OwnedColumn::make_str(x.len, d);
        } else {
            col = qe::OwnedColumn::make(t, x.len);
        }
        if (x.len) std::memcpy(col.mutable_data(), x.data, x.len * qe::byte_width(t));
        if (!x.all_valid && x.validity) {
            for (uint64_t i = 0; i < x.len; ++i)
                if (!((x.validity[i >> 6] >> (i & 63)) & 1ull)) col.set_null(i);
        }
        oc.push_back(std::move(col));
    }
    return qe::Table(std::move(s), std::move(oc));
}

std::vector<qe::AggSpec> make_aggs(const int32_t* f, const uint32_t* c, int n) {
    std::vector<qe::AggSpec> v;
    for (int i = 0; i < n; ++i) {
        const std::string nm = "a" + std::to_string(i);
        switch (f[i]) {
            case ORC_COUNT_STAR: v.push_back(qe::AggSpec::count_star(nm)); break;
            case ORC_COUNT: v.push_back(qe::AggSpec::count(c[i], nm)); break;
            case ORC_SUM: v.push_back(qe::AggSpec::sum(c[i], nm)); break;
            case ORC_MIN: v.push_back(qe::AggSpec::min(c[i], nm)); break;
            case ORC_MAX: v.push_back(qe::AggSpec::max(c[i], nm)); break;
            case ORC_AVG: v.push_back(qe::AggSpec::avg(c[i], nm)); break;
            default: throw std::invalid_argument("unknown aggregate");
        }
    }
    return v;
}

template <class F>
int guarded(F&& fn) {
    try {
        fn();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}
}  // namespace

struct ref_result {
    qe::oracle::ResultSet rs;
};

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

uint64_t ref_hash_combine(uint64_t acc, uint64_t word) {
    qe::ops::hash_combine_scalar(&acc, &word, 1);
    return acc;
}

// mode 0: the engine operator tree (Plan::lower + drain); 1: the independent
// reference oracle; 2: the morsel-parallel engine with `threads` workers.
int ref_groupby(const orc_column* cols, int ncols, const uint32_t* key_cols, int nkeys,
                const int32_t* agg_funcs, const uint32_t* agg_cols, int naggs,
                uint64_t batch_rows, int mode, unsigned threads, ref_result** out) {
    return guarded([&] {
        auto t = std::make_unique<qe::Table>(make_table(cols, ncols));
        std::vector<qe::plan::ColRef> keys;
        for (int k = 0; k < nkeys; ++k) keys.emplace_back(key_cols[k]);
        auto aggs = make_aggs(agg_funcs, agg_cols, naggs);
        auto r = std::make_unique<ref_result>();
        if (mode == 1) {
            qe::oracle::LogicalQuery q;
            q.group_by = qe::oracle::GroupBy{
                std::vector<uint32_t>(key_cols, key_cols + nkeys), aggs};
            r->rs = qe::oracle::run_reference(*t, q);
        } else {
            auto pb = qe::plan::scan(*t).aggregate(keys, aggs);
            if (mode == 2) {
                qe::exec::ParallelConfig cfg;
                cfg.threads = threads;
                cfg.morsel_rows = batch_rows;
                r->rs = qe::exec::run_plan_parallel(pb.plan(), cfg);
            } else {
                auto op = pb.build(batch_rows);
                r->rs = qe::oracle::drain_operator(*op);
            }
        }
        *out = r.release();
    });
}

int ref_join(const orc_column* probe, int nprobe, const orc_column* build, int nbuild,
             const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
             int32_t join_type, uint64_t batch_rows, int mode, ref_result** out) {
    return guarded([&] {
        auto pt = std::make_unique<qe::Table>(make_table(probe, nprobe));
        auto bt = std::make_unique<qe::Table>(make_table(build, nbuild));
        const qe::JoinType jt = join_type == ORC_LEFT ? qe::JoinType::Left : qe::JoinType::Inner;
        auto r = std::make_unique<ref_result>();
        if (mode == 1) {
            qe::oracle::JoinQuery q{std::vector<uint32_t>(probe_keys, probe_keys + nkeys),
                                    std::vector<uint32_t>(build_keys, build_keys + nkeys), jt};
            r->rs = qe::oracle::run_join_reference(*pt, *bt, q);
        } else {
            std::vector<qe::plan::ColRef> lk, rk;
            for (int k = 0; k < nkeys; ++k) {
                lk.emplace_back(probe_keys[k]);
                rk.emplace_back(build_keys[k]);
            }
            auto op = qe::plan::scan(*pt).join(qe::plan::scan(*bt), lk, rk, jt).build(batch_rows);
            r->rs = qe::oracle::drain_operator(*op);
        }
        *out = r.release();
    });
}

// Tumbling window: mode 0 the engine operator (plan window_tumbling + drain),
// 1 the independent reference oracle (run_window_reference).
int ref_window_tumbling(const orc_column* cols, int ncols, const uint32_t* key_cols, int nkeys,
                        uint32_t time_col, int64_t width, const int32_t* agg_funcs,
                        const uint32_t* agg_cols, int naggs, uint64_t batch_rows, int mode,
                        ref_result** out) {
    return guarded([&] {
        auto t = std::make_unique<qe::Table>(make_table(cols, ncols));
        auto aggs = make_aggs(agg_funcs, agg_cols, naggs);
        auto r = std::make_unique<ref_result>();
        if (mode == 1) {
            r->rs = qe::oracle::run_window_reference(
                *t, qe::tsx::WindowMode::Tumbling,
                std::vector<uint32_t>(key_cols, key_cols + nkeys), time_col, width, aggs);
        } else {
            std::vector<qe::plan::ColRef> keys;
            for (int k = 0; k < nkeys; ++k) keys.emplace_back(key_cols[k]);
            auto op = qe::plan::scan(*t)
                          .window_tumbling(keys, qe::plan::ColRef(time_col), width, aggs)
                          .build(batch_rows);
            r->rs = qe::oracle::drain_operator(*op);
        }
        *out = r.release();
    });
}

// Backward as-of join: mode 0 the engine operator (plan asof_join + drain), 1
// the independent reference oracle (run_asof_reference).
int ref_asof_join(const orc_column* probe, int nprobe, const orc_column* build, int nbuild,
                  const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
                  uint32_t probe_time, uint32_t build_time, int32_t asof_type, int32_t has_tol,
                  int64_t tol, uint64_t batch_rows, int mode, ref_result** out) {
    return guarded([&] {
        auto pt = std::make_unique<qe::Table>(make_table(probe, nprobe));
        auto bt = std::make_unique<qe::Table>(make_table(build, nbuild));
        const qe::tsx::AsofType at =
            asof_type == ORC_LEFT ? qe::tsx::AsofType::Left : qe::tsx::AsofType::Inner;
        std::optional<std::int64_t> tolerance;
        if (has_tol) tolerance = tol;
        auto r = std::make_unique<ref_result>();
        if (mode == 1) {
            r->rs = qe::oracle::run_asof_reference(
                *pt, *bt, std::vector<uint32_t>(probe_keys, probe_keys + nkeys),
                std::vector<uint32_t>(build_keys, build_keys + nkeys), probe_time, build_time, at,
                tolerance);
        } else {
            std::vector<qe::plan::ColRef> lk, rk;
            for (int k = 0; k < nkeys; ++k) {
                lk.emplace_back(probe_keys[k]);
                rk.emplace_back(build_keys[k]);
            }
            auto op = qe::plan::scan(*pt)
                          .asof_join(qe::plan::scan(*bt), lk, rk, qe::plan::ColRef(probe_time),
                                     qe::plan::ColRef(build_time), at, tolerance)
                          .build(batch_rows);
            r->rs = qe::oracle::drain_operator(*op);
        }
        *out = r.release();
    });
}

// scan(probe).join(scan(build)).aggregate({}, {COUNT(*), SUM(probe col 1)}) on the
// morsel-parallel engine (threads == 0 -> hardware concurrency).
int ref_parallel_join_count_sum(const orc_column* probe, const orc_column* build,
                                unsigned threads, uint64_t morsel_rows, int64_t* cnt,
                                int64_t* sum, int32_t* sum_valid) {
    return guarded([&] {
        auto pt = std::make_unique<qe::Table>(make_table(probe, 2));
        auto bt = std::make_unique<qe::Table>(make_table(build, 2));
        auto pb = qe::plan::scan(*pt)
                      .join(qe::plan::scan(*bt), {0}, {0}, qe::JoinType::Inner)
                      .aggregate({}, {qe::AggSpec::count_star("n"), qe::AggSpec::sum(1, "s")});
        qe::exec::ParallelConfig cfg;
        cfg.threads = threads;
        cfg.morsel_rows = morsel_rows;
        const qe::oracle::ResultSet rs = qe::exec::run_plan_parallel(pb.plan(), cfg);
        *cnt = rs.rows.at(0).at(0).i;
        *sum = rs.rows.at(0).at(1).i;
        *sum_valid = rs.rows.at(0).at(1).is_null ? 0 : 1;
    });
}

uint64_t ref_result_rows(const ref_result* r) { return r ? r->rs.num_rows() : 0; }
int ref_result_cols(const ref_result* r) { return r ? static_cast<int>(r->rs.num_cols()) : 0; }
int32_t ref_result_type(const ref_result* r, int col) {
    return static_cast<int32_t>(r->rs.types.at(static_cast<size_t>(col)));
}
// STR cells come back as their string value through ref_result_str.
int ref_result_fetch(const ref_result* r, int col, int64_t* iv, double* fv, uint8_t* valid) {
    const size_t c = static_cast<size_t>(col);
    for (size_t row = 0; row < r->rs.rows.size(); ++row) {
        const auto& cell = r->rs.rows[row].at(c);
        if (iv) iv[row] = cell.i;
        if (fv) fv[row] = cell.f;
        if (valid) valid[row] = cell.is_null ? 0 : 1;
    }
    return 0;
}
int ref_result_str(const ref_result* r, int col, uint64_t row, const char** s, uint64_t* len) {
    const auto& cell = r->rs.rows.at(row).at(static_cast<size_t>(col));
    *s = cell.s.data();
    *len = cell.s.size();
    return 0;
}
void ref_result_free(ref_result* r) { delete r; }

}  // extern "C"
