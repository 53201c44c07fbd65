/*
 * qe_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A CPU restatement of the reference engine's hash GROUP BY and hash equi-join
 * (explorer-skp/query-engine), used ONLY as the parity checker by tests/, by
 * __graft_entry__.smoke(), and as the timed CPU baseline in bench.py. Nothing in
 * the GPU product path links, loads or calls this library.
 *
 * Parity status: pinned. tests/test_oracle_golden.py checks this restatement
 * against golden vectors produced by the reference itself (compiled from its own
 * sources by oracle/Makefile into oracle/_ref/, outputs committed under
 * tests/golden/), and against the hand-written expected values in the reference's
 * own differential tests.
 *
 * Semantics followed (reference file:line):
 *   - key normalisation + seeded splitmix64 fold   ops/hash_internal.cpp:29-97,
 *                                                  ops/hash_scalar.cpp:14-29
 *   - open addressing, linear probe, pow2 capacity, dense first-seen ids,
 *     grow x2 at load 0.7, kEqual / kNeverMatch     ops/hashtable.cpp:60-163
 *   - AggCell scatter, NaN-greatest F64 order       ops/aggregate.cpp:118-155,
 *                                                  ops/agg_internal.h:34-81
 *   - result types / finalisation / NULL rules      ops/aggregate.cpp:78-97,
 *                                                  ops/agg_internal.h:169-229
 *   - global (zero-key) path: one row, even empty   ops/aggregate.cpp:258-373,
 *                                                  ops/aggregate.cpp:439-458
 *   - join build store + multiplicity lists,
 *     probe find, LEFT null-fill, output order      ops/join.cpp:133-299,
 *                                                  ops/join_internal.h:38-179
 *   - STR keys canonicalised by VALUE               ops/aggregate.cpp:164-187,
 *                                                  ops/join.cpp:48-71
 *   - morsel-parallel CPU driver (baseline only)    exec/parallel.cpp:189-599
 *   - tumbling window: bucket key + GROUP BY        tsx/window.cpp:305-394
 *   - backward as-of join                           tsx/asof.cpp:158-296
 *
 * All functions return 0 on success and a negative code on a usage error
 * (orc_last_error() then holds a message). No exceptions cross this boundary.
 */
#ifndef QE_ORACLE_H
#define QE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors qe::Type (core/types.h:18). */
enum { ORC_I32 = 0, ORC_I64 = 1, ORC_F64 = 2, ORC_BOOL = 3, ORC_TS = 4, ORC_STR = 5 };
/* Mirrors qe::AggFunc (ops/aggregate.h:61). */
enum { ORC_COUNT_STAR = 0, ORC_COUNT = 1, ORC_SUM = 2, ORC_MIN = 3, ORC_MAX = 4, ORC_AVG = 5 };
/* Mirrors qe::JoinType (ops/join.h:59). */
enum { ORC_INNER = 0, ORC_LEFT = 1 };

/* Host column view, the same fields as qe::Column (core/column.h:55-67). For
 * ORC_STR, `data` holds int32 codes resolved through the dictionary given by
 * dict_offsets (dict_size+1 entries) into dict_bytes. */
typedef struct {
  int32_t type;
  uint64_t len;
  const void* data;
  const uint64_t* validity; /* NULL => no nulls */
  int32_t all_valid;
  const uint32_t* dict_offsets;
  const char* dict_bytes;
  uint32_t dict_size;
} orc_column;

typedef struct orc_result orc_result;

/* GROUP BY `key_cols` computing `naggs` aggregates over a table of `ncols`
 * columns, fed through the pull model in batches of `batch_rows` rows (a
 * positive multiple of 64, as ops/scan.cpp:15-18 requires). Output rows are in
 * first-seen group order, keys first then aggregates. */
int orc_groupby(const orc_column* cols, int ncols, const uint32_t* key_cols, int nkeys,
                const int32_t* agg_funcs, const uint32_t* agg_cols, int naggs,
                uint64_t batch_rows, orc_result** out);

/* Hash equi-join: all probe columns then all build columns, probe batch order. */
int orc_join(const orc_column* probe, int nprobe, const orc_column* build, int nbuild,
             const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
             int32_t join_type, uint64_t batch_rows, orc_result** out);

/* Tumbling window (tsx/window.cpp:305-394): GROUP BY (key_cols..., bucket)
 * with bucket = (t / width) * width of time_col, typed as the time column;
 * output keys, bucket, aggregates in first-seen group order. */
int orc_window_tumbling(const orc_column* cols, int ncols, const uint32_t* key_cols, int nkeys,
                        uint32_t time_col, int64_t width, const int32_t* agg_funcs,
                        const uint32_t* agg_cols, int naggs, uint64_t batch_rows, orc_result** out);

/* Backward as-of join (tsx/asof.cpp): probe columns then build columns, one
 * row per matched probe row (LEFT: every probe row), in probe order. */
int orc_asof_join(const orc_column* probe, int nprobe, const orc_column* build, int nbuild,
                  const uint32_t* probe_keys, const uint32_t* build_keys, int nkeys,
                  uint32_t probe_time, uint32_t build_time, int32_t asof_type, int32_t has_tol,
                  int64_t tol, orc_result** out);

/* COUNT(*) and SUM(probe_col) over the INNER join of probe and build on
 * single I64/I32 key columns -- the sink of the 16M x 256M join workload.
 * sum_valid = 0 when no matched row had a non-null payload (SQL NULL). */
int orc_join_count_sum(const orc_column* probe_key, const orc_column* probe_val,
                       const orc_column* build_key, uint64_t batch_rows,
                       int64_t* out_count, int64_t* out_sum, int32_t* sum_valid);

/* Morsel-parallel CPU baseline (restating exec/parallel.cpp): `threads`
 * workers pull `morsel_rows`-row morsels, aggregate privately, then merge.
 * threads == 0 => hardware concurrency. */
int orc_parallel_groupby(const orc_column* cols, int ncols, const uint32_t* key_cols,
                         int nkeys, const int32_t* agg_funcs, const uint32_t* agg_cols,
                         int naggs, unsigned threads, uint64_t morsel_rows,
                         orc_result** out);

/* Morsel-parallel CPU baseline of scan(probe).join(scan(build)).aggregate(
 * COUNT(*), SUM(probe payload)): each morsel's private tree rebuilds the build
 * side (exec/parallel.cpp:101-105). */
int orc_parallel_join_count_sum(const orc_column* probe_key, const orc_column* probe_val,
                                const orc_column* build_key, const orc_column* build_val,
                                unsigned threads, uint64_t morsel_rows,
                                int64_t* out_count, int64_t* out_sum, int32_t* sum_valid);

/* Result access. Column values are widened: I32/I64/TS/BOOL/STR(code) as
 * int64, F64 as double. `valid` is one byte per row (1 = valid). */
uint64_t orc_result_rows(const orc_result* r);
int orc_result_cols(const orc_result* r);
int32_t orc_result_type(const orc_result* r, int col);
int orc_result_fetch(const orc_result* r, int col, int64_t* ivals, double* fvals,
                     uint8_t* valid);
/* For STR result columns: the string of `code` in the result's dictionary. */
int orc_result_str(const orc_result* r, int col, int64_t code, const char** s,
                   uint64_t* len);
void orc_result_free(orc_result* r);

const char* orc_last_error(void);
/* splitmix64 row hash of the reference (ops/hash_kernels.h:7-12), exposed so the
 * tests can pin it against the reference's own scalar twin. */
uint64_t orc_hash_combine(uint64_t acc, uint64_t word);

#ifdef __cplusplus
}
#endif
#endif
