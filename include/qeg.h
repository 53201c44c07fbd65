/*
 * qeg.h -- C ABI of the GB300 (sm_103a) hash GROUP BY / hash equi-join engine.
 *
 * This is the drop-in boundary beneath the reference engine's pull-based
 * operators (explorer-skp/query-engine). A host operator that implements the
 * reference's `Operator` contract (ops/operator.h:40-47) drains its children,
 * hands each batch's columns to these entry points, and re-emits the result as
 * ordinary `Batch` views. The ABI uses plain pointers, sizes and status codes:
 * no C++ types, no exceptions, no torch types.
 *
 * Column layout is the reference's (core/column.h:55-67, core/validity.h:21-63):
 * one contiguous value array per column (I32/STR 4 bytes, I64/F64/TS 8 bytes,
 * BOOL 1 byte) and an optional validity bitmap of 64-bit words, bit i of word
 * i/64, LSB-first, 1 = valid. `all_valid != 0` means "no nulls, ignore the
 * bitmap". Pointers may be device pointers (used in place) or host pointers
 * (copied to the device inside the call).
 *
 * Threading: a qeg_ctx and the objects created from it are single-threaded,
 * like the reference's operators (exec/parallel.h:15-19). Independent contexts
 * may be used concurrently from different threads; they share no mutable state.
 */
#ifndef QEG_H
#define QEG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * The reference reports errors with C++ exceptions; across this ABI each has a
 * status code and qeg_last_error() holds the message:
 *   QEG_ERR_INVALID   <- std::invalid_argument (ops/join.cpp:118-122,
 *                        ops/aggregate.cpp:85-90, ops/scan.cpp:15-18)
 *   QEG_ERR_OVERFLOW  <- std::overflow_error (ops/hashtable.cpp:64-65)
 *   QEG_ERR_OOM       <- std::bad_alloc (core/buffer.cpp:23)
 *   QEG_ERR_TIMEOUT   a bounded device-side wait ran out (no reference analogue)
 *   QEG_ERR_CUDA      any other CUDA runtime failure                        */
typedef int32_t qeg_status;
#define QEG_OK 0
#define QEG_ERR_INVALID (-1)
#define QEG_ERR_OVERFLOW (-2)
#define QEG_ERR_OOM (-3)
#define QEG_ERR_CUDA (-4)
#define QEG_ERR_TIMEOUT (-5)
#define QEG_ERR_UNSUPPORTED (-6)
#define QEG_ERR_NO_DEVICE (-7)

/* qe::Type (core/types.h:18), same numbering. */
#define QEG_I32 0
#define QEG_I64 1
#define QEG_F64 2
#define QEG_BOOL 3
#define QEG_TS 4
#define QEG_STR 5

/* qe::AggFunc (ops/aggregate.h:61), same numbering. */
#define QEG_COUNT_STAR 0
#define QEG_COUNT 1
#define QEG_SUM 2
#define QEG_MIN 3
#define QEG_MAX 4
#define QEG_AVG 5

/* qe::JoinType (ops/join.h:59), same numbering. */
#define QEG_INNER 0
#define QEG_LEFT 1

/* Aggregation strategy (no reference analogue: the reference has one CPU path). */
#define QEG_AGG_AUTO 0   /* chosen from the key-column sketch + estimator     */
#define QEG_AGG_SMEM 1   /* shared-memory private tables + global merge       */
#define QEG_AGG_GLOBAL 2 /* global-atomic table only                          */
#define QEG_AGG_PARTITIONED 3 /* single key: private tables, the other rows split
                                 by key-hash partition and aggregated one
                                 partition per CTA in shared memory           */

/* Table sizing. */
#define QEG_SIZE_LEARNED 0 /* capacity from the learned estimator             */
#define QEG_SIZE_FIXED 1   /* fixed initial capacity, overflow -> resize      */

/* Join strategy. */
#define QEG_JOIN_AUTO 0
#define QEG_JOIN_HASH 1        /* one global hash table                      */
#define QEG_JOIN_PARTITIONED 2 /* radix-partitioned build and probe          */
#define QEG_JOIN_DENSE 3       /* direct-mapped table over the key range     */

/* A column view: the fields of qe::Column (core/column.h:55-67). For QEG_STR,
 * `code_map` (host or device, `code_map_len` entries) translates each
 * dictionary code to a canonical value id; equal string values must map to
 * equal ids, which is how the reference compares STR by value
 * (ops/aggregate.cpp:164-187, ops/join.cpp:48-71). */
typedef struct qeg_column {
  int32_t type;
  int32_t all_valid;
  uint64_t len;
  const void* data;
  const uint64_t* validity;
  const int32_t* code_map;
  uint64_t code_map_len;
} qeg_column;

/* An output column: caller-owned buffers (host or device) with room for the
 * requested rows. `validity` receives ceil(rows/64) words; `all_valid` (may be
 * NULL) receives 1 when the fetched range holds no NULL. */
typedef struct qeg_out_column {
  void* data;
  uint64_t* validity;
  int32_t* all_valid;
} qeg_out_column;

/* One aggregate: qe::AggSpec (ops/aggregate.h:75-89) without the name. */
typedef struct qeg_agg_spec {
  int32_t func;
  uint32_t input_col; /* ignored for QEG_COUNT_STAR */
} qeg_agg_spec;

typedef struct qeg_agg_config {
  int32_t strategy;          /* QEG_AGG_*                                   */
  int32_t sizing;            /* QEG_SIZE_*                                  */
  uint64_t initial_capacity; /* QEG_SIZE_FIXED: first table capacity (0 = 2^20) */
  uint64_t expected_groups;  /* > 0: skip estimation, size for this many    */
  int32_t block_threads;     /* 0 = tuned                                   */
  int32_t rows_per_thread;   /* 0 = tuned                                   */
  int32_t smem_slots;        /* 0 = tuned                                   */
  int32_t hot_keys;          /* > 0: preload that many sketch heavy hitters into the
                                  CTA tables (the hottest 32 in warp-private rows);
                                  0 or -1: first-come CTA tables (the default) */
} qeg_agg_config;

typedef struct qeg_join_config {
  int32_t strategy;       /* QEG_JOIN_*                                     */
  int32_t partition_bits; /* QEG_JOIN_PARTITIONED: 0 = tuned                */
  int32_t sizing;         /* QEG_SIZE_LEARNED (0): a single-key hash table of
                             a large build side is sized from the estimated
                             distinct build keys (sketch + estimator), and
                             rebuilt at full size if it overflows;
                             QEG_SIZE_FIXED: two slots per build row       */
} qeg_join_config;

typedef struct qeg_ctx qeg_ctx;
typedef struct qeg_agg qeg_agg;
typedef struct qeg_join qeg_join;

/* ---- context --------------------------------------------------------------*/
/* Creates a context on CUDA device `device` with its own stream. Destroy every
 * qeg_agg / qeg_join created from a context before destroying the context. */
qeg_status qeg_ctx_create(int device, qeg_ctx** out);
void qeg_ctx_destroy(qeg_ctx* ctx);
/* Message of the last failing call on this context (thread-local when ctx is
 * NULL or creation failed). */
const char* qeg_last_error(const qeg_ctx* ctx);
/* The CUDA stream (cudaStream_t) all work of this context is ordered on. */
void* qeg_ctx_stream(qeg_ctx* ctx);
/* Waits for all work of the context; returns the first device error seen. */
qeg_status qeg_ctx_synchronize(qeg_ctx* ctx);
/* Number of kernels this context has launched (for launch accounting). */
uint64_t qeg_ctx_kernel_launches(const qeg_ctx* ctx);
/* Page-locked host memory for staging columns and receiving results (no
 * counterpart in the reference, whose buffers are ordinary aligned heap memory,
 * core/buffer.cpp:23): copies between it and the device run at the host link's
 * full speed. `*out` is NULL when bytes == 0. qeg_host_free(NULL) is a no-op. */
qeg_status qeg_host_alloc(uint64_t bytes, void** out);
void qeg_host_free(void* p);
/* Device-resident columns, the GPU counterpart of the reference's in-memory
 * Table (ops/table.h:24-47): device memory on the context's device that
 * outlives the calls using it, filled once and read in place by every query
 * (a qeg_column whose pointers are device pointers is used without a copy).
 * qeg_dev_upload / qeg_dev_download copy `bytes` between host memory and
 * such a buffer and return when the copy is complete. `*out` is NULL when
 * bytes == 0; qeg_dev_free(NULL) is a no-op. */
qeg_status qeg_dev_alloc(qeg_ctx* ctx, uint64_t bytes, void** out);
qeg_status qeg_dev_upload(qeg_ctx* ctx, void* dst, const void* src, uint64_t bytes);
qeg_status qeg_dev_download(qeg_ctx* ctx, void* dst, const void* src, uint64_t bytes);
void qeg_dev_free(void* p);
/* Failure-detection check, no counterpart in the reference (whose CPU hash
 * table never waits on another thread; its analogue is the bounded probe of
 * ops/hashtable.h:84-89). Runs the bounded wait that every composite-key table
 * uses on a row state word that is claimed and never published, giving up
 * after `polls` polls (0..2^20). Expected result: QEG_ERR_TIMEOUT, with the
 * context still usable afterwards. */
qeg_status qeg_ctx_check_bounded_wait(qeg_ctx* ctx, int32_t polls);

/* ---- hash aggregation: replaces qe::Aggregate (ops/aggregate.h:102-144) ----
 * create  ~ Aggregate::Aggregate + open()'s setup (ops/aggregate.cpp:206-241)
 * consume ~ one pulled batch of drain_and_build (ops/aggregate.cpp:243-437);
 *           `sel` (sel_len rows, host or device) is the batch's SelectionVector
 *           (core/column.h:73-76); sel == NULL means dense rows 0..len-1
 * finish  ~ end of the drain: the number of output rows (groups; exactly 1 for
 *           a global aggregate, even over empty input)
 * fetch   ~ Aggregate::next (ops/aggregate.cpp:439-493): rows
 *           [first, first+count) of the result, key columns then aggregates,
 *           typed by qe::agg_result_type (ops/aggregate.cpp:78-97)          */
qeg_status qeg_agg_create(qeg_ctx* ctx, const int32_t* col_types, int ncols,
                          const uint32_t* key_cols, int nkeys, const qeg_agg_spec* aggs,
                          int naggs, const qeg_agg_config* cfg, qeg_agg** out);
qeg_status qeg_agg_consume(qeg_agg* agg, const qeg_column* cols, int ncols,
                           const uint32_t* sel, uint64_t sel_len);
qeg_status qeg_agg_finish(qeg_agg* agg, uint64_t* num_rows);
qeg_status qeg_agg_result_types(const qeg_agg* agg, int32_t* types);
qeg_status qeg_agg_fetch(qeg_agg* agg, uint64_t first, uint64_t count,
                         const qeg_out_column* outs);
/* Diagnostics of the finished aggregation: table capacity, resize rounds,
 * strategy and hot-key count actually used, estimated group count. */
qeg_status qeg_agg_stats(const qeg_agg* agg, uint64_t* capacity, uint32_t* resizes,
                         int32_t* strategy, int32_t* hot_keys, double* est_groups);
void qeg_agg_destroy(qeg_agg* agg);

/* ---- tumbling window: replaces qe::tsx::Window in WindowMode::Tumbling
 * (tsx/window.h:82-100, tsx/window.cpp:305-394) --------------------------
 * GROUP BY (key_cols..., bucket_start) with bucket_start = (t / width) * width
 * of the time column (C++ truncating division, typed as the time column; a
 * NULL time is a NULL bucket, and NULL keys group together). The result is an
 * ordinary qeg_agg: consume / finish / fetch / destroy as above, output
 * columns [keys..., bucket_start, aggregates...] like Window::output_schema
 * (tsx/window.cpp:243-262). Errors mirror the Window constructor
 * (tsx/window.cpp:214-241): STR partition keys or aggregate inputs, a time
 * column that is not I32/I64/TS, or width <= 0 -> QEG_ERR_INVALID. At most 7
 * partition keys. The sliding mode (a sort, not a hash table) is not here.  */
qeg_status qeg_window_create(qeg_ctx* ctx, const int32_t* col_types, int ncols,
                             const uint32_t* key_cols, int nkeys, uint32_t time_col,
                             int64_t width, const qeg_agg_spec* aggs, int naggs,
                             const qeg_agg_config* cfg, qeg_agg** out);

/* ---- hash equi-join: replaces qe::HashJoin (ops/join.h:69-123) ------------
 * create      ~ HashJoin::HashJoin (ops/join.cpp:101-123), same key-type check
 * build       ~ one build batch of build_side (ops/join.cpp:133-197): inserts
 *               the keys (NULL keys never match) and materialises the batch's
 *               columns like BuildStore::append_row (ops/join_internal.h:64-87)
 * build_finish~ end of build_side
 * probe       ~ build_pairs_for_probe (ops/join.cpp:199-247) for one probe
 *               batch; *out_rows = rows the batch joins to (LEFT: unmatched
 *               probe rows once, build columns NULL)
 * fetch       ~ HashJoin::next (ops/join.cpp:260-299): output rows
 *               [first, first+count) of the last probed batch, probe columns
 *               then build columns. Device output buffers: one gather pass
 *               straight into them (a LEFT as-of join from a row that is a
 *               multiple of 64 copies its probe columns on a side stream).
 *               Host (or mixed) buffers: gathered on the device in chunks of
 *               2^24 rows and copied out; page-locked host memory copies at
 *               the host link's speed. One stream synchronisation per call. */
qeg_status qeg_join_create(qeg_ctx* ctx, const int32_t* probe_types, int nprobe,
                           const int32_t* build_types, int nbuild, const uint32_t* probe_keys,
                           const uint32_t* build_keys, int nkeys, int32_t join_type,
                           const qeg_join_config* cfg, qeg_join** out);
qeg_status qeg_join_build(qeg_join* j, const qeg_column* cols, int ncols);
qeg_status qeg_join_build_finish(qeg_join* j);
qeg_status qeg_join_probe(qeg_join* j, const qeg_column* cols, int ncols, uint64_t* out_rows);
qeg_status qeg_join_fetch(qeg_join* j, uint64_t first, uint64_t count,
                          const qeg_out_column* outs);
/* ---- backward as-of join: replaces qe::tsx::AsofJoin (tsx/asof.h:94-150) --
 * For each probe row with key tuple k and time t: the build row with key k
 * whose time tb is the greatest tb <= t (equal times match); with
 * has_tolerance, only when t - tb <= tolerance (uint64 arithmetic, as
 * tsx/asof.cpp:283-293). NULL keys or times never match; INNER drops an
 * unmatched probe row, LEFT emits it once with the build columns NULL. Among
 * build rows with equal (key, time) the one built last is taken (the
 * reference's stable sort then last-<=, tsx/asof.cpp:269-296). nkeys may be 0
 * (one global partition). Time columns are I32/I64/TS, read as int64.
 * The result is a qeg_join: build / build_finish / probe / fetch / destroy
 * as above; probe output rows come in probe-batch order (the reference emits
 * them in (key, time) order of its sorted probe side; the row multiset is the
 * same). Errors mirror the AsofJoin constructor (tsx/asof.cpp:130-160).      */
qeg_status qeg_asof_create(qeg_ctx* ctx, const int32_t* probe_types, int nprobe,
                           const int32_t* build_types, int nbuild, const uint32_t* probe_keys,
                           const uint32_t* build_keys, int nkeys, uint32_t probe_time,
                           uint32_t build_time, int32_t asof_type, int32_t has_tolerance,
                           int64_t tolerance, qeg_join** out);
/* The aggregate sink of scan(probe).join(scan(build)).aggregate({},
 * {COUNT(*), SUM(probe_val)}) fused into the probe: adds this batch's matched
 * row count and payload sum to the running totals (single key column). */
qeg_status qeg_join_probe_count_sum(qeg_join* j, const qeg_column* probe_key,
                                    const qeg_column* probe_val);
/* Totals of all qeg_join_probe_count_sum calls so far; *sum_valid = 0 when no
 * matched row carried a non-null payload (SQL SUM over nothing is NULL). */
qeg_status qeg_join_count_sum_result(qeg_join* j, int64_t* count, int64_t* sum,
                                     int32_t* sum_valid);
/* Strategy actually used by the build (QEG_JOIN_*), the partition bits and the
 * number of distinct non-null build keys. */
qeg_status qeg_join_stats(const qeg_join* j, int32_t* strategy, int32_t* partition_bits,
                          uint64_t* distinct_keys);
/* Hash-table sizing of the build (no counterpart in the reference, whose
 * HashTable grows from a fixed start): table slots, the estimated distinct
 * build keys it was sized from (0 when sized from the row count), and how
 * many times an estimate-sized table overflowed and was rebuilt at full
 * size. Any pointer may be NULL. */
qeg_status qeg_join_sizing_stats(const qeg_join* j, uint64_t* slots, double* est_distinct, int32_t* rebuilds);
void qeg_join_destroy(qeg_join* j);

/* ---- fused filter -> inner join -> GROUP BY --------------------------------
 * Replaces the operator chain Plan::lower builds for
 *   scan(probe).filter(probe[filter_col] <op> filter_value)
 *              .join(scan(build), {probe_key}, {build_key}, JoinType::Inner)
 *              .aggregate({group_col}, aggs)
 * (plan/plan.cpp:340-404 and 581-590: Filter ops/filter.cpp:28-66, HashJoin,
 * Aggregate) with one pass over the probe side. Restrictions of the fused
 * form: the join key is STR (by value through the code maps) or an integer
 * whose build values span < 2^24; the build side has <= 2^22 rows;
 * `group_col` is a build-side column of the joined schema (probe columns then
 * build columns) and the aggregates read probe-side columns. filter_col = -1:
 * no filter; a NULL filter operand drops the row. Output: one row per group,
 * the group column (STR as canonical value ids) then the aggregates, written
 * to `outs` (capacity `out_capacity` rows; host or device). */
#define QEG_CMP_LT 0
#define QEG_CMP_LE 1
#define QEG_CMP_GT 2
#define QEG_CMP_GE 3
#define QEG_CMP_EQ 4
#define QEG_CMP_NE 5
typedef struct qeg_pipeline_desc {
  int32_t filter_col;
  int32_t filter_op;
  double filter_value;
  uint32_t probe_key;
  uint32_t build_key;
  uint32_t group_col;
  int32_t naggs;
  qeg_agg_spec aggs[16];
} qeg_pipeline_desc;
qeg_status qeg_filter_join_agg(qeg_ctx* ctx, const qeg_column* probe, int nprobe, const qeg_column* build,
                               int nbuild, const qeg_pipeline_desc* desc, uint64_t out_capacity,
                               const qeg_out_column* outs, uint64_t* num_groups);

/* ---- key-column sketch and learned estimator ------------------------------
 * No reference analogue: the reference sizes its table by growth alone
 * (ops/hashtable.h:83-94). The estimator only picks table sizes and
 * strategies; an undersized table still grows and replays, so results never
 * depend on it.
 * qeg_sketch: 80 features of a key column over a strided sample of about
 *   `sample_rows` rows (0 = 2^20): 64 HyperLogLog register-value bins and 16
 *   count-min / heavy-hitter features; also the classic (uniform-model)
 *   distinct estimate and the sampled share of rows in the top 2048 keys.
 * The estimator is an MLP 80 -> 64 -> 64 -> 2 (ReLU, BF16 weights, FP32
 * accumulation) with two outputs: a correction to the classic estimate,
 * log2(1 + groups) = log2(1 + classic non-null groups) + 32 * out0, and the
 * share of rows carried by the 2048 most frequent keys. Weights are QEG_MLP_PARAMS float32
 * (W1[64][80] b1 W2[64][64] b2 W3[2][64] b3); a context loads
 * $QEG_ESTIMATOR_WEIGHTS or estimator_weights.f32 beside libqeg.so if present.
 * qeg_estimator_grad returns the mean-squared-error loss over the batch and
 * its gradient in the same layout; qeg_estimator_train runs Adam on the GPU. */
#define QEG_SKETCH_FEATURES 80
#define QEG_MLP_PARAMS 9474
qeg_status qeg_sketch(qeg_ctx* ctx, const qeg_column* key, uint64_t sample_rows, float* features,
                      double* classic_groups, double* top_share);
/* The batch planner's sketch (qeg_batch_create): the features and classic
 * estimate of every row range [row_offsets[q], row_offsets[q+1]) of a key
 * column, one sample of about `sample_rows` rows (0 = 2^16) per range, all in
 * one launch; features holds nqueries x QEG_SKETCH_FEATURES floats. */
qeg_status qeg_sketch_batch(qeg_ctx* ctx, const qeg_column* key, uint32_t nqueries, const uint64_t* row_offsets,
                            uint64_t sample_rows, float* features, double* classic_groups);
qeg_status qeg_estimator_init(qeg_ctx* ctx, uint64_t seed);
qeg_status qeg_estimator_set_weights(qeg_ctx* ctx, const float* params);
qeg_status qeg_estimator_get_weights(qeg_ctx* ctx, float* params);
/* The dead band (log2 units) taken off the magnitude of the network's
 * correction: corrections within it are dropped, so the classic estimate
 * stands where the network only adds noise. A weights file may carry it as
 * one float32 after the QEG_MLP_PARAMS parameters; otherwise 0.125. No
 * counterpart in the reference (the estimator is this library's). */
qeg_status qeg_estimator_set_deadband(qeg_ctx* ctx, double band);
qeg_status qeg_estimator_get_deadband(qeg_ctx* ctx, double* band);
qeg_status qeg_estimator_predict(qeg_ctx* ctx, const float* features, uint32_t n, float* out);
qeg_status qeg_estimator_grad(qeg_ctx* ctx, const float* x, const float* targets, uint32_t n, float* loss,
                              float* grad);
qeg_status qeg_estimator_train(qeg_ctx* ctx, const float* x, const float* targets, uint32_t n,
                               uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                               float* final_loss);

/* ---- batched GROUP BY: many independent queries in one persistent kernel --
 * Each query q is `SELECT key, <aggs> FROM rows [row_offsets[q],
 * row_offsets[q+1]) GROUP BY key` over one integer key column and one value
 * column stored back to back -- per query, the result of one qe::Aggregate
 * (ops/aggregate.h:102-144) over that slice; the reference runs such queries
 * one plan at a time. Aggregates read column 1 (the value) or are COUNT(*).
 * With NULLs in either column every query starts on a 64-row boundary.
 * qeg_batch_create plans every query (sketch + estimator -> table size and
 * strategy through `tuning`, the autotuner's table: the first entry with
 * log2(estimated groups) <= max_log2_groups and a matching skew class wins;
 * none -> built-in defaults), allocates one table arena and captures the run
 * into a CUDA graph. The column buffers must stay valid and unchanged while
 * the batch lives. qeg_batch_run replays the graph (asynchronous);
 * qeg_batch_finish waits for it, recomputes exactly any query whose table
 * overflowed and returns the group count of every query (nqueries values);
 * qeg_batch_fetch copies one query's result columns (key, then aggregates).
 * qeg_batch_stats reports the plan of one query. */
typedef struct qeg_batch qeg_batch;
typedef struct qeg_batch_tuning {
  double max_log2_groups; /* bucket upper bound on log2(estimated groups) */
  int32_t skewed;         /* 1: bucket of queries whose top keys carry >= 30% of rows */
  int32_t smem_slots;     /* CTA-private table slots (power of two <= 4096); 0 = global table only */
  uint64_t rows_per_item; /* rows per work item of the persistent kernel */
  int32_t peer_rows;      /* 1: a warp combines its rows of one group before applying them; 0: every
                             row is applied with atomics; -1: decided from the estimate */
  int32_t reserved;
} qeg_batch_tuning;
qeg_status qeg_batch_create(qeg_ctx* ctx, uint32_t nqueries, const uint64_t* row_offsets, const qeg_column* key,
                            const qeg_column* val, const qeg_agg_spec* aggs, int naggs,
                            const qeg_batch_tuning* tuning, int ntuning, int block_threads, qeg_batch** out);
qeg_status qeg_batch_run(qeg_batch* batch);
qeg_status qeg_batch_finish(qeg_batch* batch, uint64_t* groups);
qeg_status qeg_batch_fetch(qeg_batch* batch, uint32_t query, const qeg_out_column* outs);
qeg_status qeg_batch_stats(const qeg_batch* batch, uint32_t query, double* est_groups, float* hot_share,
                           int32_t* strategy, uint32_t* fell_back);
void qeg_batch_destroy(qeg_batch* batch);

/* ---- join COUNT/SUM sink without device allocation ------------------------
 * No counterpart in the reference (whose CPU operators allocate freely).
 * For callers that must not call cudaMalloc -- engines whose device memory
 * belongs to another allocator (a fixed arena that a stray cudaMalloc would
 * fragment or exceed), plugins in a host application that accounts for every
 * device byte, paths that cannot risk an allocation stall or failure at query
 * time -- this runs the inner join's COUNT(*) / SUM(probe_val) sink entirely
 * in a fixed scratch area built into the library: a file-scope static
 * __device__ array of about 24 MiB that every GPU loading the library holds
 * until the process exits. It allocates nothing: no cudaMalloc/cudaFree, no
 * library allocator.
 *   - All columns and `out` must be device pointers (no staging copies).
 *   - The build side is limited to 1,048,576 rows; larger builds are rejected
 *     with QEG_ERR_INVALID before any GPU work (use qeg_join_build instead).
 *   - A STR key's `code_map` is used when `code_map_len` > 0 (as everywhere
 *     else); a code outside [0, code_map_len) skips its row and sets bit 1 of
 *     out[3].
 *   - Work is enqueued on `cuda_stream` (a cudaStream_t; NULL = the legacy
 *     default stream) and not synchronised; out[0] = matched row count,
 *     out[1] = SUM of the probe payload, out[2] = 1 if that SUM is non-NULL,
 *     out[3] = 0, or bit 0 if the scratch table overflowed, bit 1 if a STR
 *     code was out of range.
 *   - The first call on a device looks up the scratch's device address (with
 *     that device current); make it before any stream capture begins.
 *   - Every call shares the one scratch array and clears what must start at
 *     zero; calls whose GPU work overlaps race and corrupt each other.
 * Errors: qeg_last_error(NULL) holds the message. */
qeg_status qeg_join_count_sum_noalloc(void* cuda_stream, const qeg_column* build_key,
                                      const qeg_column* probe_key, const qeg_column* probe_val,
                                      int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
