"""GPU GROUP BY parity against the oracle, through the C ABI (libqeg.so).

Mirrors the reference's tests/aggregate_differential_test.cpp: the hand-built
edge tables (NULL key group, composite key, global aggregate, all-NULL value
group, >2048-group tail, empty input, NaN MIN/MAX), each over the batch sizes
{64, 256, 2048}, then seeded random GROUP BY queries. Integer, key, count and
MIN/MAX cells must match exactly; F64 SUM/AVG within 1e-9 abs + 1e-9 rel.
"""
import math

import numpy as np
import pytest

import oracle as O
import qeg
from util import StrCanon, assert_same, gen_group_by, gen_schema, gen_table, gpu_rows, to_gpu

pytestmark = pytest.mark.gpu

BATCHES = [64, 256, 2048]
NAN = float("nan")


def run_gpu(ctx, cols, keys, aggs, batch_rows=None, config=None, device=False, sel=None):
    canon = StrCanon()
    gcols = [to_gpu(c, canon, device) for c in cols]
    res = qeg.groupby(ctx, gcols, keys, aggs, config=config, batch_rows=batch_rows, sel=sel)
    a = qeg.Aggregate(ctx, [c.type for c in gcols], keys, aggs)
    types = a.result_types
    a.close()
    return gpu_rows(res, types, canon)


def check(ctx, cols, keys, aggs, **kw):
    for bs in BATCHES:
        ot, orows = O.groupby(cols, keys, aggs, bs)
        gt, grows = run_gpu(ctx, cols, keys, aggs, batch_rows=bs, **kw)
        assert_same(gt, grows, ot, orows, "batch %d" % bs)


def edge_table():
    k = O.TCol(O.I32, np.array([1, 1, 2, 2, 3, 1, 2, 3, 0, 0], np.int32), np.array([1] * 8 + [0, 0], bool))
    v = O.TCol(O.I32, np.array([10, 20, 30, 40, 50, 60, 70, 80, 90, 100], np.int32),
               np.array([0] + [1] * 9, bool))
    f = O.TCol(O.F64, np.array([1.5, 2.5, 3.5, 4.5, 5.5, 6.5, 7.5, 8.5, 9.5, 10.5]),
               np.array([1, 1, 0, 1, 1, 1, 1, 1, 1, 1], bool))
    return [k, v, f]


FULL_AGGS = [(O.COUNT_STAR, 0), (O.COUNT, 1), (O.SUM, 1), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1), (O.SUM, 2),
             (O.AVG, 2)]


def test_edge_single_key_with_null_group(ctx):
    check(ctx, edge_table(), [0], FULL_AGGS)


def test_edge_composite_key_i32_f64(ctx):
    check(ctx, edge_table(), [0, 2], [(O.COUNT_STAR, 0), (O.SUM, 1)])


def test_edge_global_aggregate(ctx):
    check(ctx, edge_table(), [], FULL_AGGS)


def test_edge_all_null_value_group(ctx):
    k = O.TCol(O.I32, np.array([1, 1, 2, 2], np.int32))
    v = O.TCol(O.I32, np.array([0, 0, 5, 6], np.int32), np.array([0, 0, 1, 1], bool))
    aggs = [(O.COUNT_STAR, 0), (O.COUNT, 1), (O.SUM, 1), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1)]
    check(ctx, [k, v], [0], aggs)
    # Expected values written in the reference's test: group 1 has SUM/MIN/MAX/AVG NULL.
    gt, grows = run_gpu(ctx, [k, v], [0], aggs)
    d = {r[0]: r[1:] for r in grows}
    assert d[1] == (2, 0, None, None, None, None)
    assert d[2] == (2, 2, 11, 5, 6, 5.5)


def test_edge_skew_and_tail_over_2048_groups(ctx):
    i = np.arange(6000)
    k = O.TCol(O.I32, (i % 5).astype(np.int32))
    v = O.TCol(O.I64, ((i % 100) - 50).astype(np.int64))
    check(ctx, [k, v], [1], [(O.COUNT_STAR, 0), (O.SUM, 0)])
    check(ctx, [k, v], [0], [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MIN, 1), (O.MAX, 1)])


def test_edge_empty_input(ctx):
    cols = [O.TCol(O.I64, np.zeros(0, np.int64)), O.TCol(O.F64, np.zeros(0))]
    aggs = [(O.COUNT_STAR, 0), (O.COUNT, 0), (O.SUM, 0), (O.MIN, 0)]
    gt, grows = run_gpu(ctx, cols, [], aggs)
    assert grows == [(0, 0, None, None)]
    check(ctx, cols, [], aggs)
    gt, grows = run_gpu(ctx, cols, [0], [(O.COUNT_STAR, 0), (O.SUM, 0)])
    assert grows == []


def test_edge_nan_min_max(ctx):
    k = O.TCol(O.I32, np.array([1, 1, 2, 2, 3, 3, 4, 4], np.int32))
    f = O.TCol(O.F64, np.array([NAN, 1.5, NAN, NAN, 2.5, 3.5, NAN, 0.0]), np.array([1] * 7 + [0], bool))
    aggs = [(O.MIN, 1), (O.MAX, 1), (O.SUM, 1), (O.AVG, 1), (O.COUNT, 1)]
    check(ctx, [k, f], [0], aggs)
    check(ctx, [k, f], [], aggs)
    # Expected per key as written in the reference's test (NaN-greatest order).
    _, grows = run_gpu(ctx, [k, f], [0], aggs)
    d = {r[0]: r[1:] for r in grows}
    assert d[1][0] == 1.5 and math.isnan(d[1][1])
    assert math.isnan(d[2][0]) and math.isnan(d[2][1])
    assert d[3][0] == 2.5 and d[3][1] == 3.5
    assert math.isnan(d[4][0]) and math.isnan(d[4][1]) and d[4][4] == 1


def test_f64_key_canonicalisation(ctx):
    # {+0, -0, NaN, -NaN, 1.5} form 3 groups (tests/hashtable_test.cpp:148-163 of the reference).
    neg_nan = np.frombuffer(np.array([0xFFF8000000000001], np.uint64).tobytes(), np.float64)[0]
    k = O.TCol(O.F64, np.array([0.0, -0.0, NAN, neg_nan, 1.5]))
    gt, grows = run_gpu(ctx, [k], [0], [(O.COUNT_STAR, 0)])
    assert len(grows) == 3
    ot, orows = O.groupby([k], [0], [(O.COUNT_STAR, 0)])
    assert_same(gt, grows, ot, orows)


@pytest.mark.parametrize("seed", range(4))
def test_random_group_by(ctx, seed):
    rng = np.random.default_rng(0x6B0179 + seed)
    for it in range(50):
        types = gen_schema(rng)
        n = int(rng.integers(0, 5001))
        cols = gen_table(rng, types, n)
        keys, aggs = gen_group_by(rng, types)
        bs = int(rng.choice(BATCHES))
        ot, orows = O.groupby(cols, keys, aggs, bs)
        gt, grows = run_gpu(ctx, cols, keys, aggs, batch_rows=bs)
        assert_same(gt, grows, ot, orows, "seed %d iter %d keys %s aggs %s" % (seed, it, keys, aggs))


@pytest.mark.parametrize("strategy", [qeg.AGG_SMEM, qeg.AGG_GLOBAL])
def test_strategies_and_forced_resize(ctx, strategy):
    rng = np.random.default_rng(7 + strategy)
    n = 200_000
    k = O.TCol(O.I64, rng.integers(-(1 << 40), 1 << 40, n).astype(np.int64) % 50_000, rng.random(n) > 0.01)
    v = O.TCol(O.F64, rng.normal(0, 1e3, n), rng.random(n) > 0.05)
    w = O.TCol(O.I64, rng.integers(-(1 << 31), 1 << 31, n).astype(np.int64))
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 2), (O.SUM, 1), (O.MIN, 2), (O.MAX, 2), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1)]
    ot, orows = O.groupby([k, v, w], [0], aggs)
    # A 1024-slot first table forces several overflow -> grow -> replay rounds.
    cfg = qeg.agg_config(strategy=strategy, sizing=qeg.SIZE_FIXED, initial_capacity=1024)
    gt, grows = run_gpu(ctx, [k, v, w], [0], aggs, config=cfg)
    assert_same(gt, grows, ot, orows)


def test_selection_vector(ctx):
    rng = np.random.default_rng(11)
    n = 10_000
    cols = [O.TCol(O.I32, rng.integers(0, 100, n).astype(np.int32)), O.TCol(O.F64, rng.uniform(0, 1, n))]
    sel = np.sort(rng.choice(n, 3000, replace=False)).astype(np.uint32)
    sub = [O.TCol(c.type, c.values[sel]) for c in cols]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MAX, 1)]
    ot, orows = O.groupby(sub, [0], aggs)
    gt, grows = run_gpu(ctx, cols, [0], aggs, sel=sel)
    assert_same(gt, grows, ot, orows)


def test_device_resident_columns(ctx):
    rng = np.random.default_rng(5)
    n = 100_000
    cols = [O.TCol(O.I64, rng.integers(0, 1024, n).astype(np.int64)),
            O.TCol(O.F64, rng.uniform(0, 1000, n), rng.random(n) > 0.05)]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.AVG, 1), (O.MIN, 1), (O.MAX, 1)]
    ot, orows = O.groupby(cols, [0], aggs)
    gt, grows = run_gpu(ctx, cols, [0], aggs, device=True)
    assert_same(gt, grows, ot, orows)


def test_str_keys_group_by_value_across_dictionaries(ctx):
    # Two batches whose dictionaries hold the same strings under different codes.
    d1 = ["AAPL", "MSFT", "GOOG"]
    d2 = ["GOOG", "AAPL", "IBM", "MSFT"]
    canon = StrCanon(d1 + d2)
    b1 = [O.TCol(O.STR, np.array([0, 1, 2, 0], np.int32), None, d1), O.TCol(O.I64, np.array([1, 2, 3, 4], np.int64))]
    b2 = [O.TCol(O.STR, np.array([1, 0, 2, 3], np.int32), None, d2), O.TCol(O.I64, np.array([10, 30, 7, 20], np.int64))]
    a = qeg.Aggregate(ctx, [O.STR, O.I64], [0], [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MIN, 0)])
    a.consume([to_gpu(c, canon) for c in b1])
    a.consume([to_gpu(c, canon) for c in b2])
    a.finish()
    res = a.fetch()
    rows = {canon.values[int(k)]: (int(n), int(s), canon.values[int(m)])
            for k, n, s, m in zip(res[0][0], res[1][0], res[2][0], res[3][0])}
    assert rows == {"AAPL": (3, 15, "AAPL"), "MSFT": (2, 22, "MSFT"), "GOOG": (2, 33, "GOOG"),
                    "IBM": (1, 7, "IBM")}
    a.close()


@pytest.mark.parametrize("hot", [0, 512, 64])
@pytest.mark.parametrize("block", [0, 512])
def test_skewed_sketch_path_with_and_without_preloaded_hot_keys(ctx, hot, block):
    # 6M rows (above the sketch threshold), Zipf(1.2) keys over 2M values:
    # the learned sizing path, first-come CTA tables (hot = 0) and the
    # preloaded read-only heavy-hitter tables with warp-private rows for the
    # hottest keys (hot > 0), with the default and a forced block size.
    rng = np.random.default_rng(40 + hot + block)
    n, dom = 6 << 20, 2 << 20
    w = np.arange(1, dom + 1, dtype=np.float64) ** -1.2
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ranks = np.minimum(np.searchsorted(cdf, rng.random(n)), dom - 1)
    key = O.TCol(O.I64, (ranks.astype(np.int64) * 0x5851F42D4C957F2D % (1 << 62)) - (1 << 61))
    v1 = O.TCol(O.I64, rng.integers(-(1 << 31), 1 << 31, n))
    v2 = O.TCol(O.F64, rng.normal(0, 1e3, n), rng.random(n) > 0.05)
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.SUM, 2), (O.MIN, 1), (O.MAX, 1), (O.AVG, 2)]
    cfg = qeg.agg_config(sizing=qeg.SIZE_LEARNED, hot_keys=hot, block_threads=block)
    ot, orows = O.groupby([key, v1, v2], [0], aggs, 1 << 23)
    gt, grows = run_gpu(ctx, [key, v1, v2], [0], aggs, config=cfg)
    assert_same(gt, grows, ot, orows, "hot %d block %d" % (hot, block))


@pytest.mark.parametrize("slots,cap", [(64, 1024), (1024, 0), (128, 4096)])
def test_composite_keys_private_tables_with_flushes(ctx, slots, cap):
    # Composite keys through CTA-private tables that flush into the global
    # table whenever half full: tiny private tables force many flushes, a tiny
    # fixed global table forces the global-full path (rows spill, partial rows
    # of the final flush go to the partial-row list, grow and replay).
    rng = np.random.default_rng(50 + slots)
    n = 400000
    k1 = O.TCol(O.I32, rng.integers(0, 300, n).astype(np.int32), rng.random(n) > 0.03)
    k2 = O.TCol(O.I64, np.sort(rng.integers(0, 2000, n)), rng.random(n) > 0.03)  # ordered, like time buckets
    v1 = O.TCol(O.F64, rng.normal(0, 10, n), rng.random(n) > 0.1)
    v2 = O.TCol(O.I64, rng.integers(-1000, 1000, n))
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 2), (O.AVG, 2), (O.MIN, 3), (O.MAX, 3), (O.COUNT, 2)]
    cfg = qeg.agg_config(strategy=qeg.AGG_SMEM, smem_slots=slots,
                         sizing=qeg.SIZE_FIXED if cap else qeg.SIZE_LEARNED, initial_capacity=cap)
    ot, orows = O.groupby([k1, k2, v1, v2], [0, 1], aggs, 1 << 20)
    gt, grows = run_gpu(ctx, [k1, k2, v1, v2], [0, 1], aggs, config=cfg)
    assert_same(gt, grows, ot, orows, "slots %d cap %d" % (slots, cap))


def _zipf_rows(rng, n, dom, s):
    w = np.arange(1, dom + 1, dtype=np.float64) ** -s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(n)), dom - 1).astype(np.int64)


@pytest.mark.parametrize("case", ["i64_skew", "i32_uniform", "f64_keys", "str_keys", "few_parts_fail",
                                  "zipf_preload", "sel", "hot_preload", "count_only", "generic_fields"])
def test_partitioned_strategy(ctx, case, monkeypatch):
    """The partitioned GROUP BY (QEG_AGG_PARTITIONED): a sizing pass counts the
    rows of every key-hash partition, the first pass aggregates the preloaded
    heavy hitters in read-only private tables and appends every other row to
    its partition's region, the second pass aggregates one partition per CTA
    in shared memory, and finalize merges tail rows whose key the global table
    also holds. Cases: skewed and uniform keys, F64 keys (-0.0 / NaN
    canonicalised), STR keys through a code map, NULL keys and key 0 (side
    rows), 2 partitions of many groups (second-pass tables too full: those
    partitions go to the global table), the sketch's heavy hitters preloaded
    (5M rows), a selection vector, 64 preloaded heavy hitters, COUNT(*) alone,
    and a field set without a specialised kernel."""
    cases = ["i64_skew", "i32_uniform", "f64_keys", "str_keys", "few_parts_fail", "zipf_preload", "sel",
             "hot_preload", "count_only", "generic_fields"]
    rng = np.random.default_rng(900 + cases.index(case))
    n = 300_000
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.SUM, 2), (O.MIN, 1), (O.MAX, 1), (O.AVG, 2)]
    kvalid = rng.random(n) > 0.02
    sel = None
    cfg = qeg.agg_config(strategy=qeg.AGG_PARTITIONED)
    canon = None
    if case == "i64_skew":
        key = O.TCol(O.I64, _zipf_rows(rng, n, 100_000, 1.1) * 0x9E3779B97F4A7C1 - 12345, kvalid)
        key.values[:50] = 0
    elif case == "i32_uniform":
        key = O.TCol(O.I32, rng.integers(-(1 << 30), 1 << 30, n).astype(np.int32) % 40_000, kvalid)
    elif case == "f64_keys":
        vals = rng.integers(0, 20_000, n).astype(np.float64) - 10_000.5
        vals[::97] = -0.0
        vals[1::97] = 0.0
        vals[2::89] = np.nan
        key = O.TCol(O.F64, vals, kvalid)
    elif case == "str_keys":
        d = ["S%05d" % i for i in range(30_000)]
        key = O.TCol(O.STR, rng.integers(0, len(d), n).astype(np.int32), kvalid, d)
        aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MAX, 1), (O.MIN, 2)]
    elif case == "few_parts_fail":
        monkeypatch.setenv("QEG_AGG_PART_BITS", "1")
        key = O.TCol(O.I64, rng.integers(0, 60_000, n).astype(np.int64), kvalid)
    elif case == "zipf_preload":
        # Above the sketch threshold: the sketch's heavy hitters (up to 1024)
        # are preloaded into the read-only private tables.
        n = 5 << 20
        kvalid = rng.random(n) > 0.02
        key = O.TCol(O.I64, _zipf_rows(rng, n, 500_000, 1.3) * 0x9E3779B97F4A7C1, kvalid)
    elif case == "sel":
        key = O.TCol(O.I64, rng.integers(0, 50_000, n).astype(np.int64), kvalid)
        sel = np.sort(rng.choice(n, n // 3, replace=False)).astype(np.uint32)
    elif case == "hot_preload":
        key = O.TCol(O.I64, _zipf_rows(rng, n, 80_000, 1.2), kvalid)
        cfg = qeg.agg_config(strategy=qeg.AGG_PARTITIONED, hot_keys=64, expected_groups=60_000)
    elif case == "count_only":
        key = O.TCol(O.I64, rng.integers(0, 70_000, n).astype(np.int64), kvalid)
        aggs = [(O.COUNT_STAR, 0)]
    else:  # generic_fields: three value columns
        key = O.TCol(O.I64, rng.integers(0, 45_000, n).astype(np.int64), kvalid)
        aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MIN, 2), (O.MAX, 3), (O.AVG, 3), (O.COUNT, 1)]
    v1 = O.TCol(O.I64, rng.integers(-(1 << 31), 1 << 31, n).astype(np.int64))
    v2 = O.TCol(O.F64, rng.normal(0, 1e3, n))
    cols = [key, v1, v2]
    if case == "generic_fields":
        cols.append(O.TCol(O.I32, rng.integers(-1000, 1000, n).astype(np.int32)))
    if case == "str_keys":
        canon = StrCanon(key.dictionary)
    sub = cols if sel is None else [O.TCol(c.type, c.values[sel], None if c.valid is None else c.valid[sel],
                                           c.dictionary) for c in cols]
    ot, orows = O.groupby(sub, [0], aggs, 1 << 20)
    gcols = [to_gpu(c, canon) for c in cols]
    a = qeg.Aggregate(ctx, [c.type for c in gcols], [0], aggs, cfg)
    a.consume(gcols, sel)
    a.finish()
    st = a.stats()
    res = a.fetch()
    types = a.result_types
    a.close()
    assert st["strategy"] == qeg.AGG_PARTITIONED, st
    gt, grows = gpu_rows(res, types, canon)
    assert_same(gt, grows, ot, orows, case)


def test_partitioned_strategy_multiple_batches_and_null_values(ctx):
    """Several consume() calls: each batch's partitioned passes run after the
    previous batch's tail rows moved into the global table; a batch with NULL
    values ends the partitioned passes (its rows take the private-table path)."""
    rng = np.random.default_rng(77)
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.COUNT, 2), (O.AVG, 2), (O.MIN, 1)]
    batches = []
    for b in range(4):
        n = 120_000 + 64 * b
        key = O.TCol(O.I64, rng.integers(0, 60_000, n).astype(np.int64), rng.random(n) > 0.01)
        v1 = O.TCol(O.I64, rng.integers(-1000, 1000, n).astype(np.int64))
        v2 = O.TCol(O.F64, rng.normal(0, 1, n), (rng.random(n) > 0.2) if b == 2 else None)
        batches.append([key, v1, v2])
    whole = [O.TCol(t, np.concatenate([bt[i].values for bt in batches]),
                    np.concatenate([bt[i].valid if bt[i].valid is not None else np.ones(bt[i].n, bool)
                                    for bt in batches]))
             for i, t in enumerate([O.I64, O.I64, O.F64])]
    ot, orows = O.groupby(whole, [0], aggs, 1 << 20)
    a = qeg.Aggregate(ctx, [O.I64, O.I64, O.F64], [0], aggs, qeg.agg_config(strategy=qeg.AGG_PARTITIONED))
    for bt in batches:
        a.consume([to_gpu(c) for c in bt])
    a.finish()
    res = a.fetch()
    types = a.result_types
    a.close()
    gt, grows = gpu_rows(res, types)
    assert_same(gt, grows, ot, orows)


def test_partitioned_strategy_chosen_for_large_tables(ctx):
    """QEG_AGG_AUTO takes the partitioned strategy when the estimated global
    table is far larger than L2 (8M rows over ~6M keys): results unchanged."""
    rng = np.random.default_rng(5)
    n = 8 << 20
    key = O.TCol(O.I64, rng.integers(0, 6_000_000, n).astype(np.int64) * 7919)
    v = O.TCol(O.F64, rng.uniform(-1, 1, n))
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.MAX, 1)]
    ot, orows = O.groupby([key, v], [0], aggs, 1 << 23)
    a = qeg.Aggregate(ctx, [O.I64, O.F64], [0], aggs, qeg.agg_config(sizing=qeg.SIZE_LEARNED))
    a.consume([to_gpu(key), to_gpu(v)])
    a.finish()
    st = a.stats()
    res = a.fetch()
    types = a.result_types
    a.close()
    assert st["strategy"] == qeg.AGG_PARTITIONED, st
    gt, grows = gpu_rows(res, types)
    assert_same(gt, grows, ot, orows)
