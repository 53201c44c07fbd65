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
