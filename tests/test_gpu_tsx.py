"""Tick-data callers of the GPU hash table against the oracle: the tumbling
window (qeg_window_create, the reference's tsx::Window in Tumbling mode) and
the backward as-of join (qeg_asof_create, tsx::AsofJoin).

Window results compare exactly on keys, bucket starts, counts and integer
aggregates, F64 within 1e-9 abs + 1e-9 rel (unordered). As-of results come in
probe order on both sides and compare exactly (F64 payloads are copied, not
computed). Inputs are seeded tick-like tables: symbols with Zipf-skewed
activity, nanosecond-style timestamps, NULLs in keys, times and values."""
import numpy as np
import pytest

import oracle as O
import qeg
from util import StrCanon, assert_same, gpu_rows, to_gpu

pytestmark = pytest.mark.gpu

WAGGS = [(O.COUNT_STAR, 0), (O.COUNT, 2), (O.SUM, 2), (O.AVG, 2), (O.MIN, 2), (O.MAX, 2), (O.SUM, 3), (O.MIN, 3),
         (O.MAX, 3)]


def zipf(rng, n, dom, s=1.1):
    w = np.arange(1, dom + 1, dtype=np.float64) ** -s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(n)), dom - 1)


def ticks(rng, n, nsym, t_type=O.TS, t0=0, span=10 ** 12, nulls=0.02):
    """(sym I32, time, price F64, qty I64): times sorted with jitter."""
    sym = zipf(rng, n, nsym).astype(np.int32)
    t = np.sort(rng.integers(t0, t0 + span, n)) + rng.integers(-1000, 1000, n)
    dt = np.int32 if t_type == O.I32 else np.int64
    v = (lambda: rng.random(n) >= nulls) if nulls else (lambda: None)
    return [O.TCol(O.I32, sym, v()), O.TCol(t_type, t.astype(dt), v()),
            O.TCol(O.F64, rng.lognormal(4.6, 0.3, n), v()), O.TCol(O.I64, rng.integers(1, 10000, n), v())]


def run_window(ctx, cols, keys, tcol, width, aggs, cfg=None, chunks=1):
    w = qeg.Window(ctx, [c.type for c in cols], keys, tcol, width, aggs, cfg)
    try:
        n = cols[0].n
        cut = [n * i // chunks // 64 * 64 for i in range(chunks)] + [n]
        for a, b in zip(cut[:-1], cut[1:]):
            w.consume([to_gpu(O.TCol(c.type, c.values[a:b], None if c.valid is None else c.valid[a:b]))
                       for c in cols])
        w.finish()
        out = gpu_rows(w.fetch(), w.result_types)
        return out, w.stats() if hasattr(w, "stats") else None
    finally:
        w.close()


def check_window(ctx, cols, keys, tcol, width, aggs=WAGGS, **kw):
    (gt, grows), _ = run_window(ctx, cols, keys, tcol, width, aggs, **kw)
    ot, orows = O.window_tumbling(cols, keys, tcol, width, aggs)
    assert gt == ot
    assert len(grows) == len(orows)
    assert_same(gt, grows, ot, orows, "window keys=%s width=%d" % (keys, width))
    return len(orows)


def test_window_ticks_by_symbol_minute(ctx):
    rng = np.random.default_rng(1)
    cols = ticks(rng, 1 << 20, 500)
    assert check_window(ctx, cols, [0], 1, 60 * 10 ** 9) > 1000


def test_window_global_buckets_takes_sketch_path(ctx):
    # 5M rows and no partition key: the single-key fast path with the sketch,
    # the learned estimate and heavy-hitter preloading all read bucketed keys.
    rng = np.random.default_rng(2)
    cols = ticks(rng, 5 << 20, 50, span=10 ** 10, nulls=0.01)
    check_window(ctx, cols, [], 1, 10 ** 6, aggs=[(O.COUNT_STAR, 0), (O.SUM, 3), (O.MAX, 2)])


def test_window_i32_time_negative_times_composite_keys(ctx):
    rng = np.random.default_rng(3)
    n = 300000
    cols = ticks(rng, n, 40, t_type=O.I32, t0=-(1 << 30), span=1 << 31, nulls=0.05)
    cols.append(O.TCol(O.I64, rng.integers(0, 7, n), rng.random(n) > 0.05))
    check_window(ctx, cols, [0, 4], 1, 1 << 20)
    check_window(ctx, cols, [4], 1, 999983, aggs=[(O.COUNT_STAR, 0), (O.MIN, 1), (O.MAX, 1)])


def test_window_grow_and_replay_and_chunks(ctx):
    # A tiny fixed table: the first pass spills, grows and replays the spilled
    # rows; three consume calls.
    rng = np.random.default_rng(4)
    cols = ticks(rng, 400000, 3000)
    cfg = qeg.agg_config(sizing=qeg.SIZE_FIXED, initial_capacity=1024)
    check_window(ctx, cols, [0], 1, 10 ** 9, cfg=cfg, chunks=3)


def test_window_width_one_and_huge_width(ctx):
    rng = np.random.default_rng(5)
    cols = ticks(rng, 100000, 20, span=50000)
    check_window(ctx, cols, [0], 1, 1)
    check_window(ctx, cols, [0], 1, 1 << 62)


def test_window_empty_input(ctx):
    cols = [O.TCol(O.I32, np.zeros(0, np.int32)), O.TCol(O.TS, np.zeros(0, np.int64)),
            O.TCol(O.F64, np.zeros(0)), O.TCol(O.I64, np.zeros(0, np.int64))]
    (gt, rows), _ = run_window(ctx, cols, [0], 1, 10, WAGGS)
    assert rows == []


def test_window_rejects_bad_arguments(ctx):
    types = [O.I32, O.TS, O.F64, O.STR]
    aggs = [(O.COUNT_STAR, 0)]
    for args in (([0], 1, 0, aggs), ([0], 2, 10, aggs), ([3], 1, 10, aggs), ([0], 1, 10, [(O.MIN, 3)]),
                 ([0], 9, 10, aggs)):
        with pytest.raises(qeg.QegError):
            qeg.Window(ctx, types, *args)


# ---------------------------------------------------------------------------
# as-of join
# ---------------------------------------------------------------------------
def run_asof(ctx, probe, build, pk, bk, pt, bt, jt, tol, canon=None, build_chunks=1, probe_chunks=1):
    j = qeg.AsofJoin(ctx, [c.type for c in probe], [c.type for c in build], pk, bk, pt, bt, jt, tol)
    types = [c.type for c in probe] + [c.type for c in build]
    try:
        def sl(c, a, b):
            return O.TCol(c.type, c.values[a:b], None if c.valid is None else c.valid[a:b], c.dictionary)

        nb = build[0].n
        cut = [nb * i // build_chunks for i in range(build_chunks)] + [nb]
        for a, b in zip(cut[:-1], cut[1:]):
            j.build([to_gpu(sl(c, a, b), canon) for c in build])
        j.build_finish()
        rows = []
        npr = probe[0].n
        cut = [npr * i // probe_chunks for i in range(probe_chunks)] + [npr]
        for a, b in zip(cut[:-1], cut[1:]):
            n = j.probe([to_gpu(sl(c, a, b), canon) for c in probe])
            if n:
                rows += gpu_rows(j.fetch(0, n), types, canon)[1]
        return types, rows
    finally:
        j.close()


def check_asof(ctx, probe, build, pk, bk, pt, bt, jt, tol=None, canon=None, **kw):
    gt, grows = run_asof(ctx, probe, build, pk, bk, pt, bt, jt, tol, canon, **kw)
    ot, orows = O.asof_join(probe, build, pk, bk, pt, bt, jt, tol)
    assert len(grows) == len(orows)
    # Both sides emit in probe order: compare row by row (NaN == NaN).
    for i, (a, b) in enumerate(zip(grows, orows)):
        if a != b:
            assert O.compare(gt, [a], ot, [b]) is None, (i, a, b)
    return len(orows)


@pytest.mark.parametrize("jt", [O.INNER, O.LEFT])
@pytest.mark.parametrize("tol", [None, 5 * 10 ** 6])
def test_asof_trades_against_quotes(ctx, jt, tol):
    rng = np.random.default_rng(10)
    quotes = ticks(rng, 200000, 2000, span=10 ** 11)
    trades = ticks(rng, 300000, 2200, span=10 ** 11)
    n = check_asof(ctx, trades, quotes, [0], [0], 1, 1, jt, tol)
    assert n > 1000


def test_asof_key_strategies(ctx):
    rng = np.random.default_rng(11)
    n = 100000
    # dense small-range keys, spread int64 keys (hash), composite keys
    for kt, gen in ((O.I32, lambda m: rng.integers(0, 300, m).astype(np.int32)),
                    (O.I64, lambda m: rng.integers(0, 300, m).astype(np.int64) * 0x9E3779B97F4A7C1 + 5)):
        build = [O.TCol(kt, gen(n), rng.random(n) > 0.02), O.TCol(O.TS, rng.integers(0, 10 ** 7, n)),
                 O.TCol(O.F64, rng.random(n))]
        probe = [O.TCol(kt, gen(n), rng.random(n) > 0.02), O.TCol(O.TS, rng.integers(0, 10 ** 7, n))]
        check_asof(ctx, probe, build, [0], [0], 1, 1, O.LEFT)
    build = [O.TCol(O.I32, rng.integers(0, 30, n).astype(np.int32)), O.TCol(O.I64, rng.integers(0, 9, n)),
             O.TCol(O.TS, rng.integers(0, 10 ** 6, n)), O.TCol(O.I64, np.arange(n))]
    probe = [O.TCol(O.I32, rng.integers(0, 31, n).astype(np.int32)), O.TCol(O.I64, rng.integers(0, 10, n)),
             O.TCol(O.TS, rng.integers(0, 10 ** 6, n))]
    check_asof(ctx, probe, build, [0, 1], [0, 1], 2, 2, O.INNER)


def test_asof_equal_build_times_take_the_last_built_row(ctx):
    rng = np.random.default_rng(12)
    n = 200000
    build = [O.TCol(O.I32, rng.integers(0, 50, n).astype(np.int32)), O.TCol(O.TS, rng.integers(0, 100, n)),
             O.TCol(O.I64, np.arange(n))]
    probe = [O.TCol(O.I32, rng.integers(0, 50, n).astype(np.int32)), O.TCol(O.TS, rng.integers(-5, 105, n))]
    check_asof(ctx, probe, build, [0], [0], 1, 1, O.LEFT, build_chunks=3, probe_chunks=2)


def test_asof_zero_keys_and_empty_sides(ctx):
    rng = np.random.default_rng(13)
    n = 50000
    build = [O.TCol(O.TS, rng.integers(0, 10 ** 6, n), rng.random(n) > 0.1), O.TCol(O.I64, np.arange(n))]
    probe = [O.TCol(O.TS, rng.integers(-10, 10 ** 6 + 10, n), rng.random(n) > 0.1)]
    check_asof(ctx, probe, build, [], [], 0, 0, O.LEFT, 1000)
    check_asof(ctx, probe, build, [], [], 0, 0, O.INNER)
    empty_b = [O.TCol(O.TS, np.zeros(0, np.int64)), O.TCol(O.I64, np.zeros(0, np.int64))]
    check_asof(ctx, probe, empty_b, [], [], 0, 0, O.LEFT)
    check_asof(ctx, probe, empty_b, [], [], 0, 0, O.INNER)
    empty_p = [O.TCol(O.TS, np.zeros(0, np.int64))]
    check_asof(ctx, empty_p, build, [], [], 0, 0, O.LEFT)


def test_asof_extreme_times_and_tolerances(ctx):
    lo, hi = -(1 << 63), (1 << 63) - 1
    build = [O.TCol(O.I32, np.array([1, 1, 1, 1, 2], np.int32)), O.TCol(O.TS, np.array([lo, -2, 0, hi, 7])),
             O.TCol(O.I64, np.arange(5))]
    probe = [O.TCol(O.I32, np.array([1, 1, 1, 1, 2, 2], np.int32)),
             O.TCol(O.TS, np.array([hi, lo, 5, -3, 7, 6]))]
    for tol in (None, 0, 10, hi, -1):
        for jt in (O.INNER, O.LEFT):
            check_asof(ctx, probe, build, [0], [0], 1, 1, jt, tol)


def test_asof_i32_probe_time_and_str_keys(ctx):
    rng = np.random.default_rng(14)
    n = 40000
    bd, pd = ["S%03d" % i for i in range(80)], ["S%03d" % i for i in range(79, -1, -1)] + ["ZZZ"]
    build = [O.TCol(O.STR, rng.integers(0, len(bd), n).astype(np.int32), rng.random(n) > 0.02, bd),
             O.TCol(O.TS, rng.integers(0, 1 << 30, n)), O.TCol(O.F64, rng.random(n))]
    probe = [O.TCol(O.STR, rng.integers(0, len(pd), n).astype(np.int32), rng.random(n) > 0.02, pd),
             O.TCol(O.I32, rng.integers(0, 1 << 30, n).astype(np.int32))]
    canon = StrCanon(bd + pd)
    check_asof(ctx, probe, build, [0], [0], 1, 1, O.LEFT, canon=canon)


def test_asof_rejects_bad_arguments(ctx):
    with pytest.raises(qeg.QegError):  # F64 time column
        qeg.AsofJoin(ctx, [O.I32, O.F64], [O.I32, O.TS], [0], [0], 1, 1)
    with pytest.raises(qeg.QegError):  # key types differ
        qeg.AsofJoin(ctx, [O.I64, O.TS], [O.I32, O.TS], [0], [0], 1, 1)
    with pytest.raises(qeg.QegError):  # time column out of range
        qeg.AsofJoin(ctx, [O.I32, O.TS], [O.I32, O.TS], [0], [0], 1, 2)
    j = qeg.AsofJoin(ctx, [O.I64, O.TS], [O.I64, O.TS], [0], [0], 1, 1)
    j.build([to_gpu(O.TCol(O.I64, np.arange(4))), to_gpu(O.TCol(O.TS, np.arange(4)))])
    j.build_finish()
    with pytest.raises(qeg.QegError):  # the count/sum sink is not an as-of join
        j.probe_count_sum(to_gpu(O.TCol(O.I64, np.arange(4))), to_gpu(O.TCol(O.I64, np.arange(4))))
    j.close()


@pytest.mark.parametrize("jt", [O.INNER, O.LEFT])
def test_asof_time_ordered_sides(ctx, jt):
    # A build side in time order without NULL times takes the slot-only sort;
    # equal times within a symbol must still resolve to the last built row.
    # The probe side in time order exercises the galloping search from the
    # per-CTA hints; a shuffled copy of it must give the same rows.
    rng = np.random.default_rng(15)
    nb, npr = 300000, 600000
    bts = np.sort(rng.integers(0, 10 ** 9, nb) // 1000 * 1000)  # many equal times
    build = [O.TCol(O.I32, zipf(rng, nb, 300).astype(np.int32), rng.random(nb) > 0.01), O.TCol(O.TS, bts),
             O.TCol(O.I64, np.arange(nb))]
    pts = np.sort(rng.integers(-1000, 10 ** 9 + 1000, npr))
    probe = [O.TCol(O.I32, zipf(rng, npr, 320).astype(np.int32), rng.random(npr) > 0.01), O.TCol(O.TS, pts)]
    check_asof(ctx, probe, build, [0], [0], 1, 1, jt, None if jt == O.LEFT else 50000)
    perm = rng.permutation(npr)
    shuffled = [O.TCol(c.type, c.values[perm], None if c.valid is None else c.valid[perm]) for c in probe]
    check_asof(ctx, shuffled, build, [0], [0], 1, 1, jt)


def ticks_nonull(rng, n, nsym, t0=0, span=10 ** 12):
    sym = zipf(rng, n, nsym).astype(np.int32)
    t = np.sort(rng.integers(t0, t0 + span, n)) + rng.integers(-1000, 1000, n)
    return [O.TCol(O.I32, sym), O.TCol(O.TS, t.astype(np.int64)), O.TCol(O.F64, rng.lognormal(4.6, 0.3, n)),
            O.TCol(O.I32, rng.integers(1, 10000, n).astype(np.int32))]


def test_window_packed_key_path(ctx):
    # An I32 partition key and a TS time without NULLs: (sym, bucket index)
    # packed into one key word (single-key kernels, sketch, learned sizing),
    # including the (0, 0) group whose packed word is 0.
    rng = np.random.default_rng(20)
    cols = ticks_nonull(rng, 2 << 20, 400, t0=-5 * 10 ** 9)
    cols[0].values[:1000] = 0
    cols[1].values[:1000] = np.arange(1000)
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 3), (O.MIN, 2), (O.MAX, 2), (O.AVG, 2)]
    check_window(ctx, cols, [0], 1, 60 * 10 ** 9, aggs=aggs)
    check_window(ctx, cols, [0], 1, 10 ** 9, aggs=aggs, chunks=3)
    # 5M rows: the sketch and learned sizing run on the packed words.
    big = ticks_nonull(rng, 5 << 20, 3000, span=10 ** 11)
    check_window(ctx, big, [0], 1, 10 ** 8, aggs=aggs)


@pytest.mark.parametrize("second", ["nulls", "wide_times"])
def test_window_packed_then_unpacked(ctx, second):
    # The first batch packs; the second does not allow it (a NULL partition
    # key, or bucket indexes beyond int32), so the table converts to composite
    # rows mid-aggregation; the result must still be the oracle's.
    rng = np.random.default_rng(21)
    a = ticks_nonull(rng, 300000, 200)
    b = ticks_nonull(rng, 300000, 200)
    width = 10 ** 6
    if second == "nulls":
        b[0].valid = rng.random(300000) > 0.05
    else:
        b[1].values[::7] = np.int64(1) << 60
    cols = [O.TCol(x.type, np.concatenate([x.values, y.values]),
                   None if x.valid is None and y.valid is None else
                   np.concatenate([np.ones(x.n, bool) if x.valid is None else x.valid,
                                   np.ones(y.n, bool) if y.valid is None else y.valid])) for x, y in zip(a, b)]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 3), (O.MIN, 2), (O.MAX, 2)]
    w = qeg.Window(ctx, [c.type for c in cols], [0], 1, width, aggs)
    try:
        for part in (a, b):
            w.consume([to_gpu(c) for c in part])
        w.finish()
        gt, grows = gpu_rows(w.fetch(), w.result_types)
    finally:
        w.close()
    ot, orows = O.window_tumbling(cols, [0], 1, width, aggs)
    assert_same(gt, grows, ot, orows, second)


def test_window_unpackable_from_the_start(ctx):
    # Bucket indexes beyond int32 (width 1 on 2^40-scale times): composite keys.
    rng = np.random.default_rng(22)
    cols = ticks_nonull(rng, 200000, 100, t0=1 << 40, span=1 << 20)
    check_window(ctx, cols, [0], 1, 1, aggs=[(O.COUNT_STAR, 0), (O.SUM, 3)])


@pytest.mark.parametrize("shift", [0, 40])
def test_window_packed_i64_partition_keys(ctx, shift):
    # I64 partition keys: packed when their values fit in int32 (shift 0,
    # including negative keys), composite keys otherwise (shift 40).
    rng = np.random.default_rng(23 + shift)
    cols = ticks_nonull(rng, 500000, 300)
    cols[0] = O.TCol(O.I64, (cols[0].values.astype(np.int64) - 150) << shift)
    check_window(ctx, cols, [0], 1, 10 ** 9, aggs=[(O.COUNT_STAR, 0), (O.SUM, 3), (O.MIN, 2), (O.MAX, 2)])


@pytest.mark.parametrize("dev_inputs", [False, True])
def test_asof_left_device_fetch_matches_host_fetch(ctx, dev_inputs):
    # A LEFT as-of emits probe row k as output row k: from a word-aligned start
    # the probe columns are plain copies on a side stream (values, validity
    # words with the tail padded, the NULL flag), from any other start they are
    # gathered; STR probe codes under a dictionary are always gathered.
    import torch

    rng = np.random.default_rng(22)
    nb, npr = 50000, 200003
    build = ticks(rng, nb, 100)
    probe = ticks(rng, npr, 120)
    probe.append(O.TCol(O.I64, rng.integers(0, 99, npr)))  # no NULLs
    names = ["S%03d" % i for i in range(40)]
    probe.append(O.TCol(O.STR, rng.integers(0, 40, npr).astype(np.int32), rng.random(npr) > 0.1,
                        list(rng.permutation(names))))
    canon = StrCanon(names)
    j = qeg.AsofJoin(ctx, [c.type for c in probe], [c.type for c in build], [0], [0], 1, 1, O.LEFT, None)
    try:
        j.build([to_gpu(c) for c in build])
        j.build_finish()
        pcols = [to_gpu(c, canon, device=dev_inputs) for c in probe]  # read again by the fetches
        n = j.probe(pcols)
        assert n == npr
        for first, count, words in ((0, n, True), (64, n - 64 - 5, True), (37, n - 100, True), (n - 1, 1, True),
                                    (128, 1000, False)):
            host = j.fetch(first, count)
            flags = []
            dev = j.fetch_device(first, count, flags=flags)
            if not words:
                dev = j.fetch_device(first, count, bufs=[(v, None) for v, _ in dev], flags=flags)
            torch.cuda.synchronize()
            for c, ((hv, hvalid), (dv, dw), f) in enumerate(zip(host, dev, flags)):
                assert f == bool(np.all(hvalid)), (first, c)
                if words:
                    w = dw.cpu().numpy().view(np.uint64)
                    bits = np.unpackbits(w.view(np.uint8), bitorder="little")
                    assert np.all(bits[count:]), (first, c)  # tail padding is valid
                    assert np.array_equal(bits[:count].astype(bool), hvalid), (first, c)
                dvals = dv[:count].cpu().numpy()
                assert np.array_equal(dvals[hvalid].view(np.uint8), np.asarray(hv)[hvalid].view(np.uint8)), (first, c)
    finally:
        j.close()
