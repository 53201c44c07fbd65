"""Pins the CPU oracle to the reference engine: every golden case produced by
the reference (tests/golden/golden.json) must come out of the oracle with the
same rows in the same order (first-seen group order for GROUP BY, probe order
for joins), F64 cells within the reference's epsilon; the hash fold must match
bit for bit. Where the reference library is built (oracle/_ref), seeded random
cases are also cross-checked live."""
import math

import numpy as np
import pytest

import oracle as O
from golden_io import dec_col, dec_rows, load
from util import gen_column, gen_group_by, gen_schema, gen_table

G = load()


def same_ordered(types, a, b):
    assert len(a) == len(b)
    for ra, rb in zip(a, b):
        for t, x, y in zip(types, ra, rb):
            if x is None or y is None:
                assert x is None and y is None
            elif t == O.F64:
                assert O.float_eq(x, y), (x, y)
            else:
                assert x == y


@pytest.mark.parametrize("case", G["cases"], ids=[c["name"] for c in G["cases"]])
def test_oracle_matches_reference_golden(case):
    types = case["types"]
    exp = dec_rows(types, case["rows"])
    if case["kind"] == "groupby":
        cols = [dec_col(c) for c in case["columns"]]
        t, rows = O.groupby(cols, case["keys"], [tuple(a) for a in case["aggs"]])
    elif case["kind"] == "window":
        cols = [dec_col(c) for c in case["columns"]]
        t, rows = O.window_tumbling(cols, case["keys"], case["time_col"], case["width"],
                                    [tuple(a) for a in case["aggs"]])
    elif case["kind"] == "asof":
        probe = [dec_col(c) for c in case["probe"]]
        build = [dec_col(c) for c in case["build"]]
        t, rows = O.asof_join(probe, build, case["probe_keys"], case["build_keys"], case["probe_time"],
                              case["build_time"], case["join_type"], case["tolerance"])
        # The reference emits as-of rows in its sorted probe order, the
        # restatement in probe order: compare as multisets.
        assert t == types
        assert O.compare(t, rows, types, exp) is None
        return
    else:
        probe = [dec_col(c) for c in case["probe"]]
        build = [dec_col(c) for c in case["build"]]
        t, rows = O.join(probe, build, case["probe_keys"], case["build_keys"], case["join_type"])
    assert t == types
    same_ordered(types, rows, exp)


def test_hash_fold_pins():
    L = O.orc()
    for acc, w, h in G["hash_pins"]:
        assert L.orc_hash_combine(acc, w) == h


def test_known_answers_from_reference_tests():
    """Expected values written out in the reference's own tests."""
    by = {c["name"]: c for c in G["cases"]}
    rows = dec_rows(by["agg_edge_all_null_group"]["types"], by["agg_edge_all_null_group"]["rows"])
    d = {r[0]: r[1:] for r in rows}
    assert d[1] == (2, 0, None, None, None, None) and d[2] == (2, 2, 11, 5, 6, 5.5)
    rows = dec_rows(by["agg_edge_nan_minmax_grouped"]["types"], by["agg_edge_nan_minmax_grouped"]["rows"])
    d = {r[0]: r[1:] for r in rows}
    assert d[1][0] == 1.5 and math.isnan(d[1][1])
    assert math.isnan(d[2][0]) and math.isnan(d[2][1])
    assert d[3][:2] == (2.5, 3.5)
    assert len(by["hashtable_f64_key_canonicalisation"]["rows"]) == 3
    assert by["agg_zero_row_global"]["rows"] == [[0, 0, None, None, None, None]]
    assert by["agg_zero_row_keyed"]["rows"] == []
    # Tumbling window edge table: key 1 rows at t 0, 5 -> bucket 0; t 12 -> 10;
    # t 30 -> 30; key 2 at t 3 -> 0 and t 21 -> 20.
    rows = dec_rows(by["window_edge_single_key_w10"]["types"], by["window_edge_single_key_w10"]["rows"])
    assert sorted((r[0], r[1], r[2]) for r in rows) == [(1, 0, 2), (1, 10, 1), (1, 30, 1), (2, 0, 1), (2, 20, 1)]
    rows = dec_rows(by["window_edge_negative_time"]["types"], by["window_edge_negative_time"]["rows"])
    assert sorted(r[1] for r in rows) == [-10, 0]
    # As-of edge table: probe (1,5) has no preceding build row; (1,10) takes the
    # equal-time row (boundary >=); (1,25) -> t20; (2,15) -> t15; key 3 has no
    # partition; (1,50) -> t30.
    rows = dec_rows(by["asof_edge_single_key_left"]["types"], by["asof_edge_single_key_left"]["rows"])
    got = sorted((r[0], r[1], r[4]) for r in rows)
    assert got == [(1, 5, None), (1, 10, 100), (1, 25, 200), (1, 50, 300), (2, 15, 150), (3, 99, None)]
    rows = dec_rows(by["asof_edge_equal_build_times"]["types"], by["asof_edge_equal_build_times"]["rows"])
    assert sorted((r[0], r[1], r[4]) for r in rows) == [(1, 9, None), (1, 20, 2), (2, 40, 5)]


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built in this checkout")
def test_oracle_vs_live_reference_random():
    rng = np.random.default_rng(123)
    for _ in range(60):
        types = gen_schema(rng)
        cols = gen_table(rng, types, int(rng.integers(0, 3000)))
        keys, aggs = gen_group_by(rng, types)
        bs = int(rng.choice([64, 256, 2048]))
        t1, r1 = O.groupby(cols, keys, aggs, bs)
        t2, r2 = O.ref_groupby(cols, keys, aggs, bs)
        assert t1 == t2
        same_ordered(t1, r1, r2)
    for _ in range(40):
        nk = int(rng.integers(1, 3))
        kt = [int(rng.choice([O.I32, O.I64, O.F64])) for _ in range(nk)]
        card = int(rng.integers(1, 50))
        nb, npr = int(rng.integers(0, 500)), int(rng.integers(0, 500))
        build = [gen_column(rng, t, nb, 10, card) for t in kt] + [gen_column(rng, O.I64, nb, 10)]
        probe = [gen_column(rng, t, npr, 10, card * 2) for t in kt] + [gen_column(rng, O.F64, npr, 10)]
        jt = int(rng.integers(0, 2))
        t1, r1 = O.join(probe, build, list(range(nk)), list(range(nk)), jt)
        t2, r2 = O.ref_join(probe, build, list(range(nk)), list(range(nk)), jt)
        assert t1 == t2
        same_ordered(t1, r1, r2)


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built in this checkout")
def test_tsx_oracle_vs_live_reference_random():
    """Tumbling window and as-of join restatements against the reference's
    operators on seeded tick-like tables (duplicate build times included)."""
    rng = np.random.default_rng(321)
    for it in range(20):
        n = int(rng.integers(0, 4000))
        tt = [O.TS, O.I64, O.I32][it % 3]
        cols = [gen_column(rng, O.I32, n, 5, int(rng.integers(1, 30))),
                O.TCol(tt, rng.integers(-500, 100000, n).astype(np.int32 if tt == O.I32 else np.int64),
                       rng.random(n) > 0.03),
                gen_column(rng, O.I64, n, 10), gen_column(rng, O.F64, n, 10)]
        keys = [[0], [], [0, 2]][it % 3]
        aggs = [(O.COUNT_STAR, 0), (O.SUM, 2), (O.MIN, 3), (O.MAX, 2), (O.AVG, 3), (O.COUNT, 3)]
        w = int(rng.choice([1, 10, 1000, 77777]))
        t1, r1 = O.window_tumbling(cols, keys, 1, w, aggs)
        t2, r2 = O.ref_window_tumbling(cols, keys, 1, w, aggs, int(rng.choice([64, 2048])))
        assert t1 == t2
        same_ordered(t1, r1, r2)
    for it in range(20):
        nsym = int(rng.integers(1, 40))
        nb, npr = int(rng.integers(0, 3000)), int(rng.integers(0, 3000))
        build = [gen_column(rng, O.I32, nb, 5, nsym),
                 O.TCol(O.TS, rng.integers(0, 50000, nb).astype(np.int64), rng.random(nb) > 0.03),
                 gen_column(rng, O.F64, nb, 10)]
        probe = [gen_column(rng, O.I32, npr, 5, nsym + 3),
                 O.TCol(O.I64, rng.integers(-100, 52000, npr).astype(np.int64), rng.random(npr) > 0.03),
                 gen_column(rng, O.I64, npr, 10)]
        keys = [0] if it % 4 else []
        tol = None if it % 2 else int(rng.integers(0, 2000))
        jt = int(rng.integers(0, 2))
        t1, r1 = O.asof_join(probe, build, keys, keys, 1, 1, jt, tol)
        t2, r2 = O.ref_asof_join(probe, build, keys, keys, 1, 1, jt, tol, int(rng.choice([64, 2048])))
        assert t1 == t2
        assert O.compare(t1, r1, t2, r2) is None


def test_parallel_port_matches_single_thread():
    """The CPU baseline (port of the morsel-parallel engine) gives the same
    result as the single-threaded operator, with >= 2 workers forced."""
    rng = np.random.default_rng(9)
    n = 20000
    cols = [gen_column(rng, O.I64, n, 5, 700), gen_column(rng, O.F64, n, 5), gen_column(rng, O.I32, n, 5)]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1), (O.AVG, 2), (O.MIN, 2), (O.MAX, 1), (O.COUNT, 1)]
    t1, r1 = O.groupby(cols, [0], aggs)
    t2, r2 = O.parallel_groupby(cols, [0], aggs, threads=4, morsel_rows=1024)
    assert O.compare(t1, r1, t2, r2) is None
    pk = O.TCol(O.I64, rng.integers(0, 3000, n).astype(np.int64), rng.random(n) > 0.02)
    pv = O.TCol(O.I64, rng.integers(0, 1 << 20, n).astype(np.int64))
    bk = O.TCol(O.I64, rng.permutation(2000).astype(np.int64) // 2)
    bv = O.TCol(O.I64, np.zeros(2000, np.int64))
    assert O.join_count_sum(pk, pv, bk) == O.parallel_join_count_sum(pk, pv, bk, bv, threads=3, morsel_rows=4096)
