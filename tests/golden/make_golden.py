"""Generates the golden vectors under tests/golden/ from the REFERENCE engine
itself (explorer-skp/query-engine compiled from its own sources into
oracle/_ref/libqe_ref.so by `make -C oracle ref`).

Cases:
  * the hand-built edge tables of the reference's tests/aggregate_differential_test.cpp,
    tests/join_differential_test.cpp, tests/oracle_zero_row_test.cpp, the
    F64-key case of tests/hashtable_test.cpp, and the tumbling-window and as-of
    edge tables of tests/window_differential_test.cpp and
    tests/asof_differential_test.cpp, restated as inputs;
  * seeded random GROUP BY and join cases in the shape of the reference's
    generators (bounded magnitudes, ~15% NULLs);
  * the splitmix64 row-hash fold at boundary inputs (ops/hash_scalar.cpp).
Each expected result is the reference's operator tree output (Plan::lower +
drain); the reference's independent oracle must agree or generation stops.

Run in a checkout that has the reference tree:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, os.path.join(REPO, "query-engine_gb300"))

import oracle as O  # noqa: E402
from util import gen_column, gen_group_by, gen_schema, gen_table  # noqa: E402

NAN = float("nan")


def enc_value(t, v):
    if v is None:
        return None
    if t == O.F64:
        return float(v).hex()
    return v


def enc_col(c):
    vals = c.values.tolist()
    if c.type == O.F64:
        vals = [float(x).hex() for x in vals]
    return {"type": c.type, "values": vals, "valid": None if c.valid is None else c.valid.astype(int).tolist(),
            "dictionary": c.dictionary}


def enc_rows(types, rows):
    return [[enc_value(t, v) for t, v in zip(types, r)] for r in rows]


def col(t, values, nulls=(), dictionary=None):
    dt = {O.I32: np.int32, O.I64: np.int64, O.F64: np.float64, O.BOOL: np.uint8, O.TS: np.int64, O.STR: np.int32}[t]
    valid = None
    if nulls:
        valid = np.ones(len(values), bool)
        valid[list(nulls)] = False
    return O.TCol(t, np.array(values, dtype=dt), valid, dictionary)


def groupby_case(name, cols, keys, aggs):
    ref_t, ref_rows = O.ref_groupby(cols, keys, aggs, 2048, mode=0)
    ind_t, ind_rows = O.ref_groupby(cols, keys, aggs, 2048, mode=1)
    m = O.compare(ref_t, ref_rows, ind_t, ind_rows)
    assert m is None, (name, m)
    for bs in (64, 256):
        bt, brows = O.ref_groupby(cols, keys, aggs, bs, mode=0)
        assert O.compare(ref_t, ref_rows, bt, brows) is None, (name, bs)
    return {"kind": "groupby", "name": name, "columns": [enc_col(c) for c in cols], "keys": keys,
            "aggs": [list(a) for a in aggs], "types": ref_t, "rows": enc_rows(ref_t, ref_rows)}


def join_case(name, probe, build, pk, bk, jt):
    ref_t, ref_rows = O.ref_join(probe, build, pk, bk, jt, 2048, mode=0)
    ind_t, ind_rows = O.ref_join(probe, build, pk, bk, jt, 2048, mode=1)
    m = O.compare(ref_t, ref_rows, ind_t, ind_rows)
    assert m is None, (name, m)
    return {"kind": "join", "name": name, "probe": [enc_col(c) for c in probe], "build": [enc_col(c) for c in build],
            "probe_keys": pk, "build_keys": bk, "join_type": jt, "types": ref_t, "rows": enc_rows(ref_t, ref_rows)}


def window_case(name, cols, keys, time_col, width, aggs):
    ref_t, ref_rows = O.ref_window_tumbling(cols, keys, time_col, width, aggs, 2048, mode=0)
    ind_t, ind_rows = O.ref_window_tumbling(cols, keys, time_col, width, aggs, 2048, mode=1)
    m = O.compare(ref_t, ref_rows, ind_t, ind_rows)
    assert m is None, (name, m)
    for bs in (64, 256):
        bt, brows = O.ref_window_tumbling(cols, keys, time_col, width, aggs, bs, mode=0)
        assert O.compare(ref_t, ref_rows, bt, brows) is None, (name, bs)
    return {"kind": "window", "name": name, "columns": [enc_col(c) for c in cols], "keys": keys,
            "time_col": time_col, "width": width, "aggs": [list(a) for a in aggs], "types": ref_t,
            "rows": enc_rows(ref_t, ref_rows)}


def asof_case(name, probe, build, pk, bk, pt, bt, jt, tol, unique_build=True):
    """Expected rows: the reference's AsofJoin operator. Its independent oracle
    must agree where build (key, time) pairs are unique (the reference leaves
    the pick among equal build times to its stable sort)."""
    ref_t, ref_rows = O.ref_asof_join(probe, build, pk, bk, pt, bt, jt, tol, 2048, mode=0)
    if unique_build:
        ind_t, ind_rows = O.ref_asof_join(probe, build, pk, bk, pt, bt, jt, tol, 2048, mode=1)
        m = O.compare(ref_t, ref_rows, ind_t, ind_rows)
        assert m is None, (name, m)
    for bs in (64, 256):
        b_t, brows = O.ref_asof_join(probe, build, pk, bk, pt, bt, jt, tol, bs, mode=0)
        assert O.compare(ref_t, ref_rows, b_t, brows) is None, (name, bs)
    return {"kind": "asof", "name": name, "probe": [enc_col(c) for c in probe], "build": [enc_col(c) for c in build],
            "probe_keys": pk, "build_keys": bk, "probe_time": pt, "build_time": bt, "join_type": jt,
            "tolerance": tol, "types": ref_t, "rows": enc_rows(ref_t, ref_rows)}


def tsx_cases(rng):
    """Tumbling-window and as-of cases: the reference tests' edge tables, then
    seeded tick-like random cases."""
    cases = []
    win = [col(O.I32, [1, 1, 1, 2, 2, 1]), col(O.TS, [0, 5, 12, 3, 21, 30]),
           col(O.I64, [10, 20, 30, 40, 50, 60], nulls=[2]), col(O.F64, [1.5, 2.5, 3.5, 4.5, 5.5, 6.5])]
    all_aggs = [(O.COUNT_STAR, 0), (O.COUNT, 2), (O.SUM, 2), (O.MIN, 2), (O.MAX, 2), (O.AVG, 3)]
    cases.append(window_case("window_edge_single_key_w10", win, [0], 1, 10, all_aggs))
    cases.append(window_case("window_edge_zero_keys_w8", win, [], 1, 8, all_aggs))
    cases.append(window_case("window_edge_width_1", win, [0], 1, 1, all_aggs))
    nullk = [col(O.I32, [1, 1, 7, 7], nulls=[2, 3]), col(O.TS, [0, 10, 5, 20]), col(O.I64, [100, 200, 300, 400])]
    cases.append(window_case("window_edge_null_keys_group_together", nullk, [0], 1, 10,
                             [(O.COUNT_STAR, 0), (O.SUM, 2)]))
    cases.append(window_case("window_edge_empty", [col(O.I32, []), col(O.TS, [])], [0], 1, 10, [(O.COUNT_STAR, 0)]))
    i32ts = [col(O.I32, [1, 1, 1, 2]), col(O.I32, [7, 7, 9, 7]), col(O.I32, [0, 11, 4, 25]),
             col(O.I64, [100, 200, 300, 400])]
    cases.append(window_case("window_edge_i32_time_composite", i32ts, [0, 1], 2, 10,
                             [(O.COUNT_STAR, 0), (O.SUM, 3), (O.MIN, 2)]))
    nan_w = [col(O.I32, [1, 1, 1, 1, 2, 2, 2, 2]), col(O.TS, [0, 5, 12, 17, 1, 6, 11, 21]),
             col(O.F64, [3.0, NAN, NAN, NAN, NAN, 2.0, 0.0, 4.0], nulls=[6])]
    cases.append(window_case("window_edge_nan_minmax", nan_w, [0], 1, 10, [(O.MIN, 2), (O.MAX, 2), (O.COUNT, 2)]))
    # Negative times: C++ truncating division, (-15 / 10) * 10 = -10.
    cases.append(window_case("window_edge_negative_time", [col(O.I32, [1, 1, 1, 1, 1]),
                                                           col(O.I64, [-15, -5, -1, 0, 4]), col(O.I64, [1, 2, 3, 4, 5])],
                             [0], 1, 10, [(O.COUNT_STAR, 0), (O.SUM, 2)]))
    cases.append(window_case("window_edge_null_time", [col(O.I32, [1, 1, 2]), col(O.TS, [3, 0, 14], nulls=[1]),
                                                       col(O.I64, [1, 2, 3])], [0], 1, 10,
                             [(O.COUNT_STAR, 0), (O.SUM, 2)]))
    for it in range(12):
        n = int(rng.integers(0, 400))
        tt = [O.TS, O.I64, O.I32][it % 3]
        cols = [gen_column(rng, O.I32, n, 10, int(rng.integers(1, 8))),
                col(tt, rng.integers(0, 1000, n).tolist(), nulls=np.flatnonzero(rng.random(n) < 0.05).tolist()),
                gen_column(rng, O.I64, n, 10), gen_column(rng, O.F64, n, 10)]
        keys = [0] if it % 2 == 0 else []
        aggs = [(O.COUNT_STAR, 0), (O.SUM, 2), (O.MIN, 2), (O.MAX, 3), (O.AVG, 3), (O.COUNT, 3)]
        cases.append(window_case("window_random_%02d" % it, cols, keys, 1, int(rng.choice([1, 7, 50, 250, 5000])),
                                 aggs))
    # --- as-of edge tables (tests/asof_differential_test.cpp) ------------------
    build = [col(O.I32, [1, 1, 1, 2]), col(O.TS, [10, 20, 30, 15]), col(O.I64, [100, 200, 300, 150])]
    probe = [col(O.I32, [1, 1, 1, 2, 3, 1]), col(O.TS, [5, 10, 25, 15, 99, 50])]
    for jt in (O.INNER, O.LEFT):
        sfx = "_left" if jt else "_inner"
        cases.append(asof_case("asof_edge_single_key" + sfx, probe, build, [0], [0], 1, 1, jt, None))
        cases.append(asof_case("asof_edge_tolerance_10" + sfx, probe, build, [0], [0], 1, 1, jt, 10))
        cases.append(asof_case("asof_edge_zero_keys" + sfx, [col(O.TS, [5, 25, 35])],
                               [col(O.TS, [10, 20, 30]), col(O.I64, [100, 200, 300])], [], [], 0, 0, jt, None))
        cases.append(asof_case("asof_edge_empty_build" + sfx, probe, [col(O.I32, []), col(O.TS, [])], [0], [0], 1, 1,
                               jt, None))
        cases.append(asof_case("asof_edge_nulls_never_match" + sfx,
                               [col(O.I32, [1, 2, 2, 9], nulls=[3]), col(O.TS, [25, 30, 0, 50], nulls=[2])],
                               [col(O.I32, [1, 1, 2, 7], nulls=[3]), col(O.TS, [10, 20, 0, 5], nulls=[2]),
                                col(O.I64, [100, 200, 999, 777])], [0], [0], 1, 1, jt, None))
    cases.append(asof_case("asof_edge_empty_probe", [col(O.I32, []), col(O.TS, [])], build, [0], [0], 1, 1, O.INNER,
                           None))
    cases.append(asof_case("asof_edge_composite_key", [col(O.I32, [1, 1]), col(O.I32, [7, 9]), col(O.TS, [25, 25])],
                           [col(O.I32, [1, 1, 1]), col(O.I32, [7, 7, 9]), col(O.TS, [10, 20, 10])], [0, 1], [0, 1],
                           2, 2, O.INNER, None))
    # Equal build times within a key: the build row drained last wins.
    cases.append(asof_case("asof_edge_equal_build_times",
                           [col(O.I32, [1, 1, 2]), col(O.TS, [20, 9, 40])],
                           [col(O.I32, [1, 1, 1, 2, 2]), col(O.TS, [10, 20, 10, 40, 40]),
                            col(O.I64, [1, 2, 3, 4, 5])], [0], [0], 1, 1, O.LEFT, None, unique_build=False))
    # I32 time on the probe side against TS on the build side.
    cases.append(asof_case("asof_edge_i32_probe_time", [col(O.I32, [1, 1, 2]), col(O.I32, [15, 35, 20])], build,
                           [0], [0], 1, 1, O.LEFT, None))
    for it in range(16):
        nsym = int(rng.integers(1, 12))
        nb, npr = int(rng.integers(0, 300)), int(rng.integers(0, 300))
        # unique (key, time) on the build side, times >= 0
        pairs = rng.permutation(nsym * 2000)[:nb]
        bsym, bts = (pairs % nsym).tolist(), (pairs // nsym).tolist()
        build = [col(O.I32, bsym, nulls=np.flatnonzero(rng.random(nb) < 0.05).tolist()),
                 col(O.TS, bts, nulls=np.flatnonzero(rng.random(nb) < 0.05).tolist()),
                 gen_column(rng, O.F64, nb, 10)]
        probe = [col(O.I32, rng.integers(0, nsym + 2, npr).tolist(),
                     nulls=np.flatnonzero(rng.random(npr) < 0.05).tolist()),
                 col(O.TS, rng.integers(0, 2100, npr).tolist(), nulls=np.flatnonzero(rng.random(npr) < 0.05).tolist()),
                 gen_column(rng, O.I64, npr, 10)]
        tol = None if it % 3 else int(rng.integers(0, 300))
        keys = [0] if it % 4 != 3 else []
        cases.append(asof_case("asof_random_%02d" % it, probe, build, keys, keys, 1, 1, int(rng.integers(0, 2)), tol,
                               unique_build=bool(keys)))
    return cases


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/libqe_ref.so is missing: run `make -C oracle ref` where the reference tree exists")
    cases = []
    # --- tests/aggregate_differential_test.cpp edge tables -------------------
    edge = [col(O.I32, [1, 1, 2, 2, 3, 1, 2, 3, 0, 0], nulls=[8, 9]),
            col(O.I32, [10, 20, 30, 40, 50, 60, 70, 80, 90, 100], nulls=[0]),
            col(O.F64, [1.5, 2.5, 3.5, 4.5, 5.5, 6.5, 7.5, 8.5, 9.5, 10.5], nulls=[2])]
    full = [(O.COUNT_STAR, 0), (O.COUNT, 1), (O.SUM, 1), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1), (O.SUM, 2), (O.AVG, 2)]
    cases.append(groupby_case("agg_edge_single_key_null_group", edge, [0], full))
    cases.append(groupby_case("agg_edge_composite_i32_f64", edge, [0, 2], [(O.COUNT_STAR, 0), (O.SUM, 1)]))
    cases.append(groupby_case("agg_edge_global", edge, [], full))
    cases.append(groupby_case("agg_edge_all_null_group",
                              [col(O.I32, [1, 1, 2, 2]), col(O.I32, [0, 0, 5, 6], nulls=[0, 1])], [0],
                              [(O.COUNT_STAR, 0), (O.COUNT, 1), (O.SUM, 1), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1)]))
    i = np.arange(6000)
    skew = [col(O.I32, (i % 5).tolist()), col(O.I64, ((i % 100) - 50).tolist())]
    cases.append(groupby_case("agg_edge_tail_over_2048_groups", skew, [1], [(O.COUNT_STAR, 0), (O.SUM, 0)]))
    empty = [col(O.I64, []), col(O.F64, [])]
    cases.append(groupby_case("agg_zero_row_global", empty, [],
                              [(O.COUNT_STAR, 0), (O.COUNT, 0), (O.SUM, 0), (O.MIN, 1), (O.MAX, 1), (O.AVG, 1)]))
    cases.append(groupby_case("agg_zero_row_keyed", empty, [0], [(O.COUNT_STAR, 0), (O.SUM, 0)]))
    nan_t = [col(O.I32, [1, 1, 2, 2, 3, 3, 4, 4]), col(O.F64, [NAN, 1.5, NAN, NAN, 2.5, 3.5, NAN, 0.0], nulls=[7])]
    nan_aggs = [(O.MIN, 1), (O.MAX, 1), (O.SUM, 1), (O.AVG, 1), (O.COUNT, 1)]
    cases.append(groupby_case("agg_edge_nan_minmax_grouped", nan_t, [0], nan_aggs))
    cases.append(groupby_case("agg_edge_nan_minmax_global", nan_t, [], nan_aggs))
    neg_nan = np.frombuffer(np.array([0xFFF8000000000000], np.uint64).tobytes(), np.float64)[0]
    cases.append(groupby_case("hashtable_f64_key_canonicalisation",
                              [col(O.F64, [0.0, -0.0, NAN, neg_nan, 1.5])], [0], [(O.COUNT_STAR, 0)]))
    # --- tests/join_differential_test.cpp edge cases --------------------------
    jcases = [
        ("join_edge_single_key", [col(O.I32, [1, 2, 3, 5, 0], nulls=[4]), col(O.I64, [100, 200, 300, 500, 999])],
         [col(O.I32, [1, 1, 2, 5, 5, 5]), col(O.I64, [10, 11, 20, 50, 51, 52])], [0], [0]),
        ("join_edge_composite", [col(O.I32, [1, 1, 2, 2]), col(O.F64, [2.0, 9.0, 1.0, 2.0])],
         [col(O.I32, [1, 1, 2, 2]), col(O.F64, [1.0, 2.0, 1.0, 2.0]), col(O.I64, [11, 12, 21, 22])], [0, 1], [0, 1]),
        ("join_edge_empty_build", [col(O.I32, [1, 2, 3])], [col(O.I32, []), col(O.I64, [])], [0], [0]),
        ("join_edge_empty_probe", [col(O.I32, []), col(O.I64, [])], [col(O.I32, [1, 2, 3])], [0], [0]),
        ("join_edge_all_match", [col(O.I32, [7, 7, 7])], [col(O.I32, [7, 7, 7, 7]), col(O.I64, [1, 2, 3, 4])], [0], [0]),
        ("join_edge_fanout_3000", [col(O.I32, [7, 9, 7]), col(O.I64, [100, 200, 300])],
         [col(O.I32, [7] * 3000), col(O.I64, list(range(3000)))], [0], [0]),
        ("join_edge_null_never_matches", [col(O.I32, [1, 0, 0], nulls=[1, 2])],
         [col(O.I32, [1, 0, 2], nulls=[1]), col(O.I64, [10, 11, 12])], [0], [0]),
        ("join_zero_row_no_match", [col(O.I32, [100, 200])], [col(O.I32, [1, 2]), col(O.I64, [5, 6])], [0], [0]),
        ("join_str_cross_dictionary",
         [col(O.STR, [0, 1, 2, 2], nulls=[3], dictionary=["MSFT", "GOOG", "AAPL"])],
         [col(O.STR, [0, 1, 2, 1], dictionary=["IBM", "AAPL", "MSFT"]), col(O.I64, [1, 2, 3, 4])], [0], [0]),
    ]
    for name, probe, build, pk, bk in jcases:
        for jt in (O.INNER, O.LEFT):
            cases.append(join_case(name + ("_left" if jt else "_inner"), probe, build, pk, bk, jt))
    # --- seeded random cases --------------------------------------------------
    rng = np.random.default_rng(20260615)
    for it in range(30):
        types = gen_schema(rng)
        cols = gen_table(rng, types, int(rng.integers(0, 150)))
        keys, aggs = gen_group_by(rng, types)
        cases.append(groupby_case("agg_random_%02d" % it, cols, keys, aggs))
    for it in range(30):
        nk = int(rng.integers(1, 3))
        kt = [int(rng.choice([O.I32, O.I64, O.F64])) for _ in range(nk)]
        card = int(rng.integers(1, 20))
        nb, npr = int(rng.integers(0, 80)), int(rng.integers(0, 80))
        build = [gen_column(rng, t, nb, 10, card) for t in kt] + [gen_column(rng, O.I64, nb, 10)]
        probe = [gen_column(rng, t, npr, 10, card * 2) for t in kt] + [gen_column(rng, O.F64, npr, 10)]
        cases.append(join_case("join_random_%02d" % it, probe, build, list(range(nk)), list(range(nk)),
                               int(rng.integers(0, 2))))
    cases += tsx_cases(np.random.default_rng(20260616))
    # --- hash fold pins (ops/hash_scalar.cpp) ----------------------------------
    R = O.ref()
    seeds = [0, 1, 0x51E57A11AB1E5EED, 2**64 - 1]
    words = [0, 1, 2**63, 2**64 - 1, 0x9E3779B97F4A7C15, 0x7ff8000000000000, 123456789]
    pins = [[a, w, int(R.ref_hash_combine(a, w))] for a in seeds for w in words]

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases, "hash_pins": pins}, f,
                  separators=(",", ":"))
    print("wrote %d cases, %d hash pins" % (len(cases), len(pins)))


if __name__ == "__main__":
    main()
