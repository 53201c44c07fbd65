"""The fused filter -> inner join -> GROUP BY (qeg_filter_join_agg) against the
oracle's operators applied one after another, on data in the shape of the
dictionary-string pipeline workload: trades (sym STR codes, Zipf-skewed; price
F64 lognormal; qty I32) filtered on price > 100, joined by VALUE with a symbol
table under a different dictionary (sym STR, sector I32 over 32 values), grouped
by sector with COUNT(*), AVG(price), SUM(qty) (+ MIN/MAX/COUNT variants)."""
import numpy as np
import pytest

import oracle as O
import qeg
from util import StrCanon, assert_same, gpu_rows, to_gpu

pytestmark = pytest.mark.gpu


def make_case(seed, n=300_000, nsym=1000, nulls=True, dup_syms=False):
    rng = np.random.default_rng(seed)
    syms = ["S%04d" % i for i in range(nsym)]
    tdict = list(rng.permutation(syms))                   # trades dictionary order
    bdict = list(rng.permutation(syms + ["ZZZ%d" % i for i in range(20)]))  # symbols dictionary
    ranks = np.minimum(rng.zipf(1.3, n) - 1, nsym - 1)
    codes = np.array([tdict.index(syms[r]) for r in range(nsym)], np.int32)[ranks]
    price = np.exp(rng.normal(4.6, 0.3, n))
    qty = rng.integers(1, 10001, n).astype(np.int32)
    pv = (rng.random(n) > 0.01) if nulls else None
    kv = (rng.random(n) > 0.01) if nulls else None
    trades = [O.TCol(O.STR, codes, kv, tdict), O.TCol(O.F64, price, pv), O.TCol(O.I32, qty)]
    brow = np.arange(len(bdict), dtype=np.int32)
    if dup_syms:
        brow = np.concatenate([brow, brow[:50]])
    sector = rng.integers(0, 32, len(brow)).astype(np.int32)
    svalid = (rng.random(len(brow)) > 0.05) if nulls else None
    symbols = [O.TCol(O.STR, brow, None, bdict), O.TCol(O.I32, sector, svalid)]
    return trades, symbols


def oracle_pipeline(trades, symbols, aggs):
    ok = trades[1].values > 100
    if trades[1].valid is not None:
        ok &= trades[1].valid
    filt = [O.TCol(c.type, c.values[ok], None if c.valid is None else c.valid[ok], c.dictionary) for c in trades]
    jt, jrows = O.join(filt, symbols, [0], [0], O.INNER)
    # Joined schema: sym, price, qty, sym, sector -> group by sector (col 4).
    cols = []
    for i, t in enumerate(jt):
        vals = [r[i] for r in jrows]
        valid = np.array([v is not None for v in vals], bool)
        if t == O.STR:
            d = sorted({v for v in vals if v is not None}) or ["?"]
            arr = np.array([d.index(v) if v is not None else 0 for v in vals], np.int32)
            cols.append(O.TCol(t, arr, valid, d))
        else:
            dt = {O.I32: np.int32, O.I64: np.int64, O.F64: np.float64}[t]
            arr = np.array([v if v is not None else 0 for v in vals], dt)
            cols.append(O.TCol(t, arr, valid))
    return O.groupby(cols, [4], aggs)


# The kernels of the fused pipeline: thread-private states (the default), and
# the shared-state kernel with per-lane reductions or warp peer aggregation.
KERNELS = {"private": {}, "shared_lanes": {"QEG_PIPE_KERNEL": "shared", "QEG_PIPE_LANES": "1"},
           "shared_peers": {"QEG_PIPE_KERNEL": "shared", "QEG_PIPE_LANES": "0"}}


def use_kernel(monkeypatch, kernel):
    monkeypatch.delenv("QEG_PIPE_KERNEL", raising=False)
    monkeypatch.delenv("QEG_PIPE_LANES", raising=False)
    for k, v in KERNELS[kernel].items():
        monkeypatch.setenv(k, v)


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("seed,nulls,dup", [(1, True, False), (2, False, False), (3, True, True)])
def test_pipeline_matches_operator_chain(ctx, seed, nulls, dup, kernel, monkeypatch):
    use_kernel(monkeypatch, kernel)
    trades, symbols = make_case(seed, nulls=nulls, dup_syms=dup)
    aggs = [(O.COUNT_STAR, 0), (O.AVG, 1), (O.SUM, 2), (O.MIN, 1), (O.MAX, 2), (O.COUNT, 1)]
    ot, orows = oracle_pipeline(trades, symbols, aggs)
    canon = StrCanon(trades[0].dictionary + symbols[0].dictionary)
    gp = [to_gpu(c, canon) for c in trades]
    gb = [to_gpu(c, canon) for c in symbols]
    types, res = qeg.filter_join_agg(ctx, gp, gb, 0, 0, 4, aggs, filter_col=1, filter_op=qeg.CMP_GT,
                                     filter_value=100.0)
    gt, grows = gpu_rows(res, types, canon)
    assert_same(gt, grows, ot, orows)


def test_pipeline_integer_keys_and_filter_on_int(ctx):
    rng = np.random.default_rng(9)
    n = 200_000
    key = rng.integers(0, 5000, n).astype(np.int64)
    qty = rng.integers(1, 100, n).astype(np.int32)
    probe = [O.TCol(O.I64, key), O.TCol(O.I32, qty)]
    bkey = rng.permutation(4000).astype(np.int64) + 500
    build = [O.TCol(O.I64, bkey), O.TCol(O.I64, (bkey % 7).astype(np.int64))]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 1)]
    # qty >= 50.5 on an integer column behaves as qty > 50.
    ok = qty > 50
    filt = [O.TCol(c.type, c.values[ok]) for c in probe]
    jt, jrows = O.join(filt, build, [0], [0], O.INNER)
    cols = [O.TCol(t, np.array([r[i] for r in jrows], {O.I32: np.int32, O.I64: np.int64}[t])) for i, t in enumerate(jt)]
    ot, orows = O.groupby(cols, [3], aggs)
    types, res = qeg.filter_join_agg(ctx, [to_gpu(c) for c in probe], [to_gpu(c) for c in build], 0, 0, 3, aggs,
                                     filter_col=1, filter_op=qeg.CMP_GE, filter_value=50.5)
    gt, grows = gpu_rows(res, types)
    assert_same(gt, grows, ot, orows)


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("seed,nulls", [(4, False), (5, True)])
def test_pipeline_trades_aggregates_specialised_kernel(ctx, seed, nulls, kernel, monkeypatch):
    """The trades workload's exact aggregate list -- COUNT(*), AVG(price),
    SUM(qty) -- runs the field-set-specialised kernels (with NULL counts when
    the columns have NULLs); device-resident columns as in the benchmark;
    thread-private states (the default), and the shared-state kernel with
    per-lane reductions or warp peer aggregation."""
    use_kernel(monkeypatch, kernel)
    trades, symbols = make_case(seed, nulls=nulls)
    aggs = [(O.COUNT_STAR, 0), (O.AVG, 1), (O.SUM, 2)]
    ot, orows = oracle_pipeline(trades, symbols, aggs)
    canon = StrCanon(trades[0].dictionary + symbols[0].dictionary)
    gp = [to_gpu(c, canon, device=True) for c in trades]
    gb = [to_gpu(c, canon, device=True) for c in symbols]
    types, res = qeg.filter_join_agg(ctx, gp, gb, 0, 0, 4, aggs, filter_col=1, filter_op=qeg.CMP_GT,
                                     filter_value=100.0)
    gt, grows = gpu_rows(res, types, canon)
    assert_same(gt, grows, ot, orows)


@pytest.mark.parametrize("op,dup", [(qeg.CMP_LT, True), (qeg.CMP_GE, False), (qeg.CMP_NE, True), (qeg.CMP_EQ, False)])
def test_pipeline_trades_shape_typed_kernel_ops_and_repeated_keys(ctx, op, dup):
    """The trades shape without NULLs (4-byte STR key, F64 filter column
    aggregated as AVG, I32 SUM) takes the typed thread-private kernel for
    every comparison; repeated symbols in the build side fan a row out to
    several sectors."""
    trades, symbols = make_case(6 + op, nulls=False, dup_syms=dup)
    aggs = [(O.COUNT_STAR, 0), (O.AVG, 1), (O.SUM, 2)]
    lit = float(np.round(trades[1].values[17], 6)) if op == qeg.CMP_EQ else 100.0
    ops = {qeg.CMP_LT: np.less, qeg.CMP_GE: np.greater_equal, qeg.CMP_NE: np.not_equal, qeg.CMP_EQ: np.equal}
    if op == qeg.CMP_EQ:
        trades[1].values[::7] = lit  # rows that pass an equality test
    ok = ops[op](trades[1].values, lit)
    filt = [O.TCol(c.type, c.values[ok], None, c.dictionary) for c in trades]
    jt, jrows = O.join(filt, symbols, [0], [0], O.INNER)
    cols = []
    for i, t in enumerate(jt):
        vals = [r[i] for r in jrows]
        if t == O.STR:
            d = sorted(set(vals)) or ["?"]
            cols.append(O.TCol(t, np.array([d.index(v) for v in vals], np.int32), None, d))
        else:
            dt = {O.I32: np.int32, O.I64: np.int64, O.F64: np.float64}[t]
            cols.append(O.TCol(t, np.array(vals, dt)))
    ot, orows = O.groupby(cols, [4], aggs)
    canon = StrCanon(trades[0].dictionary + symbols[0].dictionary)
    gp = [to_gpu(c, canon, device=True) for c in trades]
    gb = [to_gpu(c, canon, device=True) for c in symbols]
    types, res = qeg.filter_join_agg(ctx, gp, gb, 0, 0, 4, aggs, filter_col=1, filter_op=op, filter_value=lit)
    gt, grows = gpu_rows(res, types, canon)
    assert_same(gt, grows, ot, orows)


@pytest.mark.parametrize("op", [qeg.CMP_LT, qeg.CMP_LE, qeg.CMP_GT, qeg.CMP_GE, qeg.CMP_EQ, qeg.CMP_NE])
@pytest.mark.parametrize("lit", [0.0, -0.0, 100.0, float("inf")])
def test_pipeline_typed_kernel_f64_filter_edges(ctx, op, lit):
    """The typed kernel compares F64 values on the integer pipes: planted
    -0.0, +0.0, NaNs, infinities and values equal to the literal must pass or
    fail exactly as IEEE comparisons do (NaN fails all but !=, -0.0 == +0.0)."""
    trades, symbols = make_case(40 + op, n=200_000, nulls=False)
    v = trades[1].values
    specials = [0.0, -0.0, float("nan"), -float("nan"), float("inf"), -float("inf"), lit, 100.0, -100.0]
    for i, x in enumerate(specials):
        v[i::97 + i] = x
    aggs = [(O.COUNT_STAR, 0), (O.AVG, 1), (O.SUM, 2)]
    ops = {qeg.CMP_LT: np.less, qeg.CMP_LE: np.less_equal, qeg.CMP_GT: np.greater,
           qeg.CMP_GE: np.greater_equal, qeg.CMP_EQ: np.equal, qeg.CMP_NE: np.not_equal}
    with np.errstate(invalid="ignore"):
        ok = ops[op](v, lit)
    filt = [O.TCol(c.type, c.values[ok], None, c.dictionary) for c in trades]
    jt, jrows = O.join(filt, symbols, [0], [0], O.INNER)
    cols = []
    for i, t in enumerate(jt):
        vals = [r[i] for r in jrows]
        if t == O.STR:
            d = sorted(set(vals)) or ["?"]
            cols.append(O.TCol(t, np.array([d.index(x) for x in vals], np.int32), None, d))
        else:
            dt = {O.I32: np.int32, O.I64: np.int64, O.F64: np.float64}[t]
            cols.append(O.TCol(t, np.array(vals, dt)))
    ot, orows = O.groupby(cols, [4], aggs)
    canon = StrCanon(trades[0].dictionary + symbols[0].dictionary)
    gp = [to_gpu(c, canon, device=True) for c in trades]
    gb = [to_gpu(c, canon, device=True) for c in symbols]
    types, res = qeg.filter_join_agg(ctx, gp, gb, 0, 0, 4, aggs, filter_col=1, filter_op=op, filter_value=lit)
    gt, grows = gpu_rows(res, types, canon)
    assert_same(gt, grows, ot, orows)
