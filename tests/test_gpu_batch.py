"""Batched GROUP BY (qeg_batch_*) against the oracle, query by query.

Each query of a batch is one GROUP BY over its slice of the (key, value)
columns, so every query is checked against the oracle's GROUP BY of that slice
(the reference's Aggregate over the same rows): keys, counts and MIN/MAX
exactly, F64 SUM/AVG within 1e-9 abs + 1e-9 rel. The batches mix row counts,
cardinalities and skews like the 4096-query workload (log-uniform sizes,
uniform or Zipf keys), scaled so the oracle finishes in seconds.
"""
import numpy as np
import pytest

import oracle as O
import qeg
from util import assert_same, gpu_rows

pytestmark = pytest.mark.gpu

AGGS = [(O.COUNT_STAR, 0), (O.COUNT, 1), (O.SUM, 1), (O.AVG, 1), (O.MIN, 1), (O.MAX, 1)]


def zipf_ranks(rng, n, dom, s):
    w = np.arange(1, dom + 1, dtype=np.float64) ** -s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(n)), dom - 1)


def make_batch(seed, nq, lo, hi, key_nulls=0.0, val_nulls=0.0, vtype=O.F64, align=1):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), nq)).astype(np.int64)
    sizes = (sizes + align - 1) // align * align
    keys, vals = [], []
    for n in sizes:
        card = int(np.exp(rng.uniform(np.log(4), np.log(max(5, n)))))
        if rng.random() < 0.5:
            r = rng.integers(0, card, n)
        else:
            r = zipf_ranks(rng, n, card, rng.uniform(0.5, 1.5))
        # Spread the ranks over int32 with a bijection (odd multiplier mod 2^32).
        keys.append(((r.astype(np.int64) * 2654435761) & 0xFFFFFFFF).astype(np.uint32).view(np.int32))
        if vtype == O.F64:
            vals.append(rng.random(n))
        else:
            vals.append(rng.integers(-(1 << 40), 1 << 40, n))
    key = np.concatenate(keys)
    val = np.concatenate(vals)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    kvalid = rng.random(len(key)) >= key_nulls if key_nulls else None
    vvalid = rng.random(len(key)) >= val_nulls if val_nulls else None
    kcol = O.TCol(O.I32, key, kvalid)
    vcol = O.TCol(vtype, val, vvalid)
    return offs, kcol, vcol


def check_batch(ctx, offs, kcol, vcol, aggs=AGGS, tuning=(), runs=1):
    kw, vw = kcol.words(), vcol.words()
    b = qeg.Batch(ctx, offs, qeg.Col(kcol.values, kw, kcol.type), qeg.Col(vcol.values, vw, vcol.type), aggs,
                  tuning=tuning)
    try:
        for _ in range(runs):
            b.run()
            groups = b.finish()
            for q in range(len(offs) - 1):
                a, z = int(offs[q]), int(offs[q + 1])
                sl = [O.TCol(c.type, c.values[a:z], None if c.valid is None else c.valid[a:z]) for c in (kcol, vcol)]
                ot, orows = O.groupby(sl, [0], aggs, 2048)
                assert int(groups[q]) == len(orows), (q, int(groups[q]), len(orows))
                gt, grows = gpu_rows(b.fetch(q), b.result_types)
                assert_same(gt, grows, ot, orows, "query %d" % q)
        return [b.stats(q) for q in range(len(offs) - 1)]
    finally:
        b.close()


def test_batch_mixed_queries(ctx):
    offs, k, v = make_batch(1, 48, 1000, 100000)
    check_batch(ctx, offs, k, v)


def test_batch_replay_twice_gives_same_results(ctx):
    offs, k, v = make_batch(2, 16, 1000, 50000)
    check_batch(ctx, offs, k, v, runs=2)


def test_batch_with_nulls_and_int_values(ctx):
    offs, k, v = make_batch(3, 24, 1000, 40000, key_nulls=0.05, val_nulls=0.1, vtype=O.I64, align=64)
    check_batch(ctx, offs, k, v)


def test_batch_tuning_table_global_only(ctx):
    offs, k, v = make_batch(4, 20, 1000, 60000)
    st = check_batch(ctx, offs, k, v, tuning=[(64.0, 0, 0, 4096), (64.0, 1, 0, 4096)])
    assert all(s["strategy"] == qeg.AGG_GLOBAL for s in st)


def test_batch_tuning_table_smem(ctx):
    offs, k, v = make_batch(5, 20, 1000, 60000)
    st = check_batch(ctx, offs, k, v, tuning=[(64.0, 0, 1024, 2048), (64.0, 1, 256, 8192)])
    assert all(s["strategy"] == qeg.AGG_SMEM for s in st)


def test_batch_empty_and_tiny_queries(ctx):
    rng = np.random.default_rng(6)
    sizes = [0, 1, 5, 0, 3000, 64, 0]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1])
    k = O.TCol(O.I32, rng.integers(-3, 4, n).astype(np.int32))
    v = O.TCol(O.F64, rng.random(n))
    check_batch(ctx, offs, k, v)


def test_batch_underestimate_reruns_exactly():
    # A private context whose estimator always answers "far fewer groups than
    # the classic estimate" (all weights zero, output bias -1, i.e. 2^-32 of
    # it): tables are sized from the sample's HyperLogLog floor alone, so a
    # query with far more groups than its sample shows overflows and is re-run
    # with larger tables; its result must still be exact.
    ctx = qeg.Context(0)
    try:
        w = np.zeros(qeg.MLP_PARAMS, np.float32)
        w[qeg.MLP_PARAMS - 2] = -1.0  # b3[0]
        qeg.estimator_set_weights(ctx, w)
        rng = np.random.default_rng(7)
        n = 1 << 20
        key = O.TCol(O.I32, rng.permutation(n).astype(np.int32))
        val = O.TCol(O.F64, rng.random(n))
        offs = np.array([0, 5000, n], dtype=np.uint64)
        key.values[:5000] = rng.integers(0, 10, 5000)
        st = check_batch(ctx, offs, key, val, aggs=[(O.COUNT_STAR, 0), (O.SUM, 1)])
        assert st[1]["fell_back"] == 1 and st[0]["fell_back"] == 0, st
    finally:
        ctx.close()


def test_batch_rejects_bad_offsets(ctx):
    k = qeg.Col(np.zeros(10, np.int32), None, qeg.I32)
    v = qeg.Col(np.zeros(10, np.float64), None, qeg.F64)
    with pytest.raises(qeg.QegError):
        qeg.Batch(ctx, [0, 6, 4, 10], k, v, [(qeg.COUNT_STAR, 0)])
    with pytest.raises(qeg.QegError):
        qeg.Batch(ctx, [0, 6, 9], k, v, [(qeg.COUNT_STAR, 0)])
