"""Failure detection without a GPU fault.

Every device-side wait of the library (a composite-key row that another thread
has claimed but not yet published) is bounded: after its poll limit the kernel
raises an error word and returns, and the host turns the word into
QEG_ERR_TIMEOUT. The reference's CPU hash table never waits on another thread;
its analogue is the invariant that a probe never loops forever
(ops/hashtable.h:84-89). These tests make the wait run out on a row state word
that nothing publishes, then check that the same context still answers a
GROUP BY correctly (against the oracle).
"""
import numpy as np
import pytest

import oracle as O
import qeg
from util import assert_same, gpu_rows

pytestmark = pytest.mark.gpu


def _small_groupby_matches_oracle(ctx, seed):
    rng = np.random.default_rng(seed)
    n = 5000
    a = rng.integers(0, 17, n).astype(np.int64)
    b = rng.integers(0, 5, n).astype(np.int32)
    v = rng.uniform(-10, 10, n)
    cols = [O.TCol(O.I64, a), O.TCol(O.I32, b), O.TCol(O.F64, v)]
    aggs = [(O.COUNT_STAR, 0), (O.SUM, 2), (O.MAX, 2)]
    et, erows = O.groupby(cols, [0, 1], aggs)
    res = qeg.groupby(ctx, [qeg.Col(a), qeg.Col(b), qeg.Col(v)], [0, 1], aggs)
    gt, grows = gpu_rows(res, et)
    assert_same(gt, grows, et, erows, "composite-key GROUP BY after a timed-out wait")


@pytest.mark.parametrize("polls", [0, 300, 1 << 16])
def test_bounded_wait_times_out_and_context_survives(polls):
    ctx = qeg.Context(0)
    try:
        with pytest.raises(qeg.QegError) as e:
            ctx.check_bounded_wait(polls)
        assert e.value.code == -5, e.value  # QEG_ERR_TIMEOUT
        assert "bounded" in str(e.value)
        # The error word was cleared: the context is usable and correct.
        ctx.synchronize()
        _small_groupby_matches_oracle(ctx, polls)
        # And the check reports again on a second run.
        with pytest.raises(qeg.QegError) as e2:
            ctx.check_bounded_wait(polls)
        assert e2.value.code == -5
    finally:
        ctx.close()


def test_bounded_wait_rejects_limits_out_of_range():
    ctx = qeg.Context(0)
    try:
        for bad in (-1, (1 << 20) + 1):
            with pytest.raises(qeg.QegError) as e:
                ctx.check_bounded_wait(bad)
            assert e.value.code == -1
        ctx.synchronize()
    finally:
        ctx.close()
