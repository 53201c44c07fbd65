"""Parity at the measured sizes: every workload the benchmark times, at its full
size, against a checker that shares no code with the library's kernels.

- 1M-row plain GROUP BY (2^20 rows, I64 key over 1024 values, F64 with 5%
  NULLs, 2048-row batches, COUNT/SUM/AVG/MIN/MAX): every cell against the
  oracle (the restatement of the reference's Aggregate).
- 16M x 256M inner join COUNT/SUM, dense and sparse keys, every strategy: the
  exact count and sum against torch (sorted build keys + binary searches).
- 512M-row Zipf(1.1) GROUP BY: every group's COUNT, SUM(I64), MIN, MAX exactly
  and SUM(F64) within the reference's epsilon against a torch reduction.
- 4096-query batch: every group count against torch.unique, every cell of the
  8 largest, the overflowed and 16 random queries against the oracle.
- 200M-trade filter -> join -> GROUP BY: every sector's COUNT, SUM(qty) and
  AVG(price) against torch.

Integers, keys and counts are compared exactly; F64 with the reference's
comparator |a-b| <= 1e-9 + 1e-9*max(|a|,|b|) (oracle/result_set.h:53-54).
The workloads are the benchmark's own generators (bench.py), seeded.
"""
import os
import sys

import pytest

import qeg

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench

    return bench


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    return torch, torch.device("cuda", 0)


def test_plain_agg_1m_exact_shape_vs_oracle(torch_dev):
    torch, dev = torch_dev
    bench = _bench()
    W = bench.AggWorkload(dev, "agg1m")
    ctx = qeg.Context(0)
    try:
        for cfg in (qeg.agg_config(sizing=qeg.SIZE_LEARNED), qeg.agg_config(sizing=qeg.SIZE_FIXED)):
            p = W.parity(qeg, ctx, cfg)
            assert p["cells_vs_oracle_2048_row_batches"], p
            assert p["groups"] == 1024
    finally:
        ctx.close()


@pytest.mark.parametrize("sparse", [False, True], ids=["dense_keys", "sparse_keys"])
def test_join_16m_x_256m_count_sum_vs_torch(torch_dev, sparse):
    torch, dev = torch_dev
    bench = _bench()
    W = bench.JoinWorkload(dev, sparse=sparse)
    exp = W.expected_torch()
    # ~2^28 * 0.98 * 0.5 * 0.98 matches.
    assert 128_000_000 < exp[0] < 130_000_000
    ctx = qeg.Context(0)
    try:
        for strat in (qeg.JOIN_AUTO, qeg.JOIN_HASH, qeg.JOIN_PARTITIONED):
            res, st = W.run(qeg, ctx, strat)
            assert res == exp, (strat, st, res, exp)
            if strat == qeg.JOIN_AUTO:
                # Dense keys take the direct-address table; sparse keys cannot.
                assert (st["strategy"] == qeg.JOIN_DENSE) != sparse, st
    finally:
        ctx.close()
        del W
        torch.cuda.empty_cache()


def test_skew_agg_512m_every_group_vs_torch(torch_dev):
    torch, dev = torch_dev
    bench = _bench()
    W = bench.AggWorkload(dev, "skew")
    ctx = qeg.Context(0)
    try:
        p = W.parity(qeg, ctx, qeg.agg_config(sizing=qeg.SIZE_LEARNED, hot_keys=-1))
        assert p["ok"], p
        assert p["groups"] > 20_000_000
    finally:
        ctx.close()
        del W
        torch.cuda.empty_cache()


def test_batch_4096_queries_sampled_vs_oracle(torch_dev):
    torch, dev = torch_dev
    bench = _bench()
    import numpy as np

    W = bench.BatchWorkload(dev)
    ctx = qeg.Context(0)
    tuning, block, _ = bench.load_tuning()
    k, v = W.cols()
    b = qeg.Batch(ctx, W.offsets, k, v, W.aggs, tuning=tuning, block_threads=block)
    try:
        b.run()
        groups = b.finish()
        stats = [b.stats(q) for q in range(len(groups))]
        true = np.array([int(torch.unique(W.key[int(W.offsets[q]):int(W.offsets[q + 1])]).numel())
                         for q in range(len(groups))])
        assert np.array_equal(true, groups.astype(np.int64))
        p = bench.batch_parity_oracle(W, b, groups, stats)
        assert p["ok"], p
        # A second replay of the captured graph gives the same results.
        b.run()
        assert np.array_equal(b.finish(), groups)
        p2 = bench.batch_parity_oracle(W, b, groups, stats, nrandom=4, seed=7)
        assert p2["ok"], p2
    finally:
        b.close()
        ctx.close()
        del W
        torch.cuda.empty_cache()


def test_pipeline_200m_per_sector_vs_torch(torch_dev):
    torch, dev = torch_dev
    bench = _bench()
    W = bench.PipelineWorkload(dev)
    ctx = qeg.Context(0)
    try:
        types, res = W.run(qeg, ctx)
        p = bench.pipeline_parity_torch(W, res)
        assert p["ok"], p
        assert p["sectors"] == 32
    finally:
        ctx.close()
        del W
        torch.cuda.empty_cache()


def test_bench_helpers_unpack_and_compare(torch_dev):
    """The checkers themselves: validity unpacking and the F64 comparator."""
    torch, dev = torch_dev
    bench = _bench()
    import numpy as np

    rng = np.random.default_rng(3)
    mask = rng.random(1000) < 0.7
    words = torch.from_numpy(qeg.pack_validity(mask).view(np.int64)).to(dev)
    assert np.array_equal(bench.unpack_bits_torch(words, 1000).cpu().numpy(), mask)
    a = torch.tensor([1.0, 1e12, float("nan"), 0.0], dtype=torch.float64, device=dev)
    b = torch.tensor([1.0 + 1e-10, 1e12 + 500.0, float("nan"), 2e-9], dtype=torch.float64, device=dev)
    assert bench.f64_close_torch(a, b) == 1  # only 0 vs 2e-9 exceeds 1e-9 + 1e-9*max
