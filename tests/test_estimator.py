"""The learned estimator: the float64 restatement is checked against finite
differences (CPU); the GPU forward/backward kernels are checked against the
restatement (gradient check); training on the GPU reduces the loss; and the
shipped network estimates group counts better than the classic estimator,
which in turn lets the GROUP BY size its table right the first time."""
import math
import os

import numpy as np
import pytest

import mlp_ref as R
import qeg

WEIGHTS = os.path.join(os.path.dirname(qeg.LIB_PATH), "estimator_weights.f32")


def random_problem(seed, n=96):
    rng = np.random.default_rng(seed)
    p = np.zeros(R.NPARAMS, np.float32)
    o = 0
    for name, shape in R.SIZES:
        k = int(np.prod(shape))
        fan = shape[1] if len(shape) == 2 else 64
        p[o:o + k] = rng.normal(0, math.sqrt(2.0 / fan), k) if len(shape) == 2 else rng.normal(0, 0.1, k)
        o += k
    p = R.to_bf16(p)
    x = rng.random((n, R.IN)).astype(np.float32)
    t = rng.random((n, R.OUT)).astype(np.float32)
    return p, x, t


def test_restatement_matches_finite_differences():
    p, x, t = random_problem(1, n=8)
    p = p.astype(np.float64)
    _, g = R.loss_and_grad(p, x, t)
    rng = np.random.default_rng(2)
    for i in rng.choice(R.NPARAMS, 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        num = (R.loss_and_grad(p + e, x, t)[0] - R.loss_and_grad(p - e, x, t)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(g[i])


@pytest.mark.gpu
def test_gpu_gradients_match_float64_restatement():
    ctx = qeg.Context(0)  # a private context: these weights are not the shipped ones
    for seed in (3, 4):
        p, x, t = random_problem(seed)
        qeg.estimator_set_weights(ctx, p)
        loss, g = qeg.estimator_grad(ctx, x, t)
        rl, rg = R.loss_and_grad(p.astype(np.float64), x, t)
        assert abs(loss - rl) <= 1e-5 * max(1.0, abs(rl))
        # FP32 accumulation against FP64: relative error per parameter block.
        scale = np.abs(rg).max()
        assert np.abs(g - rg).max() <= 2e-4 * scale, np.abs(g - rg).max() / scale
        y = qeg.estimator_predict(ctx, x)
        ry, _ = R.forward(p.astype(np.float64), x)
        assert np.abs(y - ry).max() <= 1e-4 * max(1.0, np.abs(ry).max())
    ctx.close()


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    ctx = qeg.Context(0)
    rng = np.random.default_rng(5)
    x = rng.random((2048, R.IN)).astype(np.float32)
    w = rng.normal(0, 1, (R.IN, 2))
    t = (np.tanh(x @ w / 4) * 0.5 + 0.5).astype(np.float32)
    qeg.estimator_init(ctx, 7)
    l0, _ = qeg.estimator_grad(ctx, x, t)
    l1 = qeg.estimator_train(ctx, x, t, 60, 64, 3e-3, 11)
    ctx.close()
    assert l1 < 0.2 * l0, (l0, l1)


def zipf_column(torch, n, dom, s, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    cdf = torch.arange(1, dom + 1, dtype=torch.float64, device="cuda").pow_(-s).cumsum_(0)
    cdf /= cdf[-1].clone()
    r = torch.searchsorted(cdf, torch.rand(n, generator=g, device="cuda", dtype=torch.float64)).clamp_(max=dom - 1)
    keys = (r * -7046029254386353131) ^ 0x5DEECE66D  # an odd multiplier: a bijection on int64
    torch.cuda.synchronize()  # the library reads these on its own stream
    return keys.contiguous()


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained estimator weights shipped")
def test_learned_estimator_beats_classic_and_sizes_tables(monkeypatch):
    """What the network gains over the method without it, on Zipf key columns
    whose sample is 1/8 to 1/32 of the rows: a smaller median and worst-case
    log2 error of the group-count estimate, and GROUP BY tables that need fewer
    grow-and-replay passes when sized from it. Results are exact either way."""
    torch = pytest.importorskip("torch")
    ctx = qeg.Context(0)  # loads the shipped weights
    monkeypatch.setenv("QEG_ESTIMATOR_WEIGHTS", os.path.join(os.path.dirname(WEIGHTS), "no-such-weights.f32"))
    plain = qeg.Context(0)  # no network: the classic estimator sizes its tables
    cases = [(1 << 24, 1 << 24, 0.6, 1), (1 << 24, 1 << 26, 1.1, 2), (1 << 25, 1 << 22, 1.3, 3),
             (1 << 23, 1 << 25, 0.8, 4), (1 << 24, 1 << 20, 0.4, 5), (1 << 25, 1 << 26, 1.0, 6)]
    el, ec, rl, rc = [], [], [], []
    try:
        for n, dom, s, seed in cases:
            keys = zipf_column(torch, n, dom, s, seed)
            col = qeg.Col(keys, None, qeg.I64)
            f, classic, _ = qeg.sketch(ctx, col)
            learned = qeg.learned_groups(classic, float(qeg.estimator_predict(ctx, f)[0][0]),
                                         qeg.estimator_get_deadband(ctx))
            true = int(torch.unique(keys).numel())
            el.append(abs(math.log2(max(learned, 1)) - math.log2(true)))
            ec.append(abs(math.log2(max(classic, 1)) - math.log2(true)))
            for c, out in ((ctx, rl), (plain, rc)):
                a = qeg.Aggregate(c, [qeg.I64], [0], [(qeg.COUNT_STAR, 0)], qeg.agg_config(sizing=qeg.SIZE_LEARNED))
                a.consume([col])
                assert a.finish() == true
                out.append(a.stats()["resizes"])
                a.close()
    finally:
        plain.close()
        ctx.close()
    assert np.median(el) < np.median(ec), (el, ec)
    assert max(el) < max(ec), (el, ec)
    assert sum(rl) < sum(rc), (rl, rc)


def test_shipped_weights_file_carries_parameters_and_dead_band():
    """estimator_weights.f32: QEG_MLP_PARAMS float32 parameters, then the dead
    band of the correction (log2 units) that the trainer picked, in [0, 4]."""
    if not os.path.exists(WEIGHTS):
        pytest.skip("no trained estimator weights shipped")
    w = np.fromfile(WEIGHTS, dtype="<f4")
    assert w.size == qeg.MLP_PARAMS + 1
    assert np.all(np.isfinite(w))
    assert 0.0 <= float(w[-1]) <= 4.0
