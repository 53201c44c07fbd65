"""Trains the learned cardinality / skew estimator on the GPU.

Training pairs are (sketch features, exact statistics) of seeded synthetic key
columns: the features come from qeg_sketch (a 2^20-row strided sample, what
the ordinary GROUP BY plans with) and from qeg_sketch_batch (the batch
planner's one-CTA sketch of a 2^16-row sample), the targets from the exact
GROUP BY engine over the whole column -- the number of groups and the share of
rows carried by the 2048 largest groups. Families:
uniform over a domain, Zipf(s) for s in [0.3, 1.6], a sequential key with
duplication, and a mixture (uniform background plus a heavy head). Row counts
and domains are log-uniform so the sample fraction varies from 1 to ~1/256.

The network is trained with the project's forward / backward / Adam kernels
(qeg_estimator_train) and written to query-engine_gb300/estimator_weights.f32,
with a report of its error next to the classic estimator's on held-out data.

    python query-engine_gb300/train_estimator.py [--datasets N] [--out PATH]
"""
import argparse
import json
import math
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import qeg  # noqa: E402

HOT_K = 2048


def scramble(x, salt):
    """A bijective 64-bit mix of an int64 tensor (splitmix64 finaliser written
    with logical shifts), so ranks map to spread-out keys without indexing."""
    m30, m27, m31 = (1 << 34) - 1, (1 << 37) - 1, (1 << 33) - 1
    x = x ^ salt
    x = x ^ ((x >> 30) & m30)
    x = x * -4658895280553007687  # 0xbf58476d1ce4e5b9 as int64
    x = x ^ ((x >> 27) & m27)
    x = x * -7723592293110705685  # 0x94d049bb133111eb as int64
    return x ^ ((x >> 31) & m31)


def gen_keys(rng, g, dev):
    """One seeded key column: (keys int64 tensor, description). Only
    elementwise torch ops: no gathers."""
    n = int(2 ** rng.uniform(14, 29.5))
    fam = rng.choice(["uniform", "zipf", "sequential", "mixture"], p=[0.3, 0.4, 0.1, 0.2])
    dom = int(2 ** rng.uniform(2, 28))
    salt = int(rng.integers(0, 1 << 62))
    if fam == "uniform":
        k = torch.randint(0, dom, (n,), generator=g, device=dev, dtype=torch.int64)
        desc = {"family": fam, "domain": dom}
    elif fam == "zipf":
        s = float(rng.uniform(0.3, 1.6))
        dom = min(dom, 1 << 27)
        cdf = torch.arange(1, dom + 1, dtype=torch.float64, device=dev).pow_(-s).cumsum_(0)
        cdf /= cdf[-1].clone()
        r = torch.searchsorted(cdf, torch.rand(n, generator=g, device=dev, dtype=torch.float64)).clamp_(0, dom - 1)
        del cdf
        k = scramble(r, salt)
        desc = {"family": fam, "domain": dom, "s": s}
    elif fam == "sequential":
        rep = int(2 ** rng.uniform(0, 8))
        k = scramble(torch.arange(n, device=dev, dtype=torch.int64) // rep, salt)
        desc = {"family": fam, "repeat": rep}
    else:
        head = int(2 ** rng.uniform(0, 12))
        frac = float(rng.uniform(0.1, 0.9))
        hot = torch.rand(n, generator=g, device=dev) < frac
        k = torch.where(hot, torch.randint(0, head, (n,), generator=g, device=dev, dtype=torch.int64),
                        torch.randint(head, head + dom, (n,), generator=g, device=dev, dtype=torch.int64))
        desc = {"family": fam, "domain": dom, "head": head, "hot_frac": frac}
    desc["rows"] = n
    return k.contiguous(), desc


def exact_stats(ctx, keys):
    """Exact group count and top-2048 share, from the exact GROUP BY engine."""
    cfg = qeg.agg_config(expected_groups=max(1024, min(keys.numel(), 1 << 27)))
    a = qeg.Aggregate(ctx, [qeg.I64], [0], [(qeg.COUNT_STAR, 0)], cfg)
    a.consume([qeg.Col(keys, None, qeg.I64)])
    n = a.finish()
    counts = a.fetch_torch()[1][0]
    a.close()
    torch.cuda.synchronize()
    if counts.numel() != n or n < 1:
        raise RuntimeError("group count mismatch: %d vs %d" % (counts.numel(), n))
    top = torch.sort(counts, descending=True).values[: min(HOT_K, n)]
    share = float(top.sum().item()) / max(1, keys.numel())
    return n, share


def targets(groups, share, classic):
    """The network's first output corrects the classic estimate in log space."""
    return [(math.log2(1.0 + groups) - math.log2(1.0 + classic)) / 32.0, share]


def build_set(ctx, rng, count, dev, seed):
    """Two examples per column: the column sketch of the ordinary GROUP BY
    (a 2^20-row sample) and the batch planner's per-query sketch (one CTA,
    a 2^16-row sample), with the same exact targets."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    X, T, C, D = [], [], [], []
    for i in range(count):
        keys, desc = gen_keys(rng, g, dev)
        torch.cuda.synchronize()
        col = qeg.Col(keys, None, qeg.I64)
        f, classic, _ = qeg.sketch(ctx, col)
        fb, cb = qeg.sketch_batch(ctx, col, [0, keys.numel()], 1 << 16)
        ctx.synchronize()
        groups, share = exact_stats(ctx, keys)
        ctx.synchronize()
        print("dataset %d %s groups=%d share=%.3f" % (i, desc, groups, share), flush=True)
        for feat, cl, kind in ((f, classic, "column"), (fb[0], float(cb[0]), "batch")):
            X.append(feat)
            T.append(targets(groups, share, cl))
            C.append(cl)
            d = dict(desc)
            d.update({"groups": groups, "top_share": share, "classic": cl, "sketch": kind})
            D.append(d)
        del keys
    return np.array(X, np.float32), np.array(T, np.float32), np.array(C), D


def log2_err(est, true):
    return abs(math.log2(max(est, 1.0)) - math.log2(max(true, 1.0)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--datasets", type=int, default=2000)
    ap.add_argument("--heldout", type=int, default=300)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=os.path.join(HERE, "estimator_weights.f32"))
    ap.add_argument("--report", default=None)
    ap.add_argument("--seed", type=int, default=20260615)
    ap.add_argument("--no-train", action="store_true",
                    help="evaluate the weights already in --out (and pick the dead band) without training")
    args = ap.parse_args()
    dev = torch.device("cuda", 0)
    ctx = qeg.Context(0)
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    X, T, C, D = build_set(ctx, rng, args.datasets, dev, args.seed)
    Xh, Th, Ch, Dh = build_set(ctx, rng, args.heldout, dev, args.seed + 1)
    t_data = time.time() - t0
    t1 = time.time()
    losses = []
    if args.no_train:
        qeg.estimator_set_weights(ctx, np.fromfile(args.out, dtype="<f4")[:qeg.MLP_PARAMS])
    else:
        qeg.estimator_init(ctx, args.seed)
        for phase, lr in ((args.epochs // 2, 3e-3), (args.epochs // 4, 1e-3),
                          (args.epochs - 3 * (args.epochs // 4), 3e-4)):
            losses.append(qeg.estimator_train(ctx, X, T, phase, 64, lr, args.seed + len(losses)))
    t_train = time.time() - t1
    # The dead band on the network's correction, picked on the TRAINING
    # columns: the smallest mean absolute log2 error among the bands whose
    # median error is no worse than the classic estimator's (the network's
    # small corrections are noise where the classic estimate is already
    # close; its large ones fix the classic underestimates in the tail). It is
    # stored after the parameters in the weights file and set in the context.
    Yt = qeg.estimator_predict(ctx, X)
    true_t = [d["groups"] for d in D]
    classic_median_t = float(np.median([log2_err(c, t) for c, t in zip(C, true_t)]))
    bands = {}
    for band in (0.0, 0.03, 0.06, 0.09, 0.125, 0.15, 0.2, 0.25, 0.3, 0.4, 0.5, 0.75, 1.0):
        e = [log2_err(qeg.learned_groups(c, float(y[0]), band), t) for c, y, t in zip(C, Yt, true_t)]
        bands[band] = {"mean": float(np.mean(e)), "median": float(np.median(e)), "p90": float(np.percentile(e, 90))}
    ok = [b for b in bands if bands[b]["median"] <= classic_median_t] or list(bands)
    best_band = min(ok, key=lambda b: bands[b]["mean"])
    qeg.estimator_set_deadband(ctx, best_band)
    if not args.no_train:
        w = qeg.estimator_get_weights(ctx)
        np.concatenate([w.astype("<f4"), np.array([best_band], "<f4")]).tofile(args.out)
    Y = qeg.estimator_predict(ctx, Xh)
    learned = [qeg.learned_groups(c, float(y[0]), best_band) for c, y in zip(Ch, Y)]
    learned_raw = [qeg.learned_groups(c, float(y[0]), 0.0) for c, y in zip(Ch, Y)]
    true = [d["groups"] for d in Dh]
    e_learned = [log2_err(a, b) for a, b in zip(learned, true)]
    e_raw = [log2_err(a, b) for a, b in zip(learned_raw, true)]
    e_classic = [log2_err(a, b) for a, b in zip(Ch, true)]
    share_err = [abs(float(y[1]) - d["top_share"]) for y, d in zip(Y, Dh)]
    by_kind = {}
    for kind in ("column", "batch"):
        idx = [i for i, d in enumerate(Dh) if d["sketch"] == kind]
        by_kind[kind] = {"median_learned": float(np.median([e_learned[i] for i in idx])),
                         "median_classic": float(np.median([e_classic[i] for i in idx])),
                         "p90_learned": float(np.percentile([e_learned[i] for i in idx], 90)),
                         "p90_classic": float(np.percentile([e_classic[i] for i in idx], 90))}
    report = {
        "datasets": args.datasets, "heldout": args.heldout, "epochs": args.epochs,
        "train_loss": losses, "data_s": t_data, "train_s": t_train,
        "heldout_median_abs_log2_error": {"learned": float(np.median(e_learned)),
                                          "classic": float(np.median(e_classic))},
        "heldout_p90_abs_log2_error": {"learned": float(np.percentile(e_learned, 90)),
                                       "classic": float(np.percentile(e_classic, 90))},
        "heldout_top_share_mae": float(np.mean(share_err)),
        "heldout_by_sketch": by_kind,
        "correction_deadband": best_band,
        "training_columns_classic_median": classic_median_t,
        "deadband_on_training_columns": {str(k): v for k, v in bands.items()},
        "heldout_without_deadband": {"median": float(np.median(e_raw)), "p90": float(np.percentile(e_raw, 90))},
    }
    print(json.dumps(report))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    ctx.close()


if __name__ == "__main__":
    main()
