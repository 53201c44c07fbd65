"""Autotuner of the batched GROUP BY (qeg_batch_*).

For every (group-count, skew) bucket of the batch planner it generates a
seeded synthetic batch of queries of that bucket, runs the batch under every
candidate (CTA-private table slots x rows per work item x warp peer
aggregation on/off), times the graph replays with CUDA events and keeps the
fastest; then it picks the block size on a mixed batch. The result is the
tuning table qeg_batch_create takes, written as JSON beside libqeg.so
(batch_tuning.json):

    {"tuning": [[max_log2_groups, skewed, smem_slots, rows_per_item, peer_rows], ...],
     "block_threads": B, "measured": {...}}

    python query-engine_gb300/autotune.py [--out PATH] [--queries N]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import qeg  # noqa: E402

BUCKETS = [2.0, 6.0, 10.0, 14.0, 17.0, 20.0]  # upper bounds on log2(groups)
SLOTS = [0, 256, 1024, 2048, 4096]
ITEMS = [1 << 13, 1 << 14, 1 << 16]
PEER = [0, 1]
BLOCKS = [256, 512, 1024]
AGGS = [(qeg.COUNT_STAR, 0), (qeg.SUM, 1), (qeg.AVG, 1), (qeg.MIN, 1), (qeg.MAX, 1)]


def make_batch(dev, g, rng, nq, lg_lo, lg_hi, skewed, rows_lo=1e4, rows_hi=2e6):
    """nq queries whose distinct-key domain is log-uniform in [2^lg_lo, 2^lg_hi];
    uniform keys, or Zipf(s), s in [1.1, 1.5], when `skewed` (None: a coin per
    query)."""
    sizes = np.exp(rng.uniform(np.log(rows_lo), np.log(rows_hi), nq)).astype(np.int64)
    doms = np.maximum(2, 2 ** rng.uniform(lg_lo, lg_hi, nq)).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1])
    key = torch.empty(n, dtype=torch.int32, device=dev)
    for q in range(nq):
        a, b, d = int(offs[q]), int(offs[q + 1]), int(doms[q])
        if skewed if skewed is not None else rng.random() < 0.5:
            cdf = torch.arange(1, d + 1, dtype=torch.float64, device=dev).pow_(-float(rng.uniform(1.1, 1.5)))
            cdf = cdf.cumsum_(0)
            cdf /= cdf[-1].clone()
            r = torch.searchsorted(cdf, torch.rand(b - a, generator=g, device=dev, dtype=torch.float64))
            r.clamp_(max=d - 1)
        else:
            r = torch.randint(0, d, (b - a,), generator=g, device=dev, dtype=torch.int64)
        x = (r * 2654435761 + 7919 * q) & 0xFFFFFFFF
        key[a:b] = torch.where(x >= (1 << 31), x - (1 << 32), x).to(torch.int32)
    val = torch.rand(n, generator=g, device=dev, dtype=torch.float64)
    torch.cuda.synchronize()
    return offs, key, val


def time_batch(ctx, offs, key, val, tuning, block, reps=3):
    b = qeg.Batch(ctx, offs, qeg.Col(key, None, qeg.I32), qeg.Col(val, None, qeg.F64), AGGS, tuning=tuning,
                  block_threads=block)
    stream = torch.cuda.ExternalStream(ctx.stream)
    b.run()
    b.finish()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.run()
        b.finish()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    b.close()
    return ms


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "batch_tuning.json"))
    ap.add_argument("--queries", type=int, default=192)
    ap.add_argument("--seed", type=int, default=20260615)
    args = ap.parse_args()
    dev = torch.device("cuda", 0)
    ctx = qeg.Context(0)
    rng = np.random.default_rng(args.seed)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed)
    table, measured = [], {}
    t0 = time.time()
    lo = 1.0
    for hi in BUCKETS:
        for skewed in (0, 1):
            offs, key, val = make_batch(dev, g, rng, args.queries, lo, hi, skewed)
            res = {}
            for slots in SLOTS:
                for item in ITEMS:
                    for peer in PEER:
                        # Every bucket maps to this candidate: the batch holds one bucket.
                        tun = [(64.0, 0, slots, item, peer), (64.0, 1, slots, item, peer)]
                        res[(slots, item, peer)] = time_batch(ctx, offs, key, val, tun, 512)
            best = min(res, key=res.get)
            table.append([hi, skewed, best[0], best[1], best[2]])
            measured["log2<=%g,skewed=%d" % (hi, skewed)] = {
                "rows": int(offs[-1]), "best": list(best), "best_ms": res[best],
                "all_ms": {"%d/%d/%d" % k: v for k, v in res.items()}}
            print("bucket log2<=%g skewed=%d: slots=%d rows/item=%d peer=%d %.3f ms" % (hi, skewed, best[0], best[1],
                                                                                       best[2], res[best]), flush=True)
            del key, val
        lo = hi
    # Block size on a mixed batch, with the tuned table.
    offs, key, val = make_batch(dev, g, rng, args.queries, 1.0, 20.0, None)
    blocks = {blk: time_batch(ctx, offs, key, val, [tuple(t) for t in table], blk) for blk in BLOCKS}
    block = min(blocks, key=blocks.get)
    measured["block_threads_ms"] = blocks
    out = {"tuning": table, "block_threads": block, "measured": measured,
           "device": torch.cuda.get_device_name(0), "seconds": time.time() - t0}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({"tuning": table, "block_threads": block}))
    ctx.close()


if __name__ == "__main__":
    main()
