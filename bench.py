"""Benchmark of the GPU hash-join / GROUP BY path (one JSON line on rank 0).

Default workload (the headline): the plain inner hash join of a 16M-row build
side (unique int64 keys, a random permutation of 0..2^24-1, 2% NULL keys)
against a 256M-row probe side (int64 keys, 50% drawn from the build keys and
50% from the disjoint range [2^24, 2^25), 2% NULL keys, int64 payload uniform
in [0, 2^20)), output COUNT(*) and SUM(probe payload) of the matched rows.
Synthetic, seeded data of exactly that shape is generated on the GPU.

One step = build the join table from the resident build side, then probe the
whole probe side through the fused COUNT/SUM sink. `value` is rows/s over
build + probe rows with inputs resident in HBM (inputs exceed L2, so no flush
is needed); `e2e` is the same metric through the C ABI from pinned host
buffers, host->device copies inside the timed region. `full_size_parity`
compares the result with a torch computation that uses no library kernel and
with the oracle run on the whole workload (the CPU baseline's run).

The default run adds sub-objects for the other workloads of the metric, each
with its roofline, clocks and full-size parity: `sparse_keys` (the same join
with keys spread over int64, so the hash table is used), `plain_agg` (1M rows,
1024 keys), `skew_agg` (512M Zipf rows, learned vs plain sizing), `batch`
(4096 GROUP BY queries in one persistent kernel) and `pipeline` (filter ->
join -> GROUP BY over 200M trades).

--impl reference times the reference's CPU algorithm (the oracle's port of its
morsel-parallel engine, with all host threads) on the whole join workload.
--workload selects one other workload of the engine for measurement.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(REPO, "query-engine_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

SEED = 20260615
# DRAM bytes (read + write) per probe row of the dense-table COUNT/SUM sink,
# from one ncu capture on a 64M-row probe side; the traffic grows in
# proportion to the probe rows (the 2 MiB dense bitmap stays in L2).
SINK_TRAFFIC_PER_ROW = (1082.670e6 + 3.291e6) / (1 << 26)
# The same figure for the hashed-table sink of the sparse-key join (16M-key
# table, 64M-row probe side): mostly whole 128-byte table lines, one per hit.
HASH_SINK_TRAFFIC_PER_ROW = (5139.149e6 + 46.900e6) / (1 << 26)


def replica_throughput(total_ms, rows_per_rank, steps, world, device):
    """Replicas only: every rank runs the whole workload on its own GPU. The
    job's time is the slowest rank's (an all-reduce MAX over the ranks; the
    only collective, outside the data path) and its throughput counts the rows
    of every rank: (max ms, rows/s)."""
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, rows_per_rank * steps * world / (total_ms / 1e3)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([time.time()] + [x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        """Median SM clock and active throttle reasons of the samples taken
        while [t0, t1] ran (the timed region, widened by one sampling period);
        a timed region shorter than the period falls back to every sample of
        the run, and says so."""
        time.sleep(0.3)
        rows = [r for r in self.rows if len(r) >= 10]
        window = "timed region"
        if t0 is not None:
            sel = [r for r in rows if t0 - 0.25 <= r[0] <= t1 + 0.25]
            if sel:
                rows = sel
            else:
                window = "warm-up and timed region (timed region shorter than the 200 ms sampling period)"
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 6 + i and r[6 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window": window}


def pack_bits_torch(valid):
    """bool [n] -> int64 validity words (bit i of word i/64, LSB-first)."""
    n = valid.numel()
    nw = (n + 63) // 64
    pad = torch.ones(nw * 64, dtype=torch.bool, device=valid.device)
    pad[:n] = valid
    w8 = (pad.view(-1, 8).to(torch.uint8) << torch.arange(8, device=valid.device, dtype=torch.uint8)).sum(
        1, dtype=torch.uint8)
    return w8.view(torch.int64).contiguous()


# ---------------------------------------------------------------------------
# Full-size parity helpers: independent torch computations of each workload's
# result, computed without the library's kernels.
# ---------------------------------------------------------------------------
def unpack_bits_torch(words, n):
    """int64 validity words (bit i of word i/64, LSB-first) -> bool [n]."""
    b = words.contiguous().view(torch.uint8)
    bits = (b.unsqueeze(1) >> torch.arange(8, device=b.device, dtype=torch.uint8)) & 1
    return bits.reshape(-1)[:n].bool()


def f64_close_torch(a, b):
    """The reference's F64 comparator (oracle/result_set.h:53-54,
    oracle/result_set.cpp:84-92): |a-b| <= 1e-9 + 1e-9*max(|a|,|b|), NaN equal
    to NaN. Returns the number of mismatches."""
    tol = 1e-9 + 1e-9 * torch.maximum(a.abs(), b.abs())
    ok = ((a - b).abs() <= tol) | (torch.isnan(a) & torch.isnan(b))
    return int((~ok).sum())


# ---------------------------------------------------------------------------
# Workload: 16M x 256M inner join, COUNT(*) + SUM(probe payload)
# ---------------------------------------------------------------------------
# Odd multiplier and offset of the bijection on 64-bit integers that turns the
# dense key set into a sparse one (k -> k*MUL + ADD mod 2^64): keys stay unique,
# the probe side's disjoint range stays disjoint, and the key range spans all
# of int64, so no direct-address table applies.
SPARSE_MUL = 0x9E3779B97F4A7C15 - (1 << 64)
SPARSE_ADD = 0x2545F4914F6CDD1D


class JoinWorkload:
    """`sparse=False`: the join of the task's shape -- build keys a random
    permutation of 0..nbuild-1. `sparse=True`: the same rows with every key (build
    and probe) pushed through the odd-multiplier bijection, so the build side is
    16M unique keys spread over all of int64 and the join takes the hash table."""

    def __init__(self, dev, nbuild=1 << 24, nprobe=1 << 28, seed=SEED + 2, sparse=False, distinct=None):
        """`distinct` (with sparse=True): build keys drawn with repetition from
        `distinct` values (0..distinct-1 before the bijection), so the build
        side repeats each key nbuild / distinct times on average."""
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.sparse = sparse
        self.distinct = distinct
        self.name = "join_%dMx%dM_count_sum%s" % (
            nbuild >> 20, nprobe >> 20,
            ("_repeated_keys_%dM_distinct" % (distinct >> 20)) if distinct else ("_sparse_keys" if sparse else ""))
        self.nbuild, self.nprobe = nbuild, nprobe
        if distinct:
            self.bkey = torch.randint(0, distinct, (nbuild,), generator=g, device=dev, dtype=torch.int64)
        else:
            self.bkey = torch.randperm(nbuild, generator=g, device=dev, dtype=torch.int64)
        self.bvalid = pack_bits_torch(torch.rand(nbuild, generator=g, device=dev) >= 0.02)
        hit = torch.rand(nprobe, generator=g, device=dev) < 0.5
        span = distinct or nbuild
        inb = torch.randint(0, span, (nprobe,), generator=g, device=dev, dtype=torch.int64)
        out = torch.randint(span, 2 * span, (nprobe,), generator=g, device=dev, dtype=torch.int64)
        self.pkey = torch.where(hit, inb, out)
        del inb, out, hit
        self.pvalid = pack_bits_torch(torch.rand(nprobe, generator=g, device=dev) >= 0.02)
        self.pval = torch.randint(0, 1 << 20, (nprobe,), generator=g, device=dev, dtype=torch.int64)
        if sparse:
            self.bkey.mul_(SPARSE_MUL).add_(SPARSE_ADD)
            self.pkey.mul_(SPARSE_MUL).add_(SPARSE_ADD)
        torch.cuda.synchronize()

    def rows(self):
        return self.nbuild + self.nprobe

    def algorithmic_probe_bytes(self):
        # key 8 B + payload 8 B + 1/8 B validity per probe row
        return self.nprobe * 16 + (self.nprobe + 7) // 8

    def algorithmic_build_bytes(self):
        return self.nbuild * 8 + (self.nbuild + 7) // 8

    def h2d_bytes(self):
        return self.nbuild * 8 + self.bvalid.numel() * 8 + self.nprobe * 16 + self.pvalid.numel() * 8

    def run(self, qeg, ctx, strategy, events=None, host=None, sizing=None):
        """One step: build the table from the build side, probe the whole probe
        side through the COUNT/SUM sink. `events` = [build start, probe start,
        probe end, stream] (CUDA events recorded on the library's stream)."""
        src = host if host is not None else self
        j = qeg.Join(ctx, [qeg.I64, qeg.I64], [qeg.I64], [0], [0], strategy=strategy,
                     sizing=qeg.SIZE_LEARNED if sizing is None else sizing)
        if events:
            events[0].record(events[3])
        j.build([qeg.Col(src.bkey, src.bvalid, qeg.I64)])
        j.build_finish()
        if events:
            events[1].record(events[3])
        j.probe_count_sum(qeg.Col(src.pkey, src.pvalid, qeg.I64), qeg.Col(src.pval, None, qeg.I64))
        if events:
            events[2].record(events[3])
        res = j.count_sum()
        st = j.stats()
        j.close()
        return res, st

    def host_copy(self):
        class H:
            pass

        h = H()
        for k in ("bkey", "bvalid", "pkey", "pvalid", "pval"):
            setattr(h, k, getattr(self, k).cpu().pin_memory())
        return h

    def cpu_columns(self, probe_rows):
        """The first `probe_rows` probe rows and the whole build side as oracle
        columns: (probe key, probe payload, build key, build payload)."""
        import oracle as O

        bk = self.bkey.cpu().numpy()
        bv = unpack_bits_torch(self.bvalid, self.nbuild).cpu().numpy()
        pk = self.pkey[:probe_rows].cpu().numpy()
        pv = unpack_bits_torch(self.pvalid[: (probe_rows + 63) // 64], probe_rows).cpu().numpy()
        pval = self.pval[:probe_rows].cpu().numpy()
        return (O.TCol(O.I64, pk, pv), O.TCol(O.I64, pval), O.TCol(O.I64, bk, bv),
                O.TCol(O.I64, np.zeros(self.nbuild, np.int64)))

    def expected_torch(self, chunk=1 << 25):
        """COUNT(*) and SUM(probe payload) of the inner join, from torch alone:
        the non-NULL build keys sorted, each non-NULL probe key's multiplicity
        found by two binary searches. NULL keys never match (kNeverMatch,
        ops/hashtable.cpp:135-163)."""
        bs = torch.sort(self.bkey[unpack_bits_torch(self.bvalid, self.nbuild)]).values
        count = 0
        total = 0
        for a in range(0, self.nprobe, chunk):
            b = min(self.nprobe, a + chunk)
            pk = self.pkey[a:b]
            pm = unpack_bits_torch(self.pvalid[a // 64:(b + 63) // 64], b - a)
            m = (torch.searchsorted(bs, pk, right=True) - torch.searchsorted(bs, pk)) * pm
            count += int(m.sum())
            total += int((m * self.pval[a:b]).sum())
        return count, (total if count else None)


def zipf_keys(n, domain, s, g, dev, chunk=1 << 25):
    """n keys with an exact discrete Zipf(s) rank distribution over `domain`
    values (inverse-CDF sampling), mapped through a seeded permutation so hot
    keys are spread over the key space. The CDF is summed on the host: a
    parallel float scan on the device may associate differently from run to
    run, which moves a few samples across rank boundaries."""
    cdf = torch.arange(1, domain + 1, dtype=torch.float64).pow_(-s).cumsum_(0)
    cdf = (cdf / cdf[-1]).to(dev)
    perm = torch.randperm(domain, generator=g, device=dev, dtype=torch.int64)
    out = torch.empty(n, dtype=torch.int64, device=dev)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        u = torch.rand(b - a, generator=g, device=dev, dtype=torch.float64)
        r = torch.searchsorted(cdf, u).clamp_(max=domain - 1)
        out[a:b] = perm[r]
    del cdf, perm
    return out


class AggWorkload:
    """GROUP BY workloads: `skew` = 512M rows, int64 key Zipf(1.1) over 64M
    values, I64 value U[-2^31, 2^31), F64 value N(0, 1e3); COUNT(*), SUM(I64),
    SUM(F64), MIN(I64), MAX(I64). `agg1m` = 2^20 rows, int64 key uniform over
    1024 values, F64 value U[0, 1000) with 5% NULLs; COUNT(*), SUM, AVG, MIN,
    MAX."""

    def __init__(self, dev, kind, nrows=None, seed=SEED + 3):
        import qeg

        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.kind = kind
        self.seed = seed
        if kind == "skew":
            self.n = nrows or (512 << 20)
            self.name = "skew_agg_%dM_zipf1.1_over_64M" % (self.n >> 20)
            self.key = zipf_keys(self.n, 64 << 20, 1.1, g, dev)
            self.v1 = torch.randint(-(1 << 31), 1 << 31, (self.n,), generator=g, device=dev, dtype=torch.int64)
            self.v2 = torch.randn(self.n, generator=g, device=dev, dtype=torch.float64).mul_(1e3)
            self.cols = [qeg.Col(self.key, None, qeg.I64), qeg.Col(self.v1, None, qeg.I64),
                         qeg.Col(self.v2, None, qeg.F64)]
            self.aggs = [(qeg.COUNT_STAR, 0), (qeg.SUM, 1), (qeg.SUM, 2), (qeg.MIN, 1), (qeg.MAX, 1)]
            self.row_bytes = 24
        else:
            self.name = "plain_agg_1M_1024keys"
            self.n = nrows or (1 << 20)
            self.key = torch.randint(0, 1024, (self.n,), generator=g, device=dev, dtype=torch.int64)
            self.v = torch.rand(self.n, generator=g, device=dev, dtype=torch.float64).mul_(1000)
            self.valid = pack_bits_torch(torch.rand(self.n, generator=g, device=dev) >= 0.05)
            self.cols = [qeg.Col(self.key, None, qeg.I64), qeg.Col(self.v, self.valid, qeg.F64)]
            self.aggs = [(qeg.COUNT_STAR, 0), (qeg.SUM, 1), (qeg.AVG, 1), (qeg.MIN, 1), (qeg.MAX, 1)]
            self.row_bytes = 16.125
        torch.cuda.synchronize()
        self.groups = int(torch.unique(self.key).numel())

    def run(self, qeg, ctx, config, batch_rows=None):
        a = qeg.Aggregate(ctx, [c.type for c in self.cols], [0], self.aggs, config)
        if batch_rows is None:
            a.consume(self.cols)
        else:
            for s in range(0, self.n, batch_rows):
                e = min(self.n, s + batch_rows)
                a.consume([qeg.Col(c.values[s:e], None if c.validity is None else c.validity[s // 64:(e + 63) // 64],
                                   c.type) for c in self.cols])
        n = a.finish()
        st = a.stats()
        a.close()
        return n, st

    def parity(self, qeg, ctx, config):
        """Full-size parity of one GROUP BY run. `skew`: every group's COUNT,
        SUM(I64), MIN and MAX exactly and SUM(F64) within the reference's
        epsilon against a torch reduction (torch.unique + index_add /
        scatter_reduce, no library kernel). `agg1m`: every cell against the
        oracle at the workload's own shape, 2048-row batches (results within
        the reference's comparator, oracle/result_set.cpp:129-187)."""
        import oracle as O

        if self.kind != "skew":
            a = qeg.Aggregate(ctx, [c.type for c in self.cols], [0], self.aggs, config)
            for s in range(0, self.n, 2048):
                e = min(self.n, s + 2048)
                a.consume([qeg.Col(c.values[s:e], None if c.validity is None else c.validity[s // 64:(e + 63) // 64],
                                   c.type) for c in self.cols])
            a.finish()
            got = a.fetch()
            a.close()
            key = self.key.cpu().numpy()
            val = self.v.cpu().numpy()
            valid = unpack_bits_torch(self.valid, self.n).cpu().numpy()
            et, erows = O.groupby([O.TCol(O.I64, key), O.TCol(O.F64, val, valid)], [0], self.aggs, 2048)
            types = [O.I64, O.I64, O.F64, O.F64, O.F64, O.F64]
            rows = list(zip(*[[None if not ok else (float(v) if t == O.F64 else int(v)) for v, ok in zip(vs, va)]
                              for (vs, va), t in zip(got, types)]))
            msg = O.compare(types, rows, et, erows)
            return {"cells_vs_oracle_2048_row_batches": msg is None, "groups": len(erows),
                    "mismatch": msg}
        a = qeg.Aggregate(ctx, [c.type for c in self.cols], [0], self.aggs, config)
        a.consume(self.cols)
        ng = a.finish()
        res = a.fetch_torch()
        ctx.synchronize()
        a.close()
        gkey, order = torch.sort(res[0][0])
        cols = [res[i][0][order] for i in range(1, 6)]
        allvalid = all(bool(unpack_bits_torch(res[i][1], ng).all()) for i in range(6))
        del res
        uniq, inv, cnt = torch.unique(self.key, sorted=True, return_inverse=True, return_counts=True)
        G = uniq.numel()
        s1 = torch.zeros(G, dtype=torch.int64, device=uniq.device).index_add_(0, inv, self.v1)
        s2 = torch.zeros(G, dtype=torch.float64, device=uniq.device).index_add_(0, inv, self.v2)
        mn = torch.full((G,), 1 << 62, dtype=torch.int64, device=uniq.device).scatter_reduce_(0, inv, self.v1, "amin")
        mx = torch.full((G,), -(1 << 62), dtype=torch.int64, device=uniq.device).scatter_reduce_(0, inv, self.v1,
                                                                                                   "amax")
        del inv
        same_keys = ng == G and bool(torch.equal(gkey, uniq))
        out = {"groups": G, "keys_exact": same_keys, "all_valid": allvalid}
        if same_keys:
            out["count_exact"] = bool(torch.equal(cols[0], cnt))
            out["sum_i64_exact"] = bool(torch.equal(cols[1], s1))
            out["sum_f64_mismatches"] = f64_close_torch(cols[2], s2)
            out["min_exact"] = bool(torch.equal(cols[3], mn))
            out["max_exact"] = bool(torch.equal(cols[4], mx))
        out["ok"] = bool(same_keys and allvalid and out["count_exact"] and out["sum_i64_exact"]
                         and out["sum_f64_mismatches"] == 0 and out["min_exact"] and out["max_exact"])
        del uniq, cnt, s1, s2, mn, mx, cols, gkey, order
        torch.cuda.empty_cache()
        return out


def run_agg_bench(args, dev, local, kind=None, emit=True):
    """GROUP BY workload `kind` (skew | agg1m). Returns (and with `emit`
    prints) one JSON object."""
    import qeg

    kind = kind or args.workload
    W = AggWorkload(dev, kind, nrows=args.agg_rows)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    steps = args.steps if emit else min(args.steps, 10)
    warm = args.warmup if emit else max(3, min(args.warmup, 3))
    variants = {
        "learned": qeg.agg_config(sizing=qeg.SIZE_LEARNED, hot_keys=-1),
        "plain_fixed": qeg.agg_config(sizing=qeg.SIZE_FIXED, initial_capacity=1 << 20),
        "exact_size": qeg.agg_config(expected_groups=W.groups, hot_keys=-1),
        # learned sizing held to the private-table strategy (no partitioning)
        "learned_private": qeg.agg_config(strategy=qeg.AGG_SMEM, sizing=qeg.SIZE_LEARNED, hot_keys=-1),
        # learned sizing with the radix-partitioned strategy (opt-in: heavy
        # hitters in the CTA tables, every other row through key-hash
        # partitions aggregated in shared memory)
        "learned_partitioned": qeg.agg_config(strategy=qeg.AGG_PARTITIONED, sizing=qeg.SIZE_LEARNED, hot_keys=-1),
    }
    if kind == "agg1m":
        del variants["learned_private"]
        del variants["learned_partitioned"]
    if args.variants:
        variants = {k: v for k, v in variants.items() if k in args.variants.split(",")}
    out = {}
    clk = ClockSampler(local).__enter__()
    tw0 = time.time()
    for name, cfg in variants.items():
        for _ in range(warm):
            W.run(qeg, ctx, cfg)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = ctx.launches
        e0.record(stream)
        for _ in range(steps):
            n, st = W.run(qeg, ctx, cfg)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        assert n == W.groups, (name, n, W.groups)
        out[name] = {"ms_per_step": ms, "rows_per_s": W.n / (ms / 1e3), "groups": n, "stats": st,
                     "gb_per_s": W.n * W.row_bytes / (ms / 1e3) / 1e9,
                     "launches_per_step": (ctx.launches - launches0) / steps}
    if kind == "agg1m":
        # The workload's own batching: 2048-row batches through consume().
        cfg = next(iter(variants.values()))
        W.run(qeg, ctx, cfg, batch_rows=2048)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            W.run(qeg, ctx, cfg, batch_rows=2048)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        out["batches_2048"] = {"ms_per_step": ms, "rows_per_s": W.n / (ms / 1e3)}
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    parity = W.parity(qeg, ctx, variants[next(iter(variants))])
    ok = parity.get("ok", parity.get("cells_vs_oracle_2048_row_batches"))
    assert ok, parity
    cpu = None
    if not args.no_cpu:
        cpu = cpu_agg_baseline(W, os.cpu_count() or 1)
    peak, pkind = peaks()
    best = out["learned"] if "learned" in out else next(iter(out.values()))
    line = {
        "metric": "rows/s hash aggregate (%s)" % W.name, "value": best["rows_per_s"], "unit": "rows/s",
        "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": best["ms_per_step"],
        "higher_is_better": True, "dtype": "int64+f64", "data": "synthetic (seeded, generated on the GPU)",
        "config": {"workload": W.name, "rows": W.n, "groups": W.groups, "seed": W.seed, "M": "2^20",
                   "l2": "inputs exceed L2, no flush" if W.n * W.row_bytes > 2e8 else
                   "inputs fit L2 (a correctness-sized workload)"},
        "roofline": {"bound": "hbm", "achieved": best["gb_per_s"], "peak": peak, "peak_kind": pkind,
                     "unit": "GB/s", "frac": best["gb_per_s"] / peak,
                     "algorithmic_bytes_per_row": W.row_bytes},
        "variants": out,
        "full_size_parity": parity,
        "cpu_baseline": cpu,
        "gpu_launches": out[next(iter(out))]["launches_per_step"] if out else None,
        "clocks": clocks,
        "learned_vs_plain": (out["plain_fixed"]["ms_per_step"] / best["ms_per_step"]
                             if "plain_fixed" in out else None),
    }
    ctx.close()
    del W
    torch.cuda.empty_cache()
    if emit:
        print(json.dumps(line))
    return line


# ---------------------------------------------------------------------------
# Workload: 4096 independent GROUP BY queries in one batch
# ---------------------------------------------------------------------------
class BatchWorkload:
    """`batch` = 4096 GROUP BY queries over back-to-back slices: per-query row
    counts log-uniform in [1e3, 1e7]; int32 keys with a distinct-value domain
    log-uniform in [4, 1e6], half uniform and half Zipf(s), s uniform in
    [0.5, 1.5]; F64 values uniform [0, 1); COUNT(*), SUM, AVG, MIN, MAX grouped
    by key. Ranks are spread over int32 by an odd-multiplier bijection."""

    name = "batch_4096q_loguniform_1e3_1e7"

    def __init__(self, dev, nq=4096, lo=1e3, hi=1e7, seed=SEED + 4):
        import qeg

        rng = np.random.default_rng(seed)
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), nq)).astype(np.int64)
        doms = np.exp(rng.uniform(np.log(4), np.log(1e6), nq)).astype(np.int64)
        zipf = rng.random(nq) < 0.5
        ss = rng.uniform(0.5, 1.5, nq)
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
        self.n = int(self.offsets[-1])
        self.key = torch.empty(self.n, dtype=torch.int32, device=dev)
        self.val = torch.rand(self.n, generator=g, device=dev, dtype=torch.float64)
        for q in range(nq):
            a, b, d = int(self.offsets[q]), int(self.offsets[q + 1]), int(doms[q])
            if zipf[q]:
                cdf = torch.arange(1, d + 1, dtype=torch.float64, device=dev).pow_(-float(ss[q])).cumsum_(0)
                cdf /= cdf[-1].clone()
                r = torch.searchsorted(cdf, torch.rand(b - a, generator=g, device=dev, dtype=torch.float64))
                r.clamp_(max=d - 1)
            else:
                r = torch.randint(0, d, (b - a,), generator=g, device=dev, dtype=torch.int64)
            x = (r * 2654435761 + 12345 * q) & 0xFFFFFFFF
            self.key[a:b] = torch.where(x >= (1 << 31), x - (1 << 32), x).to(torch.int32)
        torch.cuda.synchronize()
        self.meta = {"sizes": sizes, "domains": doms, "zipf": zipf, "s": ss}
        self.aggs = [(qeg.COUNT_STAR, 0), (qeg.SUM, 1), (qeg.AVG, 1), (qeg.MIN, 1), (qeg.MAX, 1)]
        self.row_bytes = 12

    def cols(self):
        import qeg

        return qeg.Col(self.key, None, qeg.I32), qeg.Col(self.val, None, qeg.F64)


# ---------------------------------------------------------------------------
# Workload: filter -> join -> GROUP BY over dictionary strings
# ---------------------------------------------------------------------------
class PipelineWorkload:
    """`pipeline` = trades of 200M rows (sym: STR dictionary codes over 10k
    symbols, Zipf(1.0); price: F64 lognormal(4.6, 0.3); qty: I32 uniform
    [1, 10000]) filtered on price > 100, inner-joined by symbol VALUE with a
    10k-row symbol table under its own dictionary order (sector: I32 uniform
    over 32), grouped by sector: COUNT(*), AVG(price), SUM(qty)."""

    name = "pipeline_trades200M_sym10k_sector32"

    def __init__(self, dev, n=200_000_000, nsym=10_000, seed=SEED + 5):
        import qeg

        rng = np.random.default_rng(seed)
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.n = n
        names = ["SYM%05d" % i for i in range(nsym)]
        tperm = rng.permutation(nsym)  # trades dictionary: code c holds names[tperm[c]]
        bperm = rng.permutation(nsym)  # symbol table dictionary
        # Canonical value id of a name = its index in `names`.
        self.tmap = torch.from_numpy(tperm.astype(np.int32)).to(dev)
        self.bmap = torch.from_numpy(bperm.astype(np.int32)).to(dev)
        inv_t = np.argsort(tperm)  # name index -> trades code
        cdf = torch.arange(1, nsym + 1, dtype=torch.float64, device=dev).pow_(-1.0).cumsum_(0)
        cdf /= cdf[-1].clone()
        self.sym = torch.empty(n, dtype=torch.int32, device=dev)
        code_of = torch.from_numpy(inv_t.astype(np.int32)).to(dev)
        for a in range(0, n, 1 << 26):
            b = min(n, a + (1 << 26))
            r = torch.searchsorted(cdf, torch.rand(b - a, generator=g, device=dev, dtype=torch.float64))
            self.sym[a:b] = code_of[r.clamp_(max=nsym - 1)]
        self.price = torch.randn(n, generator=g, device=dev, dtype=torch.float64).mul_(0.3).add_(4.6).exp_()
        self.qty = torch.randint(1, 10001, (n,), generator=g, device=dev, dtype=torch.int32)
        self.bsym = torch.arange(nsym, dtype=torch.int32, device=dev)  # symbol table row i = code i
        self.sector = torch.randint(0, 32, (nsym,), generator=g, device=dev, dtype=torch.int32)
        torch.cuda.synchronize()
        self.aggs = [(qeg.COUNT_STAR, 0), (qeg.AVG, 1), (qeg.SUM, 2)]
        self.row_bytes = 16

    def cols(self, host=None):
        import qeg

        src = host or self
        probe = [qeg.Col(src.sym, None, qeg.STR, src.tmap), qeg.Col(src.price, None, qeg.F64),
                 qeg.Col(src.qty, None, qeg.I32)]
        build = [qeg.Col(src.bsym, None, qeg.STR, src.bmap), qeg.Col(src.sector, None, qeg.I32)]
        return probe, build

    def run(self, qeg, ctx, host=None):
        probe, build = self.cols(host)
        return qeg.filter_join_agg(ctx, probe, build, 0, 0, 4, self.aggs, filter_col=1, filter_op=qeg.CMP_GT,
                                   filter_value=100.0, capacity=64)

    def host_copy(self):
        class H:
            pass

        h = H()
        for k in ("sym", "price", "qty", "bsym", "sector", "tmap", "bmap"):
            setattr(h, k, getattr(self, k).cpu().pin_memory())
        return h


def pipeline_parity_torch(W, res):
    """Every sector's COUNT(*) and SUM(qty) exactly and AVG(price) within the
    reference's epsilon, against torch alone: the filter as a mask, each
    trade's sector through the symbol VALUE (code -> canonical id -> symbol
    row), bincount / index_add per sector."""
    keep = W.price > 100
    row_of_id = torch.argsort(W.bmap)  # canonical id -> symbol-table row
    sec = W.sector[row_of_id[W.tmap[W.sym.long()].long()]].long()[keep]
    cnt = torch.bincount(sec, minlength=32)
    sq = torch.zeros(32, dtype=torch.int64, device=sec.device).index_add_(0, sec, W.qty[keep].long())
    sp = torch.zeros(32, dtype=torch.float64, device=sec.device).index_add_(0, sec, W.price[keep])
    present = cnt > 0
    gkey = torch.as_tensor(np.asarray(res[0][0]), device=sec.device).long()
    order = torch.argsort(gkey)
    gkey = gkey[order]
    gcnt = torch.as_tensor(np.asarray(res[1][0]), device=sec.device)[order]
    gavg = torch.as_tensor(np.asarray(res[2][0]), device=sec.device)[order]
    gsum = torch.as_tensor(np.asarray(res[3][0]), device=sec.device)[order]
    want = torch.nonzero(present).flatten()
    same = bool(torch.equal(gkey, want))
    out = {"sectors": int(present.sum()), "keys_exact": same}
    if same:
        out["count_exact"] = bool(torch.equal(gcnt.long(), cnt[want]))
        out["sum_qty_exact"] = bool(torch.equal(gsum.long(), sq[want]))
        out["avg_price_mismatches"] = f64_close_torch(gavg.double(), sp[want] / cnt[want].double())
    out["ok"] = bool(same and out["count_exact"] and out["sum_qty_exact"] and out["avg_price_mismatches"] == 0)
    return out


def run_pipeline_bench(args, dev, local, emit=True):
    import qeg

    W = PipelineWorkload(dev)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    steps = args.steps if emit else min(args.steps, 10)
    warm = args.warmup if emit else max(3, min(args.warmup, 3))
    for _ in range(max(warm, 0)):
        types, res = W.run(qeg, ctx)
    clk = ClockSampler(local).__enter__()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launches
    tw0 = time.time()
    e0.record(stream)
    for _ in range(steps):
        types, res = W.run(qeg, ctx)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    ms = e0.elapsed_time(e1) / steps
    launches = (ctx.launches - launches0) / steps
    parity = pipeline_parity_torch(W, res)
    assert parity["ok"], parity
    e2e = None
    if not args.no_e2e:
        host = W.host_copy()
        W.run(qeg, ctx, host=host)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            W.run(qeg, ctx, host=host)
        e2e_s = (time.perf_counter() - t0) / 3
        h2d = W.n * W.row_bytes + 10_000 * 8 + 10_000 * 4 * 2
        e2e = {"value": W.n / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 64 * 8 * 4}
    rows_s = W.n / (ms / 1e3)
    gbs = W.n * W.row_bytes / (ms / 1e3) / 1e9
    peak, kind = peaks()
    line = {
        "metric": "rows/s fused filter->join->aggregate (%s)" % W.name, "value": rows_s, "unit": "rows/s",
        "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
        "data": "synthetic (seeded, generated on the GPU); inputs 3.2 GB > L2",
        "config": {"workload": W.name, "rows": W.n, "groups": parity["sectors"], "seed": SEED + 5},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_kind": kind, "note": "whole call (translation tables, kernel, result copy)"},
        "full_size_parity": parity,
        "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
    }
    ctx.close()
    del W
    torch.cuda.empty_cache()
    if emit:
        print(json.dumps(line))
    return line


class TickWorkload:
    """Tick data for the time-series callers of the hash table: `trades`
    (n rows: sym I32 over 10k symbols, Zipf(1.0); ts TS nanoseconds over one
    6.5 h session, non-decreasing; price F64 lognormal(4.6, 0.3); qty I32
    uniform [1, 10000]) and `quotes` (m rows: sym, ts alike; bid F64; ask F64).
    `window` = GROUP BY (sym, 1-minute bucket of ts): COUNT(*), SUM(qty),
    MIN(price), MAX(price), AVG(price). `asof` = trades LEFT as-of join quotes
    on sym by ts (the quote in force at each trade), all columns out."""

    SESSION_NS = 23_400 * 10 ** 9
    T0 = 1_700_000_000 * 10 ** 9

    def __init__(self, dev, n=200_000_000, m=50_000_000, nsym=10_000, seed=SEED + 7):
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.n, self.m, self.nsym = n, m, nsym
        cdf = torch.arange(1, nsym + 1, dtype=torch.float64).pow_(-1.0).cumsum_(0)
        cdf = (cdf / cdf[-1]).to(dev)

        def side(rows):
            sym = torch.empty(rows, dtype=torch.int32, device=dev)
            ts = torch.empty(rows, dtype=torch.int64, device=dev)
            step = self.SESSION_NS // rows
            for a in range(0, rows, 1 << 26):
                b = min(rows, a + (1 << 26))
                r = torch.searchsorted(cdf, torch.rand(b - a, generator=g, device=dev, dtype=torch.float64))
                sym[a:b] = r.clamp_(max=nsym - 1).to(torch.int32)
                i = torch.arange(a, b, device=dev, dtype=torch.int64)
                ts[a:b] = self.T0 + i * step + torch.randint(0, step, (b - a,), generator=g, device=dev)
            return sym, ts

        self.sym, self.ts = side(n)
        self.price = torch.randn(n, generator=g, device=dev, dtype=torch.float64).mul_(0.3).add_(4.6).exp_()
        self.qty = torch.randint(1, 10001, (n,), generator=g, device=dev, dtype=torch.int32)
        self.qsym, self.qts = side(m)
        self.bid = torch.randn(m, generator=g, device=dev, dtype=torch.float64).mul_(0.3).add_(4.6).exp_()
        self.ask = self.bid + torch.rand(m, generator=g, device=dev, dtype=torch.float64).mul_(0.05)
        torch.cuda.synchronize()
        self.trade_bytes = 4 + 8 + 8 + 4
        self.quote_bytes = 4 + 8 + 8 + 8

    def trades(self, qeg, src=None):
        src = src or self
        return [qeg.Col(src.sym, None, qeg.I32), qeg.Col(src.ts, None, qeg.TS), qeg.Col(src.price, None, qeg.F64),
                qeg.Col(src.qty, None, qeg.I32)]

    def quotes(self, qeg, src=None):
        src = src or self
        return [qeg.Col(src.qsym, None, qeg.I32), qeg.Col(src.qts, None, qeg.TS), qeg.Col(src.bid, None, qeg.F64),
                qeg.Col(src.ask, None, qeg.F64)]


WINDOW_NS = 60 * 10 ** 9


def run_window_bench(args, dev, local):
    import qeg
    import oracle as O

    W = TickWorkload(dev, n=args.ticks, m=args.ticks // 4)
    name = "window_trades%dM_sym10k_1min" % (W.n // 1_000_000)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    aggs = [(qeg.COUNT_STAR, 0), (qeg.SUM, 3), (qeg.MIN, 2), (qeg.MAX, 2), (qeg.AVG, 2)]
    types = [qeg.I32, qeg.TS, qeg.F64, qeg.I32]

    def step(src=None):
        w = qeg.Window(ctx, types, [0], 1, WINDOW_NS, aggs)
        w.consume(W.trades(qeg, src))
        ng = w.finish()
        return w, ng

    for _ in range(max(args.warmup, 0)):
        w, ng = step()
        w.close()
    clk = ClockSampler(local).__enter__()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launches
    tw0 = time.time()
    e0.record(stream)
    for k in range(args.steps):
        w, ng = step()
        if k + 1 < args.steps:
            w.close()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    ms = e0.elapsed_time(e1) / args.steps
    launches = (ctx.launches - launches0) / args.steps
    stats = w.stats()
    # Check: the group count and the COUNT/SUM totals against torch.
    minute = torch.div(W.ts, WINDOW_NS, rounding_mode="trunc")
    pair = (W.sym.to(torch.int64) << 40) | (minute - minute.min())
    true_groups = int(torch.unique(pair).numel())
    del pair, minute
    res = w.fetch_torch()
    assert ng == true_groups, (ng, true_groups)
    assert int(res[2][0].sum()) == W.n and int(res[3][0].sum()) == int(W.qty.sum(dtype=torch.int64))
    w.close()
    e2e = None
    if not args.no_e2e:
        host = type("H", (), {})()
        for a in ("sym", "ts", "price", "qty"):
            setattr(host, a, getattr(W, a).cpu().pin_memory())
        hw, _ = step(host)
        out = hw.fetch_pinned()  # page-locked result buffers, reused by the timed steps
        hw.close()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            hw, ngr = step(host)
            out = hw.fetch_pinned(bufs=out)
            hw.close()
        e2e_s = (time.perf_counter() - t0) / 2
        e2e = {"value": W.n / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": W.n * W.trade_bytes,
               "d2h_bytes_per_step": int(sum(ngr * v.element_size() + (ngr + 63) // 64 * 8 for v, _ in out))}
    cpu = None
    if not args.no_cpu:
        k = 1 << 23
        cols = [O.TCol(O.I32, W.sym[:k].cpu().numpy()), O.TCol(O.TS, W.ts[:k].cpu().numpy()),
                O.TCol(O.F64, W.price[:k].cpu().numpy()), O.TCol(O.I32, W.qty[:k].cpu().numpy())]
        t0 = time.perf_counter()
        O.window_tumbling(cols, [0], 1, WINDOW_NS, aggs)
        dt = time.perf_counter() - t0
        cpu = {"value": k / dt, "unit": "rows/s", "cores": 1, "kind": "port",
               "sample": "first %d trades (%.1f s), the Window operator is single-threaded" % (k, dt)}
    gbs = W.n * W.trade_bytes / (ms / 1e3) / 1e9
    peak, kind = peaks()
    print(json.dumps({
        "metric": "rows/s tumbling window (%s)" % name, "value": W.n / (ms / 1e3), "unit": "rows/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+int64+f64",
        "data": "synthetic (seeded, generated on the GPU); inputs %.1f GB > L2" % (W.n * W.trade_bytes / 1e9),
        "config": {"workload": name, "rows": W.n, "groups": ng, "width_ns": WINDOW_NS, "stats": stats,
                   "seed": SEED + 7},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_kind": kind, "note": "24 B per trade row read once; whole call"},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clocks,
    }))


def run_asof_bench(args, dev, local):
    import qeg
    import oracle as O

    W = TickWorkload(dev, n=args.ticks, m=args.ticks // 4)
    name = "asof_trades%dM_quotes%dM_sym10k" % (W.n // 1_000_000, W.m // 1_000_000)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    ptypes = [qeg.I32, qeg.TS, qeg.F64, qeg.I32]
    btypes = [qeg.I32, qeg.TS, qeg.F64, qeg.F64]
    bufs = [None]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def step(timed=False):
        j = qeg.AsofJoin(ctx, ptypes, btypes, [0], [0], 1, 1, qeg.LEFT)
        if timed:
            ev[0].record(stream)
        j.build(W.quotes(qeg))
        j.build_finish()
        if timed:
            ev[1].record(stream)
        n = j.probe(W.trades(qeg))
        if timed:
            ev[2].record(stream)
        bufs[0] = j.fetch_device(0, n, bufs[0])
        if timed:
            ev[3].record(stream)
        j.close()
        return n

    for _ in range(max(args.warmup, 0)):
        n = step()
    clk = ClockSampler(local).__enter__()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launches
    tw0 = time.time()
    e0.record(stream)
    for k in range(args.steps):
        n = step(timed=(k == args.steps - 1))
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    ms = e0.elapsed_time(e1) / args.steps
    launches = (ctx.launches - launches0) / args.steps
    rows = W.n + W.m
    phases = {"build_sort_ms": ev[0].elapsed_time(ev[1]), "probe_ms": ev[1].elapsed_time(ev[2]),
              "fetch_ms": ev[2].elapsed_time(ev[3])}
    # Check every output row against torch: quotes sorted stably by (sym, ts),
    # the last one at or before each trade's time within its symbol.
    assert n == W.n
    span = int(W.SESSION_NS).bit_length() + 1
    qkey = (W.qsym.to(torch.int64) << span) | (W.qts - W.T0)
    qsorted, qorder = torch.sort(qkey, stable=True)
    tkey = (W.sym.to(torch.int64) << span) | (W.ts - W.T0)
    pos = torch.searchsorted(qsorted, tkey, right=True) - 1
    okp = pos >= 0
    cand = qorder[pos.clamp(min=0)]
    okp &= W.qsym[cand] == W.sym
    out_ts, out_bid = bufs[0][5][0][:n], bufs[0][6][0][:n]
    words = bufs[0][5][1]
    valid = ((words.view(torch.uint8).unsqueeze(1) >> torch.arange(8, device=dev, dtype=torch.uint8)) & 1)
    valid = valid.flatten()[:n].bool()
    assert bool((valid == okp).all()), "as-of matches differ from the torch check"
    assert bool((out_ts[okp] == W.qts[cand[okp]]).all()) and bool((out_bid[okp] == W.bid[cand[okp]]).all())
    matched = int(okp.sum())
    del qkey, qsorted, qorder, tkey, pos, cand, okp, valid
    e2e = None
    if not args.no_e2e:
        # Host-resident trades and quotes (page-locked), all 8 output columns
        # back into page-locked host buffers reused across steps.
        host = type("H", (), {})()
        for a in ("sym", "ts", "price", "qty", "qsym", "qts", "bid", "ask"):
            setattr(host, a, getattr(W, a).cpu().pin_memory())

        def host_step(out, tm=None):
            t = [time.perf_counter()]
            j = qeg.AsofJoin(ctx, ptypes, btypes, [0], [0], 1, 1, qeg.LEFT)
            j.build(W.quotes(qeg, host))
            j.build_finish()
            if tm is not None:
                ctx.synchronize()
                t.append(time.perf_counter())
            nh = j.probe(W.trades(qeg, host))
            if tm is not None:
                ctx.synchronize()
                t.append(time.perf_counter())
            out = j.fetch_pinned(0, nh, out)
            j.close()
            if tm is not None:
                t.append(time.perf_counter())
                tm.update({k: round((t[i + 1] - t[i]) * 1e3, 2) for i, k in
                           enumerate(("build_ms", "probe_ms", "fetch_ms"))})
            return nh, out

        nh, out = host_step(None)
        nh, out = host_step(out)  # the memory pool has grown to the host path's staging buffers
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            nh, out = host_step(out)
        e2e_s = (time.perf_counter() - t0) / 3
        e2e_phases = {}
        host_step(out, e2e_phases)  # one more, synchronised between phases
        nw = (nh + 63) // 64
        assert nh == W.n and torch.equal(out[5][1][:nw], bufs[0][5][1][:nw].cpu())
        hv = ((out[5][1][:nw].view(torch.uint8).unsqueeze(1) >> torch.arange(8, dtype=torch.uint8)) & 1)
        hv = hv.flatten()[:nh].bool()
        assert torch.equal(out[5][0][:nh][hv], bufs[0][5][0][:n].cpu()[hv]), "host fetch differs from device fetch"
        e2e = {"value": rows / e2e_s, "unit": "rows/s",
               "h2d_bytes_per_step": W.n * W.trade_bytes + W.m * W.quote_bytes,
               "d2h_bytes_per_step": int(sum(nh * v.element_size() + (nh + 63) // 64 * 8 for v, _ in out)),
               "phases": e2e_phases}
        del host, out
    cpu = None
    if not args.no_cpu:
        k, kq = 1 << 22, 1 << 20
        probe = [O.TCol(O.I32, W.sym[:k].cpu().numpy()), O.TCol(O.TS, W.ts[:k].cpu().numpy()),
                 O.TCol(O.F64, W.price[:k].cpu().numpy()), O.TCol(O.I32, W.qty[:k].cpu().numpy())]
        build = [O.TCol(O.I32, W.qsym[:kq].cpu().numpy()), O.TCol(O.TS, W.qts[:kq].cpu().numpy()),
                 O.TCol(O.F64, W.bid[:kq].cpu().numpy()), O.TCol(O.F64, W.ask[:kq].cpu().numpy())]
        t0 = time.perf_counter()
        O.asof_join(probe, build, [0], [0], 1, 1, O.LEFT)
        dt = time.perf_counter() - t0
        cpu = {"value": (k + kq) / dt, "unit": "rows/s", "cores": 1, "kind": "port",
               "sample": "first %d trades x first %d quotes (the same time prefix, %.1f s); the AsofJoin "
                         "operator is single-threaded" % (k, kq, dt)}
    alg = W.n * W.trade_bytes + W.m * W.quote_bytes + W.n * (W.trade_bytes + W.quote_bytes + 8 / 8)
    gbs = alg / (ms / 1e3) / 1e9
    peak, kind = peaks()
    print(json.dumps({
        "metric": "rows/s as-of join (%s)" % name, "value": rows / (ms / 1e3), "unit": "rows/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+int64+f64",
        "data": "synthetic (seeded, generated on the GPU); inputs %.1f GB > L2"
                % ((W.n * W.trade_bytes + W.m * W.quote_bytes) / 1e9),
        "config": {"workload": name, "trades": W.n, "quotes": W.m, "matched": matched, "phases": phases,
                   "seed": SEED + 7,
                   "output": "all 8 columns gathered into HBM buffers"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_kind": kind,
                     "note": "inputs read once + output (52 B/row + validity) written once; whole step"},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clocks,
    }))


def load_tuning():
    path = os.path.join(REPO, "query-engine_gb300", "batch_tuning.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return [tuple(t) for t in d["tuning"]], int(d.get("block_threads", 0)), path
    except Exception:
        return [], 0, None


def batch_parity_oracle(W, b, groups, stats, nrandom=16, seed=SEED + 44):
    """Every cell of a fixed sample of the batch's queries against the oracle
    (the restatement of the reference's GROUP BY, oracle/result_set.cpp:129-187
    comparator): the 8 largest queries, every query that overflowed its table
    and was re-run, and `nrandom` seeded random ones."""
    import oracle as O

    nq = len(groups)
    sizes = np.diff(W.offsets.astype(np.int64))
    fell = [q for q in range(nq) if stats[q]["fell_back"]]
    largest = [int(q) for q in np.argsort(-sizes, kind="stable")[:8]]
    rng = np.random.default_rng(seed)
    rand = [int(q) for q in rng.choice(nq, nrandom, replace=False)]
    sample = sorted(set(largest + fell + rand))
    types = [O.I32, O.I64, O.F64, O.F64, O.F64, O.F64]
    bad = []
    rows_checked = 0
    for q in sample:
        a, z = int(W.offsets[q]), int(W.offsets[q + 1])
        et, erows = O.groupby([O.TCol(O.I32, W.key[a:z].cpu().numpy()), O.TCol(O.F64, W.val[a:z].cpu().numpy())],
                              [0], W.aggs)
        got = b.fetch(q)
        rows = list(zip(*[[None if not ok else (float(v) if t == O.F64 else int(v)) for v, ok in zip(vs, va)]
                          for (vs, va), t in zip(got, types)]))
        msg = O.compare(types, rows, et, erows)
        rows_checked += z - a
        if msg or int(groups[q]) != len(erows):
            bad.append((q, msg))
    return {"queries_vs_oracle": len(sample), "largest": largest, "overflowed": fell, "rows_checked": rows_checked,
            "mismatches": bad, "ok": not bad}


def run_batch_bench(args, dev, local, emit=True):
    import qeg

    W = BatchWorkload(dev)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    steps = args.steps if emit else min(args.steps, 10)
    warm = args.warmup if emit else max(3, min(args.warmup, 3))
    tuning, block, tpath = load_tuning()
    k, v = W.cols()
    t0 = time.perf_counter()
    b = qeg.Batch(ctx, W.offsets, k, v, W.aggs, tuning=tuning, block_threads=block)
    ctx.synchronize()
    plan_s = time.perf_counter() - t0
    for _ in range(max(warm, 0)):
        b.run()
        groups = b.finish()
    clk = ClockSampler(local).__enter__()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launches
    tw0 = time.time()
    e0.record(stream)
    for _ in range(steps):
        b.run()
        groups = b.finish()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    ms = e0.elapsed_time(e1) / steps
    launches = (ctx.launches - launches0) / steps
    stats = [b.stats(q) for q in range(len(groups))]
    fell = sum(st["fell_back"] for st in stats)
    # Exact group counts (torch.unique per query) for the estimate report.
    true = np.array([int(torch.unique(W.key[int(W.offsets[q]):int(W.offsets[q + 1])]).numel())
                     for q in range(len(groups))])
    parity = {"group_counts_vs_torch_unique": bool(np.array_equal(true, groups.astype(np.int64)))}
    parity.update(batch_parity_oracle(W, b, groups, stats))
    parity["ok"] = parity["ok"] and parity["group_counts_vs_torch_unique"]
    assert parity["ok"], parity
    est = np.array([st["est_groups"] for st in stats])
    fb = [q for q in range(len(groups)) if stats[q]["fell_back"]]
    fell_ratio = sorted(float(true[q] / max(est[q], 1.0)) for q in fb)
    lerr = np.abs(np.log2(np.maximum(est, 1)) - np.log2(np.maximum(true, 1)))
    b.close()
    rows_s = W.n / (ms / 1e3)
    gbs = W.n * W.row_bytes / (ms / 1e3) / 1e9

    # The plain GPU path: the same queries one at a time through the ordinary
    # GROUP BY with fixed initial sizing (grow on overflow).
    plain = None
    if not args.no_plain:
        nq = len(groups)
        cfg = qeg.agg_config(sizing=qeg.SIZE_FIXED)
        offs = W.offsets

        def plain_step():
            for q in range(nq):
                a, z = int(offs[q]), int(offs[q + 1])
                ag = qeg.Aggregate(ctx, [qeg.I32, qeg.F64], [0], W.aggs, cfg)
                ag.consume([qeg.Col(W.key[a:z], None, qeg.I32), qeg.Col(W.val[a:z], None, qeg.F64)])
                ag.finish()
                ag.close()

        plain_step()
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        plain_step()
        ctx.synchronize()
        pms = (time.perf_counter() - p0) * 1e3
        plain = {"ms_per_step": pms, "rows_per_s": W.n / (pms / 1e3)}
    peak, kind = peaks()
    line = {
        "metric": "rows/s batched hash aggregate (%s)" % W.name, "value": rows_s, "unit": "rows/s",
        "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
        "data": "synthetic (seeded, generated on the GPU); inputs %.1f GB > L2" % (W.n * W.row_bytes / 1e9),
        "config": {"workload": W.name, "queries": len(groups), "rows": W.n, "seed": SEED + 4,
                   "tuning": os.path.relpath(tpath, REPO) if tpath else None,
                   "block_threads": block or 512},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_kind": kind, "note": "graph replay (aggregate + finalize) time, 12 B per row"},
        "full_size_parity": parity,
        "gpu_launches": launches, "clocks": clocks, "plan_s": plan_s,
        "estimate_log2_error": {"median": float(np.median(lerr)), "p90": float(np.percentile(lerr, 90))},
        "fell_back_queries": int(fell),
        "fell_back_true_over_est": {"min": fell_ratio[0] if fell_ratio else None,
                                    "median": fell_ratio[len(fell_ratio) // 2] if fell_ratio else None,
                                    "max": fell_ratio[-1] if fell_ratio else None},
        "plain_sequential": plain,
        "batched_vs_plain": (plain["ms_per_step"] / ms) if plain else None,
    }
    ctx.close()
    del W
    torch.cuda.empty_cache()
    if emit:
        print(json.dumps(line))
    return line


def operator_bench(timeout=600):
    """The drop-in operators through the reference's pull interface
    (Operator::open/next/close over a Scan of 2048-row host batches, output
    drained on the host): the 1M-row plain GROUP BY through GpuAggregate and
    the 16M x 256M join through GpuHashJoin; then the same two over GpuScans
    of DeviceTables uploaded once (columns read in place). Runs the C++ driver
    query-engine_gb300/host/bench_operators.cpp (built by the package build)."""
    import qeg  # noqa: F401  (loads libqeg.so first)
    import build as qbuild

    exe = qbuild.build_operator_bench()
    out = {}
    for name, argv in (("agg", ["agg", str(1 << 20), "5"]),
                       ("join", ["join", str(1 << 24), str(1 << 28), "2"]),
                       ("agg_resident", ["agg_resident", str(1 << 20), "5"]),
                       ("join_resident", ["join_resident", str(1 << 24), str(1 << 28), "2"])):
        r = subprocess.run([exe] + argv, capture_output=True, text=True, timeout=timeout)
        try:
            out[name] = json.loads(r.stdout.strip().splitlines()[-1])
        except Exception:
            out[name] = {"error": (r.stdout + r.stderr)[-500:], "rc": r.returncode}
    return out


def cpu_agg_baseline(W, threads, sample_rows=1 << 23):
    """Times the oracle's port of the reference's morsel-parallel GROUP BY
    (exec/parallel.cpp:402-599, per-worker partial tables and a serial merge)
    on the first `sample_rows` rows of the workload with every host thread."""
    import oracle as O

    n = min(W.n, sample_rows)
    cols = []
    for c in W.cols:
        vals = c.values[:n].cpu().numpy()
        valid = None
        if c.validity is not None:
            valid = np.unpackbits(c.validity[: (n + 63) // 64].cpu().numpy().view(np.uint8),
                                  bitorder="little")[:n].astype(bool)
        cols.append(O.TCol(c.type, vals, valid))
    morsel = max(1024, -(-n // (threads * 4)) // 64 * 64)
    t0 = time.perf_counter()
    O.parallel_groupby(cols, [0], W.aggs, threads=threads, morsel_rows=morsel)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "rows/s", "cores": threads, "kind": "port",
            "sample": "first %d rows (%.1f s), morsels of %d rows" % (n, dt, morsel)}


def cpu_reference(sample, threads, probe_rows, nbuild):
    """Times the oracle's port of the reference's morsel-parallel engine
    (exec/parallel.cpp:374-599) on the given probe rows: each morsel's private
    tree rebuilds the whole build side (exec/parallel.cpp:101-105), so morsels
    are sized to one per thread. Returns (rows/s, seconds, (count, sum))."""
    import oracle as O

    pk, pv, bk, bv = sample
    morsel = -(-probe_rows // threads)
    morsel = -(-morsel // 64) * 64
    t0 = time.perf_counter()
    res = O.parallel_join_count_sum(pk, pv, bk, bv, threads=threads, morsel_rows=morsel)
    dt = time.perf_counter() - t0
    return (nbuild + probe_rows) / dt, dt, res


def run_join_bench(args, dev, local, world, rank, threads, sparse=False, sub=False, cpu_later=None):
    """The join workload: one step = build + probe through the COUNT/SUM sink.
    Returns the JSON object (rank 0) with roofline, e2e, CPU baseline and the
    full-size parity check. `sub` = a secondary line: fewer steps, no CPU arms.
    With `cpu_later` (a list), the CPU baseline is not run here: a function
    that runs it and completes the returned object is appended instead, so a
    caller can time its GPU workloads first."""
    import qeg

    strat = {"auto": qeg.JOIN_AUTO, "hash": qeg.JOIN_HASH, "dense": qeg.JOIN_DENSE,
             "partitioned": qeg.JOIN_PARTITIONED}[args.strategy]
    steps = min(args.steps, 10) if sub else args.steps
    warm = max(3, min(args.warmup, 3)) if sub else args.warmup
    W = JoinWorkload(dev, args.build_rows, args.probe_rows, sparse=sparse)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    step_ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    clk = ClockSampler(local).__enter__()
    for _ in range(max(warm, 0)):
        res, st = W.run(qeg, ctx, strat)
    torch.cuda.synchronize()
    ctx.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    phase_ev = []
    barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    tw0 = time.time()
    step_ev[0].record(stream)
    t0 = time.perf_counter()
    for _ in range(steps):
        pe = [torch.cuda.Event(enable_timing=True) for _ in range(3)] + [stream]
        res, st = W.run(qeg, ctx, strat, events=pe)
        phase_ev.append(pe)
    step_ev[1].record(stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    barrier()
    launches = ctx.launches - launches0
    total_ms, value = replica_throughput(step_ev[0].elapsed_time(step_ev[1]), W.rows(), steps, world, dev)
    build_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in phase_ev]))
    probe_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in phase_ev]))
    ms_per_step = total_ms / steps
    peak, peak_kind = peaks()
    achieved = W.algorithmic_probe_bytes() / (probe_ms / 1e3) / 1e9
    strategy_name = {1: "hash", 2: "partitioned", 3: "dense"}.get(st["strategy"], str(st["strategy"]))

    # Full-size parity: the result against torch alone (no library kernel).
    exp = W.expected_torch()
    parity = {"count_sum_vs_torch": res == exp, "expected": {"count": exp[0], "sum": exp[1]}}

    e2e = None
    if not args.no_e2e:
        host = W.host_copy()
        W.run(qeg, ctx, strat, host=host)
        torch.cuda.synchronize()
        # Each step timed on its own (the result read back ends it); the
        # median is reported with every step's time: the host link is shared
        # with the machine's other work.
        n_e2e = 3 if sub else max(5, min(args.steps, 10))
        step_s = []
        for _ in range(n_e2e):
            t1 = time.perf_counter()
            r2, _ = W.run(qeg, ctx, strat, host=host)
            step_s.append(time.perf_counter() - t1)
            assert r2 == res
        dt = float(np.median(step_s))
        e2e = {"value": W.rows() / dt, "unit": "rows/s", "h2d_bytes_per_step": W.h2d_bytes(),
               "d2h_bytes_per_step": 24, "steps": n_e2e, "stat": "median of per-step times",
               "step_ms": [round(x * 1e3, 2) for x in step_s],
               "min_ms": round(min(step_s) * 1e3, 2), "max_ms": round(max(step_s) * 1e3, 2)}
        del host

    # The other strategies on the same data (same step definition).
    alts = {}
    if args.strategy == "auto":
        names = (("hash", qeg.JOIN_HASH), ("partitioned", qeg.JOIN_PARTITIONED))
        for name, sid in names:
            if name == strategy_name:
                continue
            tt = []
            for i in range(3):
                e = [torch.cuda.Event(enable_timing=True) for _ in range(3)] + [stream]
                a0 = torch.cuda.Event(enable_timing=True)
                a1 = torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                ares, _ = W.run(qeg, ctx, sid, events=e)
                a1.record(stream)
                torch.cuda.synchronize()
                assert ares == res, (name, ares, res)
                if i:
                    tt.append((a0.elapsed_time(a1), e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])))
            step = float(np.mean([x[0] for x in tt]))
            bms = float(np.mean([x[1] for x in tt]))
            pms = float(np.mean([x[2] for x in tt]))
            alts[name] = {"strategy": name, "value": W.rows() / (step / 1e3), "ms_per_step": step,
                          "build_ms": bms, "probe_ms": pms,
                          "probe_gbs": W.algorithmic_probe_bytes() / (pms / 1e3) / 1e9,
                          "probe_frac": W.algorithmic_probe_bytes() / (pms / 1e3) / 1e9 / peak}
            parity[name + "_equal"] = True

    cpu = None
    cpu_job = None
    if rank == 0 and not args.no_cpu and not sub:
        # The reference's algorithm (the oracle's port of its morsel-parallel
        # engine) on the WHOLE workload, every host thread: one run, which is
        # also a full-size parity check against the oracle.
        sample = list(W.cpu_columns(W.nprobe))
        nbuild, nprobe = W.nbuild, W.nprobe

        def cpu_job(out):
            import oracle as O

            v, dt, cres = cpu_reference(sample, threads, nprobe, nbuild)
            out["full_size_parity"]["count_sum_vs_oracle"] = cres == res
            c = {"value": v, "unit": "rows/s", "cores": threads, "kind": "port",
                 "sample": "the whole workload (%d build + %d probe rows, %.1f s, one run)" % (nbuild, nprobe, dt)}
            # Second reference point: the single-threaded operator tree (scan
            # -> join -> aggregate, the restatement of Plan::lower + drain).
            k1 = min(nprobe, 1 << 23)
            t1 = time.perf_counter()
            r1 = O.join_count_sum(O.TCol(O.I64, sample[0].values[:k1], sample[0].valid[:k1]),
                                  O.TCol(O.I64, sample[1].values[:k1]), sample[2])
            dt1 = time.perf_counter() - t1
            c["single_thread"] = {"value": (nbuild + k1) / dt1, "unit": "rows/s", "cores": 1,
                                  "sample": "full %d-row build + first %d probe rows (%.1f s), count %d"
                                            % (nbuild, k1, dt1, r1[0])}
            out["cpu_baseline"] = c
            sample.clear()
            assert out["full_size_parity"]["count_sum_vs_oracle"], out["full_size_parity"]
    ok = all(v for k, v in parity.items() if k != "expected")
    assert ok, parity
    kernel = {"dense": "probe_sink_lean_kernel (dense, unique keys)",
              "hash": "probe_sink_lean_kernel (hash table)"}.get(strategy_name, "probe_sink_pipe_kernel")
    out = {
        "metric": "rows/s hash join (build+probe rows), inner join COUNT(*)+SUM(payload)",
        "value": value, "unit": "rows/s", "n_gpus": world, "steps": steps, "warmup": warm,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int64", "data": "synthetic (seeded, generated on the GPU)",
        "config": {"workload": W.name, "build_rows": W.nbuild, "probe_rows": W.nprobe, "seed": SEED + 2,
                   "M": "2^20", "keys": "sparse (odd-multiplier bijection over int64)" if sparse
                   else "dense (permutation of 0..build_rows-1)",
                   "null_keys": "2% both sides", "probe_hit_rate": 0.5, "strategy": strategy_name,
                   "l2": "inputs exceed L2 (4.3 GB probe side), no flush", "parallelism": "replicas"
                   if world > 1 else "single GPU", "result": {"count": res[0], "sum": res[1]}},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (SINK_TRAFFIC_PER_ROW * W.nprobe if strategy_name == "dense"
                                 else HASH_SINK_TRAFFIC_PER_ROW * W.nprobe if HASH_SINK_TRAFFIC_PER_ROW
                                 else None),
                     "traffic_source": "ncu dram bytes of the same sink on a 64M-row probe side, scaled by "
                                       "probe rows",
                     "probe_ms": probe_ms, "algorithmic_bytes": W.algorithmic_probe_bytes(),
                     "build_ms": build_ms,
                     "build_probe_frac": (W.algorithmic_probe_bytes() + W.algorithmic_build_bytes())
                     / ((build_ms + probe_ms) / 1e3) / 1e9 / peak},
        "full_size_parity": parity,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "wall_s": wall,
    }
    for name, a in alts.items():
        out[name + "_strategy"] = a
    ctx.close()
    del W
    torch.cuda.empty_cache()
    if cpu_job is not None:
        if cpu_later is not None:
            cpu_later.append(lambda: cpu_job(out))
        else:
            cpu_job(out)
    return out


def run_join_sizing_bench(args, dev, local, emit=True):
    """Learned vs plain table sizing of a hashed join whose build side repeats
    its keys: 16M build rows over 1M distinct sparse keys, 256M probe rows
    (half hits), COUNT(*) + SUM(payload). Plain sizing gives the table two
    slots per build row (2^25); learned sizing sketches the build keys and
    gives it four per estimated distinct key. One step = build + probe."""
    import qeg

    W = JoinWorkload(dev, args.build_rows, args.probe_rows, sparse=True, distinct=1 << 20)
    ctx = qeg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    steps = min(args.steps, 10)
    warm = max(3, min(args.warmup, 3))
    peak, pkind = peaks()
    exp = W.expected_torch()
    out = {}
    clk = ClockSampler(local).__enter__()
    tw0 = time.time()
    for name, sizing in (("learned", qeg.SIZE_LEARNED), ("plain_fixed", qeg.SIZE_FIXED)):
        for _ in range(warm):
            res, st = W.run(qeg, ctx, qeg.JOIN_AUTO, sizing=sizing)
        ctx.synchronize()
        evs = []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            pe = [torch.cuda.Event(enable_timing=True) for _ in range(3)] + [stream]
            res, st = W.run(qeg, ctx, qeg.JOIN_AUTO, events=pe, sizing=sizing)
            evs.append(pe)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        bms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
        pms = float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
        out[name] = {"ms_per_step": ms, "rows_per_s": W.rows() / (ms / 1e3), "build_ms": bms, "probe_ms": pms,
                     "probe_frac": W.algorithmic_probe_bytes() / (pms / 1e3) / 1e9 / peak, "stats": st,
                     "count_sum_vs_torch": res == exp}
    clocks = clk.summary(tw0, time.time())
    clk.__exit__(None, None, None)
    parity = {"learned_vs_torch": out["learned"]["count_sum_vs_torch"],
              "plain_vs_torch": out["plain_fixed"]["count_sum_vs_torch"],
              "expected": {"count": exp[0], "sum": exp[1]}}
    assert parity["learned_vs_torch"] and parity["plain_vs_torch"], parity
    best = out["learned"]
    line = {
        "metric": "rows/s hash join (build+probe rows), inner join COUNT(*)+SUM(payload), learned vs plain sizing",
        "value": best["rows_per_s"], "unit": "rows/s", "n_gpus": 1, "steps": steps, "warmup": warm,
        "ms_per_step": best["ms_per_step"], "higher_is_better": True, "dtype": "int64",
        "data": "synthetic (seeded, generated on the GPU)",
        "config": {"workload": W.name, "build_rows": W.nbuild, "probe_rows": W.nprobe, "distinct_build_keys": 1 << 20,
                   "seed": SEED + 2, "keys": "sparse (odd-multiplier bijection over int64), repeated on the build side",
                   "null_keys": "2% both sides", "probe_hit_rate": 0.5},
        "roofline": {"bound": "hbm", "kernel": "probe_sink_lean_kernel (hash table)",
                     "achieved": W.algorithmic_probe_bytes() / (best["probe_ms"] / 1e3) / 1e9, "peak": peak,
                     "peak_kind": pkind, "unit": "GB/s", "frac": best["probe_frac"], "probe_ms": best["probe_ms"]},
        "variants": out,
        "learned_vs_plain": out["plain_fixed"]["ms_per_step"] / best["ms_per_step"],
        "full_size_parity": parity,
        "clocks": clocks,
    }
    ctx.close()
    del W
    torch.cuda.empty_cache()
    if emit:
        print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="join")
    ap.add_argument("--strategy", default="auto", choices=["auto", "hash", "dense", "partitioned"])
    ap.add_argument("--sparse", action="store_true", help="join workload: sparse keys (hash table)")
    ap.add_argument("--headline-only", action="store_true",
                    help="join workload: skip the secondary workloads of the default run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--agg-rows", type=int, default=None)
    ap.add_argument("--ticks", type=int, default=200_000_000, help="trades of the window/asof workloads")
    ap.add_argument("--variants", default=None)
    ap.add_argument("--build-rows", type=int, default=1 << 24)
    ap.add_argument("--probe-rows", type=int, default=1 << 28)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, threads)
        return

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    if args.workload in ("skew", "agg1m"):
        run_agg_bench(args, dev, local)
        return
    if args.workload == "batch":
        run_batch_bench(args, dev, local)
        return
    if args.workload == "pipeline":
        run_pipeline_bench(args, dev, local)
        return
    if args.workload == "window":
        run_window_bench(args, dev, local)
        return
    if args.workload == "asof":
        run_asof_bench(args, dev, local)
        return
    if args.workload == "join_sizing":
        run_join_sizing_bench(args, dev, local)
        return
    if args.workload == "operators":
        print(json.dumps(operator_bench()))
        return

    t_start = time.perf_counter()
    cpu_later = []  # the join's CPU baseline runs after every GPU measurement
    out = run_join_bench(args, dev, local, world, rank, threads, sparse=args.sparse, cpu_later=cpu_later)
    if world == 1 and not args.headline_only and not args.sparse:
        # The default run also measures, each on its own data and each with
        # its full-size parity check: the same join over sparse keys (the hash
        # table), the 1M-row plain GROUP BY, the 512M-row skewed GROUP BY
        # (learned vs plain sizing), the 4096-query batch and the fused
        # filter -> join -> aggregate pipeline.
        sub = argparse.Namespace(**vars(args))
        sub.no_cpu = True
        out["sparse_keys"] = run_join_bench(sub, dev, local, world, rank, threads, sparse=True, sub=True)
        out["repeated_keys"] = run_join_sizing_bench(sub, dev, local, emit=False)
        sub.no_cpu = args.no_cpu
        out["plain_agg"] = run_agg_bench(sub, dev, local, kind="agg1m", emit=False)
        out["skew_agg"] = run_agg_bench(sub, dev, local, kind="skew", emit=False)
        out["batch"] = run_batch_bench(sub, dev, local, emit=False)
        out["pipeline"] = run_pipeline_bench(sub, dev, local, emit=False)
        out["operators"] = operator_bench()
        while cpu_later:
            cpu_later.pop(0)()
        fsp = {"join": out["full_size_parity"]}
        for k in ("sparse_keys", "repeated_keys", "plain_agg", "skew_agg", "batch", "pipeline"):
            fsp[k] = out[k]["full_size_parity"]
        fsp["operators_agg"] = {"ok": bool(out["operators"].get("agg", {}).get("check_counts_vs_host"))}
        fsp["operators_join"] = {"ok": bool(out["operators"].get("join", {}).get("check_count_sum_vs_host"))}
        fsp["operators_agg_resident"] = {
            "ok": bool(out["operators"].get("agg_resident", {}).get("check_counts_vs_host"))}
        fsp["operators_join_resident"] = {
            "ok": bool(out["operators"].get("join_resident", {}).get("check_count_sum_vs_host"))}
        out["full_size_parity_all"] = all(
            v.get("ok", all(x for kk, x in v.items() if kk not in ("expected",) and isinstance(x, bool)))
            for v in fsp.values())
    while cpu_later:
        cpu_later.pop(0)()
    out["bench_wall_s"] = time.perf_counter() - t_start
    if rank == 0:
        print(json.dumps(out))


def run_reference(args, threads):
    """The reference arm: the reference's CPU algorithm for this path (the
    oracle's port of its morsel-parallel engine, exec/parallel.cpp:374-599) on
    the host cores with every thread, on the WHOLE join workload (16M build +
    256M probe rows) per step. The reference itself compiles only where its
    source tree is present, so the port stands in for it."""
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else None
    if dev is None:
        print(json.dumps({"impl": "reference", "unavailable": "no GPU to generate the synthetic data on"}))
        return
    W = JoinWorkload(dev, args.build_rows, args.probe_rows)
    name, nbuild, nprobe = W.name, W.nbuild, W.nprobe
    sample = W.cpu_columns(nprobe)
    del W
    torch.cuda.empty_cache()
    warm = max(0, min(args.warmup, 1))
    steps = max(1, min(args.steps, 3))
    for _ in range(warm):
        cpu_reference(sample, threads, nprobe, nbuild)
    vals, times = [], []
    for _ in range(steps):
        v, dt, res = cpu_reference(sample, threads, nprobe, nbuild)
        vals.append(v)
        times.append(dt)
    ms = np.array(times) * 1e3
    total_s = float(np.sum(times))
    v = (nbuild + nprobe) * steps / total_s
    print(json.dumps({
        "impl": "reference", "metric": "rows/s hash join (build+probe rows), inner join COUNT(*)+SUM(payload)",
        "value": v, "unit": "rows/s", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": float(np.mean(ms)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded)",
        "config": {"workload": name, "build_rows": nbuild, "probe_rows": nprobe,
                   "keys": "dense (permutation of 0..build_rows-1)", "null_keys": "2% both sides",
                   "probe_hit_rate": 0.5, "result": {"count": res[0], "sum": res[1]},
                   "ms_p50": float(np.percentile(ms, 50)), "ms_p99": float(np.percentile(ms, 99)),
                   "steps_note": "each step is the whole workload (%.0f s); steps capped at 3 to keep the run "
                                 "within a few minutes" % float(np.mean(times))},
        "cpu_baseline": {"value": v, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": "the whole workload per step (%d build + %d probe rows), morsels of "
                                   "probe_rows/threads, each rebuilding the build side" % (nbuild, nprobe)},
        "e2e": {"value": v, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    main()
