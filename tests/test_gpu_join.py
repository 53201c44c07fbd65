"""GPU hash-join parity against the oracle, through the C ABI (libqeg.so).

Mirrors the reference's tests/join_differential_test.cpp: the hand-built edge
cases (single key with matches / misses / NULL key, composite (i32, f64) key,
empty build side, empty probe side, all-match cross product, a 3000-row
fan-out past the 2048-row output batch, NULL never equals NULL) for INNER and
LEFT, then seeded random join cases, then the fused COUNT(*)/SUM sink under
every strategy. Join output is unordered: both sides are canonicalised.
"""
import numpy as np
import pytest

import oracle as O
import qeg
from util import StrCanon, assert_same, gen_column, gpu_rows, to_gpu

pytestmark = pytest.mark.gpu


def i32(v, nulls=()):
    valid = None
    if nulls:
        valid = np.ones(len(v), bool)
        valid[list(nulls)] = False
    return O.TCol(O.I32, np.array(v, np.int32), valid)


def i64(v, nulls=()):
    valid = None
    if nulls:
        valid = np.ones(len(v), bool)
        valid[list(nulls)] = False
    return O.TCol(O.I64, np.array(v, np.int64), valid)


def f64(v):
    return O.TCol(O.F64, np.array(v, np.float64))


def run_gpu(ctx, probe, build, pk, bk, jt, strategy=qeg.JOIN_AUTO, fetch_chunk=2048, build_batches=1):
    canon = StrCanon([s for c in probe + build if c.type == O.STR for s in c.dictionary])
    j = qeg.Join(ctx, [c.type for c in probe], [c.type for c in build], pk, bk, jt, strategy=strategy)
    try:
        nb = build[0].n
        step = max(64, -(-nb // build_batches) // 64 * 64) if nb else 1
        for s in range(0, max(nb, 1), step):
            e = min(nb, s + step)
            part = []
            for c in build:
                valid = None if c.valid is None else c.valid[s:e]
                part.append(to_gpu(O.TCol(c.type, c.values[s:e], valid, c.dictionary), canon))
            j.build(part)
        j.build_finish()
        n = j.probe([to_gpu(c, canon) for c in probe])
        cols = None
        for first in range(0, n, fetch_chunk):
            part = j.fetch(first, min(fetch_chunk, n - first))
            cols = part if cols is None else [(np.concatenate([a[0], b[0]]), np.concatenate([a[1], b[1]]))
                                              for a, b in zip(cols, part)]
        types = [c.type for c in probe] + [c.type for c in build]
        if cols is None:
            return types, []
        return gpu_rows(cols, types, canon)
    finally:
        j.close()


def check(ctx, probe, build, pk, bk, **kw):
    for jt in (O.INNER, O.LEFT):
        ot, orows = O.join(probe, build, pk, bk, jt)
        gt, grows = run_gpu(ctx, probe, build, pk, bk, jt, **kw)
        assert_same(gt, grows, ot, orows, "join type %d" % jt)


def test_edge_single_key_match_miss_null(ctx):
    build = [i32([1, 1, 2, 5, 5, 5]), i64([10, 11, 20, 50, 51, 52])]
    probe = [i32([1, 2, 3, 5, 0], nulls=[4]), i64([100, 200, 300, 500, 999])]
    check(ctx, probe, build, [0], [0])
    check(ctx, probe, build, [0], [0], strategy=qeg.JOIN_HASH)


def test_edge_composite_key(ctx):
    build = [i32([1, 1, 2, 2]), f64([1.0, 2.0, 1.0, 2.0]), i64([11, 12, 21, 22])]
    probe = [i32([1, 1, 2, 2]), f64([2.0, 9.0, 1.0, 2.0])]
    check(ctx, probe, build, [0, 1], [0, 1])


def test_edge_empty_build(ctx):
    build = [i32([]), i64([])]
    probe = [i32([1, 2, 3])]
    check(ctx, probe, build, [0], [0])


def test_edge_empty_probe(ctx):
    build = [i32([1, 2, 3])]
    probe = [i32([]), i64([])]
    check(ctx, probe, build, [0], [0])


def test_edge_all_match_cross(ctx):
    build = [i32([7, 7, 7, 7]), i64([1, 2, 3, 4])]
    probe = [i32([7, 7, 7])]
    check(ctx, probe, build, [0], [0])


def test_edge_fanout_over_output_batch(ctx):
    build = [i32([7] * 3000), i64(list(range(3000)))]
    probe = [i32([7, 9, 7]), i64([100, 200, 300])]
    check(ctx, probe, build, [0], [0])
    check(ctx, probe, build, [0], [0], strategy=qeg.JOIN_HASH, fetch_chunk=1000)


def test_edge_null_never_matches_null(ctx):
    build = [i32([1, 0, 2], nulls=[1]), i64([10, 11, 12])]
    probe = [i32([1, 0, 0], nulls=[1, 2])]
    check(ctx, probe, build, [0], [0])


def test_f64_keys_canonicalised(ctx):
    nan = float("nan")
    build = [f64([0.0, nan, 1.5]), i64([1, 2, 3])]
    probe = [f64([-0.0, nan, 1.5, 2.5])]
    check(ctx, probe, build, [0], [0])


def test_str_keys_join_by_value_across_dictionaries(ctx):
    bdict = ["IBM", "AAPL", "MSFT"]
    pdict = ["MSFT", "GOOG", "AAPL"]
    build = [O.TCol(O.STR, np.array([0, 1, 2, 1], np.int32), None, bdict), i64([1, 2, 3, 4])]
    probe = [O.TCol(O.STR, np.array([0, 1, 2, 2], np.int32), np.array([1, 1, 1, 0], bool), pdict)]
    check(ctx, probe, build, [0], [0])


@pytest.mark.parametrize("seed", range(3))
def test_random_joins(ctx, seed):
    rng = np.random.default_rng(0x301D + seed)
    for it in range(40):
        nk = int(rng.integers(1, 3))
        kt = [int(rng.choice([O.I32, O.I64, O.F64])) for _ in range(nk)]
        card = int(rng.integers(1, 80))
        nb, npr = int(rng.integers(0, 3000)), int(rng.integers(0, 3000))
        build = [gen_column(rng, t, nb, 10, card) for t in kt] + [gen_column(rng, O.I64, nb, 10)]
        probe = [gen_column(rng, t, npr, 10, card * 2) for t in kt] + [gen_column(rng, O.F64, npr, 10)]
        jt = int(rng.integers(0, 2))
        strategy = int(rng.choice([qeg.JOIN_AUTO, qeg.JOIN_HASH]))
        ot, orows = O.join(probe, build, list(range(nk)), list(range(nk)), jt)
        gt, grows = run_gpu(ctx, probe, build, list(range(nk)), list(range(nk)), jt, strategy=strategy,
                            build_batches=int(rng.integers(1, 4)))
        assert_same(gt, grows, ot, orows, "seed %d iter %d" % (seed, it))


@pytest.mark.parametrize("strategy", [qeg.JOIN_AUTO, qeg.JOIN_HASH, qeg.JOIN_DENSE])
@pytest.mark.parametrize("dup", [False, True])
@pytest.mark.parametrize("kernel", ["default", "pipe0", "pipe2", "pipe4", "pipe8", "tma"])
def test_count_sum_sink(ctx, strategy, dup, kernel, monkeypatch):
    """The 16M x 256M join workload's shape at 1/64 scale: unique (or
    duplicated) build keys, probe keys half hits and half from a disjoint
    range, 2% NULL keys on both sides, SUM over an int64 payload. `kernel`
    picks the sink kernel: the default (the small-register kernel at high
    occupancy, for every table kind), the 4-rows-per-thread kernel, 128-row
    or 256-row pipelined warp tiles, the
    cp.async-staged kernel, or the opt-in TMA-staged kernel (each 2M-row half
    is large enough for it)."""
    if kernel == "tma":
        monkeypatch.setenv("QEG_SINK_TMA", "1")
    elif kernel != "default":
        monkeypatch.setenv("QEG_SINK_PIPE", kernel[-1])
    rng = np.random.default_rng(99 + strategy + 10 * dup)
    nb, npr = 1 << 18, 1 << 22
    bkey = rng.permutation(nb).astype(np.int64)
    if dup:
        bkey = bkey // 3
    bvalid = rng.random(nb) >= 0.02
    hit = rng.random(npr) < 0.5
    pkey = np.where(hit, rng.integers(0, nb, npr), rng.integers(nb, 2 * nb, npr)).astype(np.int64)
    pvalid = rng.random(npr) >= 0.02
    pval = rng.integers(0, 1 << 20, npr).astype(np.int64)
    exp = O.join_count_sum(O.TCol(O.I64, pkey, pvalid), O.TCol(O.I64, pval), O.TCol(O.I64, bkey, bvalid))
    j = qeg.Join(ctx, [O.I64, O.I64], [O.I64], [0], [0], strategy=strategy)
    j.build([qeg.Col(bkey, qeg.pack_validity(bvalid))])
    j.build_finish()
    half = npr // 2
    j.probe_count_sum(qeg.Col(pkey[:half], qeg.pack_validity(pvalid[:half])), qeg.Col(pval[:half]))
    j.probe_count_sum(qeg.Col(pkey[half:], qeg.pack_validity(pvalid[half:])), qeg.Col(pval[half:]))
    got = j.count_sum()
    st = j.stats()
    j.close()
    assert got == exp
    if strategy == qeg.JOIN_HASH:
        assert st["strategy"] == qeg.JOIN_HASH
    else:
        assert st["strategy"] == qeg.JOIN_DENSE


@pytest.mark.parametrize("kt,vt", [(O.I64, O.I64), (O.I32, O.I64), (O.I64, O.I32), (O.I32, O.I32)])
@pytest.mark.parametrize("kernel", ["default", "pipe2"])
def test_count_sum_dense_types_and_tails(ctx, kt, vt, kernel, monkeypatch):
    # Dense table of unique keys over every key/payload width, probe sides
    # whose length is not a multiple of the 64-row chunk (the per-row tail),
    # NULLs in keys and payloads, negative keys and payloads, and one probe
    # batch with no payload NULLs at all.
    if kernel != "default":
        monkeypatch.setenv("QEG_SINK_PIPE", kernel[-1])
    rng = np.random.default_rng(31 + kt + 3 * vt)
    nb = 50000
    bkey = rng.permutation(nb).astype(np.int64) - 20000
    build = O.TCol(kt, bkey.astype(np.int32 if kt == O.I32 else np.int64), rng.random(nb) >= 0.05)
    j = qeg.Join(ctx, [kt, vt], [kt], [0], [0], strategy=qeg.JOIN_DENSE)
    j.build([to_gpu(build)])
    j.build_finish()
    exp = [0, 0]
    for npr, vnull in ((1000003, 0.03), (64 * 1000 + 63, 0.0), (17, 0.5)):
        pkey = rng.integers(-30000, nb, npr)
        pkey = pkey.astype(np.int32 if kt == O.I32 else np.int64)
        pval = rng.integers(-(1 << 30), 1 << 30, npr).astype(np.int32 if vt == O.I32 else np.int64)
        pk = O.TCol(kt, pkey, rng.random(npr) >= 0.02)
        pv = O.TCol(vt, pval, (rng.random(npr) >= vnull) if vnull else None)
        c, sm = O.join_count_sum(pk, pv, build)
        exp = [exp[0] + c, (exp[1] or 0) + (sm or 0)]
        j.probe_count_sum(to_gpu(pk), to_gpu(pv))
    got = j.count_sum()
    assert j.stats()["strategy"] == qeg.JOIN_DENSE
    j.close()
    assert got == tuple(exp)


def test_count_sum_sparse_keys_use_hash(ctx):
    rng = np.random.default_rng(4)
    nb, npr = 100_000, 1_000_000
    bkey = rng.integers(-(1 << 62), 1 << 62, nb).astype(np.int64)
    pkey = np.where(rng.random(npr) < 0.5, bkey[rng.integers(0, nb, npr)], rng.integers(-(1 << 62), 1 << 62, npr))
    pval = rng.integers(-1000, 1000, npr).astype(np.int64)
    exp = O.join_count_sum(O.TCol(O.I64, pkey.astype(np.int64)), O.TCol(O.I64, pval), O.TCol(O.I64, bkey))
    j = qeg.Join(ctx, [O.I64, O.I64], [O.I64], [0], [0])
    j.build([qeg.Col(bkey)])
    j.build_finish()
    j.probe_count_sum(qeg.Col(pkey.astype(np.int64)), qeg.Col(pval))
    assert j.count_sum() == exp
    assert j.stats()["strategy"] == qeg.JOIN_HASH
    j.close()


@pytest.mark.parametrize("bloom,sweeps", [("0", "1"), ("1", "1"), ("0", "3"), ("1", "2")])
@pytest.mark.parametrize("kt,vt", [(O.I64, O.I64), (O.I32, O.I64), (O.I64, O.I32), (O.I32, O.I32)])
@pytest.mark.parametrize("dup", [False, True])
def test_count_sum_hashed_bloom_filter(ctx, bloom, sweeps, kt, vt, dup, monkeypatch):
    """The hashed COUNT/SUM sink with (QEG_JOIN_BLOOM=1) and without (=0) the
    build keys' Bloom filter in front of the table, probing directly
    (QEG_JOIN_SWEEPS=1) or in sweeps over windows of the table's hash range
    (=2, =3): sparse keys over the whole key width (with key 0 on both sides,
    which has its own table slot), 2% NULL keys, payload NULLs, duplicated
    build keys, and probe sides whose length is not a multiple of the 64-row
    chunk."""
    monkeypatch.setenv("QEG_JOIN_BLOOM", bloom)
    monkeypatch.setenv("QEG_JOIN_SWEEPS", sweeps)
    rng = np.random.default_rng(7 + kt + 5 * vt + 11 * dup)
    dt = np.int32 if kt == O.I32 else np.int64
    nb = 70_001
    lim = (1 << 31) - 1 if kt == O.I32 else (1 << 62)
    bkey = rng.integers(-lim, lim, nb).astype(dt)
    if dup:
        bkey[nb // 2:] = bkey[: nb - nb // 2]
    bkey[5] = 0
    build = O.TCol(kt, bkey, rng.random(nb) >= 0.02)
    j = qeg.Join(ctx, [kt, vt], [kt], [0], [0], strategy=qeg.JOIN_HASH)
    j.build([to_gpu(build)])
    j.build_finish()
    exp = [0, None]
    for npr, vnull in ((1_000_003, 0.03), (64 * 999 + 5, 0.0)):
        pkey = np.where(rng.random(npr) < 0.5, bkey[rng.integers(0, nb, npr)],
                        rng.integers(-lim, lim, npr).astype(dt)).astype(dt)
        pkey[:3] = 0
        pval = rng.integers(-(1 << 30), 1 << 30, npr).astype(np.int32 if vt == O.I32 else np.int64)
        pk = O.TCol(kt, pkey, rng.random(npr) >= 0.02)
        pv = O.TCol(vt, pval, (rng.random(npr) >= vnull) if vnull else None)
        c, sm = O.join_count_sum(pk, pv, build)
        exp = [exp[0] + c, sm if exp[1] is None else (exp[1] + (sm or 0))]
        j.probe_count_sum(to_gpu(pk), to_gpu(pv))
    got = j.count_sum()
    assert j.stats()["strategy"] == qeg.JOIN_HASH
    j.close()
    assert got == tuple(exp)


def test_count_sum_bloom_filter_by_table_size(ctx):
    """Without an override the filter comes with tables of 32 MB or more (here
    2^21 build rows, a 2^22-slot table): the result is unchanged."""
    rng = np.random.default_rng(12)
    nb, npr = 1 << 21, 1 << 22
    bkey = rng.integers(-(1 << 62), 1 << 62, nb).astype(np.int64)
    pkey = np.where(rng.random(npr) < 0.5, bkey[rng.integers(0, nb, npr)], rng.integers(-(1 << 62), 1 << 62, npr))
    pval = rng.integers(0, 1 << 20, npr).astype(np.int64)
    pvalid = rng.random(npr) >= 0.02
    exp = O.join_count_sum(O.TCol(O.I64, pkey.astype(np.int64), pvalid), O.TCol(O.I64, pval), O.TCol(O.I64, bkey))
    j = qeg.Join(ctx, [O.I64, O.I64], [O.I64], [0], [0])
    j.build([qeg.Col(bkey)])
    j.build_finish()
    j.probe_count_sum(qeg.Col(pkey.astype(np.int64), qeg.pack_validity(pvalid)), qeg.Col(pval))
    assert j.count_sum() == exp
    assert j.stats()["strategy"] == qeg.JOIN_HASH
    j.close()


@pytest.mark.parametrize("dup", [False, True])
@pytest.mark.parametrize("ktype", [O.I64, O.I32])
@pytest.mark.parametrize("bits", [0, 6])
@pytest.mark.parametrize("vnulls", [False, True])
@pytest.mark.parametrize("bloom", ["0", "1"])
def test_partitioned_count_sum_sink(ctx, dup, ktype, bits, vnulls, bloom, monkeypatch):
    """The radix-partitioned join (the probe side split by key-hash partition
    in one tile-sorted pass, then probed in partition order against the hash
    table) against the oracle: unique or duplicated build keys, NULL keys on
    both sides, 64-bit and 32-bit keys (negative values included), automatic
    or fixed partition bits, with and without the build keys' Bloom filter
    (rows it rules out are not partitioned); with payload NULLs the direct
    hashed sink runs."""
    monkeypatch.setenv("QEG_JOIN_BLOOM", bloom)
    rng = np.random.default_rng(500 + dup + 2 * (ktype == O.I32) + bits + 7 * vnulls)
    nb, npr = 1 << 17, (1 << 21) + 77
    dt = np.int64 if ktype == O.I64 else np.int32
    bkey = (rng.permutation(nb) - nb // 3).astype(dt)
    if dup:
        bkey = (bkey // 3).astype(dt)
    bkey[:5] = 0  # key word 0 marks an empty slot: it must still join
    bvalid = rng.random(nb) >= 0.02
    hit = rng.random(npr) < 0.5
    pkey = np.where(hit, bkey[rng.integers(0, nb, npr)], rng.integers(nb, 2 * nb, npr)).astype(dt)
    pvalid = rng.random(npr) >= 0.02
    pval = rng.integers(-(1 << 20), 1 << 20, npr).astype(np.int64)
    vvalid = (rng.random(npr) >= 0.05) if vnulls else np.ones(npr, bool)
    exp = O.join_count_sum(O.TCol(ktype, pkey, pvalid), O.TCol(O.I64, pval, vvalid), O.TCol(ktype, bkey, bvalid))
    j = qeg.Join(ctx, [ktype, O.I64], [ktype], [0], [0], strategy=qeg.JOIN_PARTITIONED, partition_bits=bits)
    j.build([qeg.Col(bkey, qeg.pack_validity(bvalid))])
    j.build_finish()
    st = j.stats()
    assert st["strategy"] == qeg.JOIN_PARTITIONED and st["partition_bits"] == (bits or st["partition_bits"]) > 0, st
    j.probe_count_sum(qeg.Col(pkey, qeg.pack_validity(pvalid)),
                      qeg.Col(pval, qeg.pack_validity(vvalid) if vnulls else None))
    got = j.count_sum()
    j.close()
    assert got == exp


def test_partitioned_join_materialises_pairs(ctx):
    """A materialising probe of a partitioned join uses the global table and
    returns the oracle's rows."""
    rng = np.random.default_rng(77)
    nb, npr = 3000, 20000
    bkey = rng.integers(-500, 500, nb).astype(np.int64)
    pkey = rng.integers(-600, 600, npr).astype(np.int64)
    pv = rng.integers(0, 100, npr).astype(np.int64)
    probe = [O.TCol(O.I64, pkey), O.TCol(O.I64, pv)]
    build = [O.TCol(O.I64, bkey)]
    ot, orows = O.join(probe, build, [0], [0], O.INNER)
    j = qeg.Join(ctx, [O.I64, O.I64], [O.I64], [0], [0], strategy=qeg.JOIN_PARTITIONED)
    j.build([qeg.Col(bkey)])
    j.build_finish()
    assert j.stats()["strategy"] == qeg.JOIN_PARTITIONED
    j.probe([qeg.Col(pkey), qeg.Col(pv)])
    res = j.fetch()
    j.close()
    gt, grows = gpu_rows(res, ot)
    assert_same(gt, grows, ot, orows, "partitioned join pairs")


@pytest.mark.parametrize("jt", [O.INNER, O.LEFT])
def test_device_fetch_matches_host_fetch(ctx, jt):
    # Device output buffers take the single-pass gather (values and packed
    # validity written directly); it must equal the host fetch bit for bit,
    # including ranges that start inside a validity word and STR code maps.
    import torch

    rng = np.random.default_rng(77)
    nb, npr = 5000, 20000
    d = ["k%02d" % i for i in range(40)]
    build = [gen_column(rng, O.I64, nb, 10, 3000), gen_column(rng, O.F64, nb, 10), gen_column(rng, O.I32, nb, 20),
             O.TCol(O.STR, rng.integers(0, 40, nb).astype(np.int32), rng.random(nb) > 0.1, d)]
    probe = [gen_column(rng, O.I64, npr, 10, 4000), gen_column(rng, O.BOOL, npr, 10),
             O.TCol(O.STR, rng.integers(0, 40, npr).astype(np.int32), rng.random(npr) > 0.1, d[::-1])]
    canon = StrCanon(d)
    j = qeg.Join(ctx, [c.type for c in probe], [c.type for c in build], [0], [0], jt)
    try:
        j.build([to_gpu(c, canon) for c in build])
        j.build_finish()
        n = j.probe([to_gpu(c, canon) for c in probe])
        assert n > 1000
        for first, count in ((0, n), (37, n - 100), (n - 1, 1)):
            host = j.fetch(first, count)
            dev = j.fetch_device(first, count)
            torch.cuda.synchronize()
            for (hv, hvalid), (dv, dw) in zip(host, dev):
                dvals = dv[:count].cpu().numpy()
                words = dw.cpu().numpy().view(np.uint64)
                dvalid = np.unpackbits(words.view(np.uint8), bitorder="little")[:count].astype(bool)
                assert np.array_equal(dvalid, hvalid)
                assert np.array_equal(dvals[dvalid].view(np.uint8), np.asarray(hv)[hvalid].view(np.uint8))
    finally:
        j.close()


def test_host_fetch_in_row_chunks(ctx):
    # Host outputs are gathered on the device 2^24 rows at a time and copied
    # out chunk by chunk: a fetch over more than one chunk (pageable numpy and
    # page-locked torch buffers) must equal the device fetch bit for bit.
    import torch

    rng = np.random.default_rng(78)
    nb, npr = 1 << 16, (1 << 24) + 4099
    bkey = rng.permutation(nb).astype(np.int64)
    build = [O.TCol(O.I64, bkey), O.TCol(O.F64, rng.random(nb), rng.random(nb) > 0.1)]
    probe = [O.TCol(O.I64, rng.integers(0, nb + nb // 4, npr), rng.random(npr) > 0.02),
             O.TCol(O.I32, rng.integers(0, 1000, npr).astype(np.int32))]
    j = qeg.Join(ctx, [c.type for c in probe], [c.type for c in build], [0], [0], O.LEFT)
    try:
        j.build([to_gpu(c) for c in build])
        j.build_finish()
        pcols = [to_gpu(c) for c in probe]
        n = j.probe(pcols)
        assert n == npr
        for first, count in ((0, n), (64 * 5, n - 64 * 5 - 3), (3, (1 << 24) + 1)):
            dev = j.fetch_device(first, count)
            host = j.fetch(first, count)
            pinned = j.fetch_pinned(first, count)
            torch.cuda.synchronize()
            for (hv, hvalid), (pv, pw), (dv, dw) in zip(host, pinned, dev):
                nw = (count + 63) // 64
                assert torch.equal(pw[:nw], dw[:nw].cpu())
                dvalid = np.unpackbits(dw[:nw].cpu().numpy().view(np.uint8), bitorder="little")[:count].astype(bool)
                assert np.array_equal(dvalid, hvalid)
                dvals = dv[:count].cpu().numpy()
                assert np.array_equal(dvals[dvalid], np.asarray(hv)[dvalid])
                assert np.array_equal(dvals[dvalid], pv[:count].numpy()[dvalid])
    finally:
        j.close()


@pytest.mark.parametrize("kt", [O.I64, O.I32])
@pytest.mark.parametrize("scale", [None, "0.001"])
def test_learned_table_sizing_of_repeated_build_keys(ctx, kt, scale, monkeypatch):
    """A 2M-row build side over about 100k distinct sparse keys: learned sizing
    (the default) sketches the build keys and gives the table 4 slots per
    estimated distinct key (a power of two, below the plain size) instead of
    2 per build row; a forced underestimate
    (QEG_JOIN_EST_SCALE) overflows the small table, which is rebuilt at full
    size. COUNT/SUM and the materialised pairs (INNER and LEFT, a probe sample)
    equal the oracle's and plain sizing's either way."""
    if scale:
        monkeypatch.setenv("QEG_JOIN_EST_SCALE", scale)
    rng = np.random.default_rng(31 + kt)
    dt = np.int32 if kt == O.I32 else np.int64
    lim = (1 << 31) - 1 if kt == O.I32 else (1 << 62)
    nb, nd, npr = 1 << 21, 100_000, 1 << 22
    distinct = rng.integers(-lim, lim, nd).astype(dt)
    bkey = distinct[rng.integers(0, nd, nb)]
    bkey[7] = 0
    build = O.TCol(kt, bkey, rng.random(nb) >= 0.02)
    pkey = np.where(rng.random(npr) < 0.5, distinct[rng.integers(0, nd, npr)],
                    rng.integers(-lim, lim, npr).astype(dt)).astype(dt)
    pkey[:5] = 0
    pval = rng.integers(-(1 << 30), 1 << 30, npr).astype(np.int64)
    pk = O.TCol(kt, pkey, rng.random(npr) >= 0.02)
    pv = O.TCol(O.I64, pval, rng.random(npr) >= 0.01)
    exp = O.join_count_sum(pk, pv, build)
    stats = {}
    for sizing in (qeg.SIZE_LEARNED, qeg.SIZE_FIXED):
        j = qeg.Join(ctx, [kt, O.I64], [kt], [0], [0], strategy=qeg.JOIN_HASH, sizing=sizing)
        j.build([to_gpu(build)])
        j.build_finish()
        j.probe_count_sum(to_gpu(pk), to_gpu(pv))
        got = j.count_sum()
        stats[sizing] = j.stats()
        j.close()
        assert got == exp, (sizing, got, exp)
    full = 1 << 22  # two slots per build row
    assert stats[qeg.SIZE_FIXED]["slots"] == full and stats[qeg.SIZE_FIXED]["est_distinct"] == 0
    learned = stats[qeg.SIZE_LEARNED]
    if scale:
        assert learned["rebuilds"] == 1 and learned["slots"] == full, learned
    else:
        assert learned["rebuilds"] == 0 and learned["slots"] < full, learned
        assert 0.5 * nd < learned["est_distinct"] < 8 * nd, learned
    # Pair materialisation over the same table (a probe sample, both join types).
    m = 20_000
    ps = [O.TCol(kt, pkey[:m], pk.valid[:m]), O.TCol(O.I64, pval[:m])]
    bs = [build, O.TCol(O.I64, rng.integers(0, 1000, nb).astype(np.int64))]
    for jt in (O.INNER, O.LEFT):
        ot, orows = O.join(ps, bs, [0], [0], jt)
        gt, grows = run_gpu(ctx, ps, bs, [0], [0], jt, strategy=qeg.JOIN_HASH)
        assert_same(gt, grows, ot, orows, "join type %d" % jt)
