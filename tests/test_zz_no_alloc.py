"""The no-allocation join COUNT/SUM sink (qeg_join_count_sum_noalloc).

Some callers cannot call cudaMalloc: engines whose device memory belongs to
another allocator (a fixed arena that a stray allocation would fragment or
exceed), plugins in a host application that accounts for every device byte,
latency paths that cannot risk an allocation stall or failure at query time.
This entry point serves them from a fixed scratch array built into libqeg.so.

These tests call it through the C ABI and check its results against the
oracle (the CPU restatement of the reference's HashJoin feeding a
COUNT(*)/SUM aggregate) and against the allocating entry point
(qeg_join_build / qeg_join_probe_count_sum), on two calls in a row, so that
the second call also proves the shared scratch is cleared between calls.
Results are integers, compared exactly. This file is collected last on
purpose: a run that stops at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
import qeg

pytestmark = pytest.mark.gpu


def _case(seed, nbuild, nprobe, dup, payload_nulls=0.0, hit_rate=0.5):
    """Seeded host columns: build keys (a permutation, or with duplicates), 2%
    NULL keys on both sides, probe keys half from the build range and half from
    a disjoint range, an int64 payload (optionally with NULLs)."""
    rng = np.random.default_rng(seed)
    bkey = rng.permutation(nbuild).astype(np.int64)
    if dup:
        bkey //= 3
    bvalid = rng.random(nbuild) >= 0.02
    hit = rng.random(nprobe) < hit_rate
    pkey = np.where(hit, rng.integers(0, nbuild, nprobe), rng.integers(nbuild, 2 * nbuild, nprobe)).astype(np.int64)
    pvalid = rng.random(nprobe) >= 0.02
    pval = rng.integers(0, 1 << 20, nprobe).astype(np.int64)
    vvalid = None if payload_nulls == 0 else rng.random(nprobe) >= payload_nulls
    return bkey, bvalid, pkey, pvalid, pval, vvalid


def _device_cols(torch, bkey, bvalid, pkey, pvalid, pval, vvalid):
    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def words(mask):
        return None if mask is None else dev(qeg.pack_validity(mask).view(np.int64))

    cols = (qeg.Col(dev(bkey), words(bvalid), qeg.I64), qeg.Col(dev(pkey), words(pvalid), qeg.I64),
            qeg.Col(dev(pval), words(vvalid), qeg.I64))
    torch.cuda.synchronize()  # the allocating entry point reads them on the library's own stream
    return cols


def _oracle(bkey, bvalid, pkey, pvalid, pval, vvalid):
    return O.join_count_sum(O.TCol(O.I64, pkey, pvalid), O.TCol(O.I64, pval, vvalid), O.TCol(O.I64, bkey, bvalid))


def _allocating(ctx, bk, pk, pv):
    j = qeg.Join(ctx, [qeg.I64, qeg.I64], [qeg.I64], [0], [0], strategy=qeg.JOIN_HASH)
    j.build([bk])
    j.build_finish()
    j.probe_count_sum(pk, pv)
    res = j.count_sum()
    j.close()
    return res


def _noalloc(torch, bk, pk, pv):
    out = torch.full((4,), -7, dtype=torch.int64, device="cuda")
    qeg.join_count_sum_noalloc(torch.cuda.current_stream().cuda_stream, bk, pk, pv, out)
    torch.cuda.synchronize()
    got = out.cpu().tolist()
    assert got[3] == 0, "scratch flags %d (bit 0 overflow, bit 1 STR code out of range)" % got[3]
    return got[0], (got[1] if got[2] else None)


def test_noalloc_matches_oracle_and_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    ctx = qeg.Context(0)
    try:
        cases = [_case(1, 1 << 18, 1 << 22, dup=False), _case(2, 1 << 20, 1 << 21, dup=True)]
        for host in cases:
            exp = _oracle(*host)
            bk, pk, pv = _device_cols(torch, *host)
            assert _allocating(ctx, bk, pk, pv) == exp
            assert _noalloc(torch, bk, pk, pv) == exp
    finally:
        ctx.close()


def test_noalloc_sum_is_null_when_every_matched_payload_is_null():
    torch = pytest.importorskip("torch")
    # Every payload NULL: the matched count is positive, the SUM is NULL.
    host = _case(3, 1 << 12, 1 << 16, dup=False, payload_nulls=1.0)
    exp = _oracle(*host)
    assert exp[0] > 0 and exp[1] is None
    bk, pk, pv = _device_cols(torch, *host)
    for _ in range(2):
        assert _noalloc(torch, bk, pk, pv) == exp
    # No probe key matches: count 0 and a NULL SUM (the reference's empty SUM).
    host = _case(4, 1 << 12, 1 << 14, dup=False, hit_rate=0.0)
    exp = _oracle(*host)
    assert exp == (0, None)
    bk, pk, pv = _device_cols(torch, *host)
    assert _noalloc(torch, bk, pk, pv) == exp


def test_noalloc_call_captured_in_a_cuda_graph():
    """The call enqueues only a memset and kernels, so a caller can capture it
    in a CUDA graph (after one plain call on the device, which looks up the
    scratch array's address) and replay it; each replay re-reads the columns."""
    torch = pytest.importorskip("torch")
    host = _case(5, 1 << 16, 1 << 20, dup=True, payload_nulls=0.1)
    exp = _oracle(*host)
    bk, pk, pv = _device_cols(torch, *host)
    assert _noalloc(torch, bk, pk, pv) == exp  # the plain call before capture
    s = torch.cuda.Stream()
    out = torch.full((4,), -7, dtype=torch.int64, device="cuda")
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        qeg.join_count_sum_noalloc(s.cuda_stream, bk, pk, pv, out)

    def replay():
        out.fill_(-7)
        g.replay()
        torch.cuda.synchronize()
        got = out.cpu().tolist()
        assert got[3] == 0
        return got[0], (got[1] if got[2] else None)

    assert replay() == exp
    assert replay() == exp
    # New payload values in the same buffer: the replay sums them.
    pval2 = (host[4] * 3 + 1).astype(np.int64)
    pv.values.copy_(torch.from_numpy(pval2))
    torch.cuda.synchronize()
    exp2 = _oracle(host[0], host[1], host[2], host[3], pval2, host[5])
    assert exp2 != exp
    assert replay() == exp2


def _str_col(torch, codes, cmap, cm_len):
    """A raw STR column (codes + code map on the device) whose code_map_len
    is given explicitly; returns it with the tensors that back it."""
    d = torch.from_numpy(codes).cuda()
    m = torch.from_numpy(cmap).cuda()
    torch.cuda.synchronize()
    raw = qeg.Column(qeg.STR, 1, codes.size, d.data_ptr(), None, m.data_ptr(), cm_len)
    return raw, (d, m)


def _call_raw(torch, b, k, v):
    out = torch.full((4,), -7, dtype=torch.int64, device="cuda")
    st = qeg.lib().qeg_join_count_sum_noalloc(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                              ctypes.byref(b), ctypes.byref(k), ctypes.byref(v),
                                              ctypes.c_void_p(out.data_ptr()))
    assert st == 0
    torch.cuda.synchronize()
    return out.cpu().tolist()


def test_noalloc_str_keys_follow_the_code_map_rule():
    """A STR key's code map is applied only when code_map_len > 0, as in the
    allocating path; a code outside the map skips its row and sets bit 1."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    nb, npr = 1000, 50000
    bcodes = rng.permutation(nb).astype(np.int32)
    pcodes = rng.integers(0, 2 * nb, npr).astype(np.int32)
    pval = rng.integers(0, 1 << 20, npr).astype(np.int64)
    ident = np.arange(2 * nb, dtype=np.int32)
    shifted = (ident + 7).astype(np.int32)  # a map that moves every id
    keep = []
    pv = torch.from_numpy(pval).cuda()
    torch.cuda.synchronize()
    vraw = qeg.Column(qeg.I64, 1, npr, pv.data_ptr(), None, None, 0)
    # code_map_len == 0: the pointer is ignored, codes compare as themselves
    # (the build map differs from the probe map, so applying them would change
    # the matches).
    braw, kb = _str_col(torch, bcodes, shifted, 0)
    praw, kp = _str_col(torch, pcodes, ident, 0)
    keep += [kb, kp]
    exp = _oracle(bcodes.astype(np.int64), None, pcodes.astype(np.int64), None, pval, None)
    ctx = qeg.Context(0)
    try:
        for _ in range(2):
            got = _call_raw(torch, braw, praw, vraw)
            assert got[3] == 0 and (got[0], got[1] if got[2] else None) == exp
        # Through the allocating path, with the same raw columns.
        ja = qeg.Join(ctx, [qeg.STR, qeg.I64], [qeg.STR], [0], [0], strategy=qeg.JOIN_HASH)
        st = qeg.lib().qeg_join_build(ja.p, ctypes.byref(braw), 1)
        assert st == 0
        ja.build_finish()
        assert qeg.lib().qeg_join_probe_count_sum(ja.p, ctypes.byref(praw), ctypes.byref(vraw)) == 0
        assert ja.count_sum() == exp
        ja.close()
    finally:
        ctx.close()
    # A probe code one past its map's end: the row is skipped and flagged.
    bad = pcodes.copy()
    bad[17] = 2 * nb
    praw2, kp2 = _str_col(torch, bad, ident, 2 * nb)
    braw2, kb2 = _str_col(torch, bcodes, ident, 2 * nb)
    keep += [kp2, kb2]
    got = _call_raw(torch, braw2, praw2, vraw)
    assert got[3] == 2
    okrows = np.ones(npr, bool)
    okrows[17] = False
    exp2 = _oracle(bcodes.astype(np.int64), None, bad.astype(np.int64), okrows, pval, None)
    assert (got[0], got[1] if got[2] else None) == exp2


def test_noalloc_rejects_build_beyond_limit():
    torch = pytest.importorskip("torch")
    n = (1 << 20) + 1
    bk = qeg.Col(torch.zeros(n, dtype=torch.int64, device="cuda"), None, qeg.I64)
    pk = qeg.Col(torch.zeros(4, dtype=torch.int64, device="cuda"), None, qeg.I64)
    out = torch.zeros(4, dtype=torch.int64, device="cuda")
    with pytest.raises(qeg.QegError) as e:
        qeg.join_count_sum_noalloc(torch.cuda.current_stream().cuda_stream, bk, pk, pk, out)
    assert e.value.code == -1 and "1048576" in str(e.value)
