"""The no-allocation join COUNT/SUM sink (qeg_join_count_sum_noalloc).

It exists for callers that may not call cudaMalloc -- code running while a CUDA
graph is captured, engines whose device memory is owned by another allocator,
latency-critical paths that cannot risk an allocation at query time -- and runs
in a fixed scratch array built into libqeg.so. These tests call it through the
C ABI and check its results against the allocating entry point
(qeg_join_build / qeg_join_probe_count_sum) on two calls in a row, so that the
second call also proves the shared scratch is cleared between calls. Results
are integers, compared exactly. This file is collected last on purpose.
"""
import numpy as np
import pytest

import qeg

pytestmark = pytest.mark.gpu


def _case(torch, seed, nbuild, nprobe, dup):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    bkey = torch.randperm(nbuild, generator=g, device="cuda", dtype=torch.int64)
    if dup:
        bkey = bkey // 3
    bvalid = torch.rand(nbuild, generator=g, device="cuda") >= 0.02
    hit = torch.rand(nprobe, generator=g, device="cuda") < 0.5
    pkey = torch.where(hit, torch.randint(0, nbuild, (nprobe,), generator=g, device="cuda"),
                       torch.randint(nbuild, 2 * nbuild, (nprobe,), generator=g, device="cuda"))
    pvalid = torch.rand(nprobe, generator=g, device="cuda") >= 0.02
    pval = torch.randint(0, 1 << 20, (nprobe,), generator=g, device="cuda", dtype=torch.int64)

    def words(mask):
        return torch.from_numpy(qeg.pack_validity(mask.cpu().numpy()).view(np.int64)).cuda()

    cols = (qeg.Col(bkey, words(bvalid), qeg.I64), qeg.Col(pkey.contiguous(), words(pvalid), qeg.I64),
            qeg.Col(pval, None, qeg.I64))
    # The allocating entry point runs on the library's own stream.
    torch.cuda.synchronize()
    return cols


def _expected(ctx, bk, pk, pv):
    j = qeg.Join(ctx, [qeg.I64, qeg.I64], [qeg.I64], [0], [0], strategy=qeg.JOIN_HASH)
    j.build([bk])
    j.build_finish()
    j.probe_count_sum(pk, pv)
    res = j.count_sum()
    j.close()
    return res


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    ctx = qeg.Context(0)
    try:
        out = torch.zeros(4, dtype=torch.int64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        cases = [_case(torch, 1, 1 << 18, 1 << 22, dup=False), _case(torch, 2, 1 << 20, 1 << 21, dup=True)]
        for bk, pk, pv in cases:
            exp = _expected(ctx, bk, pk, pv)
            qeg.join_count_sum_noalloc(stream, bk, pk, pv, out)
            torch.cuda.synchronize()
            got = out.cpu().tolist()
            assert got[3] == 0, "scratch table overflow reported"
            assert (got[0], got[1] if got[2] else None) == exp
    finally:
        ctx.close()


def test_noalloc_rejects_build_beyond_limit():
    torch = pytest.importorskip("torch")
    n = (1 << 20) + 1
    bk = qeg.Col(torch.zeros(n, dtype=torch.int64, device="cuda"), None, qeg.I64)
    pk = qeg.Col(torch.zeros(4, dtype=torch.int64, device="cuda"), None, qeg.I64)
    out = torch.zeros(4, dtype=torch.int64, device="cuda")
    with pytest.raises(qeg.QegError) as e:
        qeg.join_count_sum_noalloc(torch.cuda.current_stream().cuda_stream, bk, pk, pk, out)
    assert e.value.code == -1 and "1048576" in str(e.value)
