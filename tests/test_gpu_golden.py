"""The GPU path against the golden vectors produced by the reference engine
(tests/golden/golden.json): every GROUP BY and join case, through the C ABI.
Output is unordered (both sides canonicalised); F64 within 1e-9 abs + rel."""
import pytest

import qeg
from golden_io import dec_col, dec_rows, load
from util import StrCanon, assert_same, gpu_rows, to_gpu

pytestmark = pytest.mark.gpu

G = load()


@pytest.mark.parametrize("case", G["cases"], ids=[c["name"] for c in G["cases"]])
def test_gpu_matches_reference_golden(ctx, case):
    types = case["types"]
    exp = dec_rows(types, case["rows"])
    if case["kind"] == "groupby":
        cols = [dec_col(c) for c in case["columns"]]
        canon = StrCanon([s for c in cols if c.dictionary for s in c.dictionary])
        aggs = [tuple(a) for a in case["aggs"]]
        res = qeg.groupby(ctx, [to_gpu(c, canon) for c in cols], case["keys"], aggs)
        gt, rows = gpu_rows(res, types, canon)
    else:
        probe = [dec_col(c) for c in case["probe"]]
        build = [dec_col(c) for c in case["build"]]
        canon = StrCanon([s for c in probe + build if c.dictionary for s in c.dictionary])
        j = qeg.Join(ctx, [c.type for c in probe], [c.type for c in build], case["probe_keys"], case["build_keys"],
                     case["join_type"])
        j.build([to_gpu(c, canon) for c in build])
        j.build_finish()
        n = j.probe([to_gpu(c, canon) for c in probe])
        gt, rows = gpu_rows(j.fetch(0, n), types, canon) if n else (types, [])
        j.close()
    assert_same(gt, rows, types, exp, case["name"])
