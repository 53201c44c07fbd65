"""The GPU path against the golden vectors produced by the reference engine
(tests/golden/golden.json): every GROUP BY, join, tumbling-window and as-of
case, through the C ABI.
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
    elif case["kind"] == "window":
        cols = [dec_col(c) for c in case["columns"]]
        w = qeg.Window(ctx, [c.type for c in cols], case["keys"], case["time_col"], case["width"],
                       [tuple(a) for a in case["aggs"]])
        w.consume([to_gpu(c) for c in cols])
        w.finish()
        gt, rows = gpu_rows(w.fetch(), types)
        w.close()
    else:
        probe = [dec_col(c) for c in case["probe"]]
        build = [dec_col(c) for c in case["build"]]
        canon = StrCanon([s for c in probe + build if c.dictionary for s in c.dictionary])
        if case["kind"] == "asof":
            j = qeg.AsofJoin(ctx, [c.type for c in probe], [c.type for c in build], case["probe_keys"],
                             case["build_keys"], case["probe_time"], case["build_time"], case["join_type"],
                             case["tolerance"])
        else:
            j = qeg.Join(ctx, [c.type for c in probe], [c.type for c in build], case["probe_keys"],
                         case["build_keys"], case["join_type"])
        j.build([to_gpu(c, canon) for c in build])
        j.build_finish()
        n = j.probe([to_gpu(c, canon) for c in probe])
        gt, rows = gpu_rows(j.fetch(0, n), types, canon) if n else (types, [])
        j.close()
    assert_same(gt, rows, types, exp, case["name"])
