"""Shared helpers for the parity tests: seeded generators in the shape of the
reference's oracle generators (oracle/generators.h:125-135 of the reference:
bounded integer magnitudes so SUM fits in int64, finite F64 data, ~15% NULLs),
conversion of the same columns to the oracle and to the GPU C ABI, and the
conversion of GPU results to oracle-style rows."""
import math

import numpy as np

import oracle as O
import qeg

I32_ABS = 30000
I64_ABS = 1_000_000_000
F64_ABS = 1_000_000.0


def gen_column(rng, t, n, null_pct=15, card=None, dictionary=None):
    valid = None
    if null_pct > 0:
        valid = rng.random(n) >= null_pct / 100.0
    if t == O.I32:
        v = (rng.integers(-I32_ABS, I32_ABS + 1, n) if card is None else rng.integers(0, card, n)).astype(np.int32)
    elif t in (O.I64, O.TS):
        v = (rng.integers(-I64_ABS, I64_ABS + 1, n) if card is None else rng.integers(0, card, n)).astype(np.int64)
    elif t == O.F64:
        v = rng.uniform(-F64_ABS, F64_ABS, n) if card is None else rng.integers(0, card, n).astype(np.float64)
    elif t == O.BOOL:
        v = rng.integers(0, 2, n).astype(np.uint8)
    elif t == O.STR:
        v = rng.integers(0, len(dictionary), n).astype(np.int32)
        return O.TCol(t, v, valid, dictionary)
    else:
        raise ValueError(t)
    return O.TCol(t, v, valid)


def gen_schema(rng, min_cols=2, max_cols=5):
    n = int(rng.integers(min_cols, max_cols + 1))
    types = [int(rng.choice([O.I32, O.I64, O.F64, O.BOOL, O.TS])) for _ in range(n)]
    types[0] = int(rng.choice([O.I32, O.I64, O.F64]))
    return types


def gen_table(rng, types, n, null_pct=15):
    cols = []
    for t in types:
        card = int(rng.integers(1, 60)) if rng.random() < 0.6 else None
        cols.append(gen_column(rng, t, n, null_pct, card))
    return cols


def gen_group_by(rng, types):
    nk = int(rng.integers(0, 4))
    keys = [int(k) for k in rng.choice(len(types), min(nk, len(types)), replace=False)]
    aggs = []
    for _ in range(int(rng.integers(1, 5))):
        f = int(rng.integers(0, 6))
        c = int(rng.integers(0, len(types)))
        if f in (O.SUM, O.AVG) and types[c] == O.BOOL:
            f = O.COUNT
        aggs.append((f, c))
    return keys, aggs


class StrCanon:
    """Host-side STR canonicalisation: every dictionary code is mapped to a
    value id shared by all dictionaries, so equal strings compare equal
    (ops/aggregate.cpp:164-187, ops/join.cpp:48-71 of the reference). With a
    known universe of strings the ids are their sorted ranks, which makes them
    order-preserving, as MIN/MAX over STR (compared by value) requires."""

    def __init__(self, universe=None):
        self.ids = {}
        self.values = []
        for s in sorted(set(universe or [])):
            self.ids[s] = len(self.values)
            self.values.append(s)

    def code_map(self, dictionary):
        out = np.zeros(max(1, len(dictionary)), dtype=np.int32)
        for i, s in enumerate(dictionary):
            if s not in self.ids:
                self.ids[s] = len(self.values)
                self.values.append(s)
            out[i] = self.ids[s]
        return out


def to_gpu(col, canon=None, device=False):
    """An oracle TCol as a qeg.Col (host numpy buffers, or torch CUDA tensors)."""
    w = col.words()
    cm = None
    if col.type == O.STR:
        cm = canon.code_map(col.dictionary)
    vals = col.values
    if device:
        import torch

        vals = torch.from_numpy(np.ascontiguousarray(vals)).cuda()
        w = None if w is None else torch.from_numpy(w.view(np.int64)).cuda()
        cm = None if cm is None else torch.from_numpy(cm).cuda()
        torch.cuda.synchronize()  # the library reads them on its own stream
    return qeg.Col(vals, w, col.type, cm)


def gpu_rows(result, types, canon=None):
    """GPU result columns [(values, valid)] -> (types, rows) like the oracle's."""
    cols = []
    for (vals, valid), t in zip(result, types):
        out = []
        for v, ok in zip(vals.tolist(), valid.tolist()):
            if not ok:
                out.append(None)
            elif t == O.F64:
                out.append(float(v))
            elif t == O.STR:
                out.append(canon.values[int(v)])
            else:
                out.append(int(v))
        cols.append(out)
    n = len(cols[0]) if cols else 0
    return list(types), [tuple(c[i] for c in cols) for i in range(n)]


def assert_same(types_a, rows_a, types_b, rows_b, what=""):
    m = O.compare(types_a, rows_a, types_b, rows_b)
    assert m is None, "%s: %s" % (what, m)


def isnan(x):
    return isinstance(x, float) and math.isnan(x)
