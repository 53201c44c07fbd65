"""Loads tests/golden/golden.json (generated from the reference engine by
tests/golden/make_golden.py) into oracle columns and expected rows."""
import json
import os

import numpy as np

import oracle as O

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")
DT = {O.I32: np.int32, O.I64: np.int64, O.F64: np.float64, O.BOOL: np.uint8, O.TS: np.int64, O.STR: np.int32}


def load():
    with open(PATH) as f:
        return json.load(f)


def dec_col(c):
    t = c["type"]
    vals = c["values"]
    if t == O.F64:
        vals = [float.fromhex(v) for v in vals]
    valid = None if c["valid"] is None else np.array(c["valid"], bool)
    return O.TCol(t, np.array(vals, dtype=DT[t]), valid, c["dictionary"])


def dec_rows(types, rows):
    out = []
    for r in rows:
        out.append(tuple(None if v is None else (float.fromhex(v) if t == O.F64 else v) for t, v in zip(types, r)))
    return out
