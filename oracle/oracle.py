"""TEST INFRASTRUCTURE, NOT PRODUCT CODE.

ctypes binding of the CPU oracle (oracle/liboracle.so, a restatement of the
reference engine's hash GROUP BY / hash join semantics) and, where it was built,
of the reference engine itself (oracle/_ref/libqe_ref.so). Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.

It also restates the reference's result comparator (oracle/result_set.cpp:49-187
of the reference): both sides canonicalised by sorting on all columns (NULL
first, NaN greatest), integer-family cells compared exactly, F64 cells within
|a-b| <= 1e-9 + 1e-9*max(|a|,|b|) (oracle/result_set.h:53-54), NaN == NaN.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqe_ref.so")

I32, I64, F64, BOOL, TS, STR = 0, 1, 2, 3, 4, 5
COUNT_STAR, COUNT, SUM, MIN, MAX, AVG = 0, 1, 2, 3, 4, 5
INNER, LEFT = 0, 1
ABS_EPS = 1e-9
REL_EPS = 1e-9


class OrcColumn(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("len", ctypes.c_uint64), ("data", ctypes.c_void_p),
                ("validity", ctypes.c_void_p), ("all_valid", ctypes.c_int32),
                ("dict_offsets", ctypes.c_void_p), ("dict_bytes", ctypes.c_void_p),
                ("dict_size", ctypes.c_uint32)]


class TCol:
    """A host column for the oracle: numpy values, optional bool validity mask,
    and for STR a list of dictionary strings (values are int32 codes)."""

    def __init__(self, type, values, valid=None, dictionary=None):
        self.type = type
        self.values = np.ascontiguousarray(values)
        self.valid = None if valid is None else np.asarray(valid, dtype=bool)
        self.dictionary = dictionary
        self._keep = []

    @property
    def n(self):
        return len(self.values)

    def words(self):
        if self.valid is None:
            return None
        nw = (self.n + 63) // 64
        padded = np.ones(max(nw, 1) * 64, dtype=bool)
        padded[: self.n] = self.valid
        return np.packbits(padded, bitorder="little").view(np.uint64).copy()

    def orc(self):
        w = self.words()
        self._keep = [w]
        offs = bytes_ = None
        size = 0
        if self.type == STR:
            enc = [s.encode() for s in self.dictionary]
            offs = np.zeros(len(enc) + 1, dtype=np.uint32)
            offs[1:] = np.cumsum([len(e) for e in enc])
            bytes_ = np.frombuffer(b"".join(enc) + b"\0", dtype=np.uint8)
            size = len(enc)
            self._keep += [offs, bytes_]
        return OrcColumn(self.type, self.n, self.values.ctypes.data if self.n else None,
                         None if w is None else w.ctypes.data, 1 if w is None else 0,
                         None if offs is None else offs.ctypes.data,
                         None if bytes_ is None else bytes_.ctypes.data, size)


def build(ref=False):
    """Builds liboracle.so (and the reference library when ref=True and the
    reference sources are present)."""
    subprocess.run(["make", "-C", HERE, "-s", "liboracle.so"], check=True)
    if ref and os.path.isdir(os.environ.get("REF_ROOT", "/root/reference")):
        subprocess.run(["make", "-C", HERE, "-s", "-j8", "ref"], check=True)


_orc = None
_ref = None


def _bind(L, prefix):
    vp, u64, i32, c, P = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int, ctypes.POINTER
    common = {
        prefix + "_result_rows": (u64, [vp]),
        prefix + "_result_cols": (c, [vp]),
        prefix + "_result_type": (i32, [vp, c]),
        prefix + "_result_fetch": (c, [vp, c, vp, vp, vp]),
        prefix + "_result_free": (None, [vp]),
        prefix + "_last_error": (ctypes.c_char_p, []),
        prefix + "_hash_combine": (u64, [u64, u64]),
    }
    for name, (r, a) in common.items():
        f = getattr(L, name)
        f.restype, f.argtypes = r, a


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        _bind(L, "orc")
        vp, u64, i32, c, P = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int, ctypes.POINTER
        for name, (r, a) in {
            "orc_groupby": (c, [vp, c, vp, c, vp, vp, c, u64, P(vp)]),
            "orc_join": (c, [vp, c, vp, c, vp, vp, c, i32, u64, P(vp)]),
            "orc_join_count_sum": (c, [vp, vp, vp, u64, P(ctypes.c_int64), P(ctypes.c_int64), P(i32)]),
            "orc_parallel_groupby": (c, [vp, c, vp, c, vp, vp, c, ctypes.c_uint, u64, P(vp)]),
            "orc_parallel_join_count_sum": (c, [vp, vp, vp, vp, ctypes.c_uint, u64, P(ctypes.c_int64),
                                                P(ctypes.c_int64), P(i32)]),
            "orc_result_str": (c, [vp, c, ctypes.c_int64, P(ctypes.c_char_p), P(u64)]),
            "orc_window_tumbling": (c, [vp, c, vp, c, ctypes.c_uint32, ctypes.c_int64, vp, vp, c, u64, P(vp)]),
            "orc_asof_join": (c, [vp, c, vp, c, vp, vp, c, ctypes.c_uint32, ctypes.c_uint32, i32, i32,
                                  ctypes.c_int64, P(vp)]),
        }.items():
            f = getattr(L, name)
            f.restype, f.argtypes = r, a
        _orc = L
    return _orc


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        _bind(L, "ref")
        vp, u64, i32, c, P = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int, ctypes.POINTER
        for name, (r, a) in {
            "ref_groupby": (c, [vp, c, vp, c, vp, vp, c, u64, c, ctypes.c_uint, P(vp)]),
            "ref_join": (c, [vp, c, vp, c, vp, vp, c, i32, u64, c, P(vp)]),
            "ref_parallel_join_count_sum": (c, [vp, vp, ctypes.c_uint, u64, P(ctypes.c_int64),
                                                P(ctypes.c_int64), P(i32)]),
            "ref_result_str": (c, [vp, c, u64, P(ctypes.c_char_p), P(u64)]),
            "ref_window_tumbling": (c, [vp, c, vp, c, ctypes.c_uint32, ctypes.c_int64, vp, vp, c, u64, c, P(vp)]),
            "ref_asof_join": (c, [vp, c, vp, c, vp, vp, c, ctypes.c_uint32, ctypes.c_uint32, i32, i32,
                                  ctypes.c_int64, u64, c, P(vp)]),
        }.items():
            f = getattr(L, name)
            f.restype, f.argtypes = r, a
        _ref = L
    return _ref


class OracleError(RuntimeError):
    pass


def _cols(cols):
    arr = (OrcColumn * max(1, len(cols)))()
    for i, c in enumerate(cols):
        arr[i] = c.orc()
    return arr


def _rows(L, prefix, res):
    """Materialises a result handle as a list of row tuples (None = NULL)."""
    get = lambda n: getattr(L, prefix + n)
    nr = get("_result_rows")(res)
    nc = get("_result_cols")(res)
    cols = []
    for c in range(nc):
        t = get("_result_type")(res, c)
        iv = np.zeros(max(nr, 1), dtype=np.int64)
        fv = np.zeros(max(nr, 1), dtype=np.float64)
        ok = np.zeros(max(nr, 1), dtype=np.uint8)
        get("_result_fetch")(res, c, iv.ctypes.data, fv.ctypes.data, ok.ctypes.data)
        vals = []
        for r in range(nr):
            if not ok[r]:
                vals.append(None)
            elif t == F64:
                vals.append(float(fv[r]))
            elif t == STR:
                s = ctypes.c_char_p()
                ln = ctypes.c_uint64()
                if prefix == "orc":
                    get("_result_str")(res, c, int(iv[r]), ctypes.byref(s), ctypes.byref(ln))
                else:
                    get("_result_str")(res, c, r, ctypes.byref(s), ctypes.byref(ln))
                vals.append(ctypes.string_at(s, ln.value).decode())
            else:
                vals.append(int(iv[r]))
        cols.append((t, vals))
    get("_result_free")(res)
    types = [t for t, _ in cols]
    rows = list(zip(*[v for _, v in cols])) if cols else []
    return types, rows


def _check(L, prefix, st):
    if st != 0:
        raise OracleError(getattr(L, prefix + "_last_error")().decode())


def _agg_arrays(keys, aggs):
    k = (ctypes.c_uint32 * max(1, len(keys)))(*keys)
    f = (ctypes.c_int32 * len(aggs))(*[a[0] for a in aggs])
    c = (ctypes.c_uint32 * len(aggs))(*[a[1] for a in aggs])
    return k, f, c


def groupby(cols, keys, aggs, batch_rows=2048):
    """The oracle's GROUP BY: returns (types, rows) in first-seen group order."""
    L = orc()
    arr = _cols(cols)
    k, f, c = _agg_arrays(keys, aggs)
    res = ctypes.c_void_p()
    _check(L, "orc", L.orc_groupby(arr, len(cols), k, len(keys), f, c, len(aggs), batch_rows, ctypes.byref(res)))
    return _rows(L, "orc", res)


def parallel_groupby(cols, keys, aggs, threads=0, morsel_rows=1024):
    L = orc()
    arr = _cols(cols)
    k, f, c = _agg_arrays(keys, aggs)
    res = ctypes.c_void_p()
    _check(L, "orc", L.orc_parallel_groupby(arr, len(cols), k, len(keys), f, c, len(aggs), threads,
                                            morsel_rows, ctypes.byref(res)))
    return _rows(L, "orc", res)


def join(probe, build_, pkeys, bkeys, jtype=INNER, batch_rows=2048):
    L = orc()
    pa, ba = _cols(probe), _cols(build_)
    pk = (ctypes.c_uint32 * len(pkeys))(*pkeys)
    bk = (ctypes.c_uint32 * len(bkeys))(*bkeys)
    res = ctypes.c_void_p()
    _check(L, "orc", L.orc_join(pa, len(probe), ba, len(build_), pk, bk, len(pkeys), jtype, batch_rows,
                                ctypes.byref(res)))
    return _rows(L, "orc", res)


def window_tumbling(cols, keys, time_col, width, aggs, batch_rows=2048):
    """GROUP BY (keys..., (t / width) * width of time_col): the tumbling Window."""
    L = orc()
    arr = _cols(cols)
    k, f, c = _agg_arrays(keys, aggs)
    res = ctypes.c_void_p()
    _check(L, "orc", L.orc_window_tumbling(arr, len(cols), k, len(keys), time_col, width, f, c, len(aggs),
                                           batch_rows, ctypes.byref(res)))
    return _rows(L, "orc", res)


def asof_join(probe, build_, pkeys, bkeys, ptime, btime, jtype=INNER, tolerance=None):
    """Backward as-of join: probe columns then build columns."""
    L = orc()
    pa, ba = _cols(probe), _cols(build_)
    pk = (ctypes.c_uint32 * max(1, len(pkeys)))(*pkeys)
    bk = (ctypes.c_uint32 * max(1, len(bkeys)))(*bkeys)
    res = ctypes.c_void_p()
    _check(L, "orc", L.orc_asof_join(pa, len(probe), ba, len(build_), pk, bk, len(pkeys), ptime, btime, jtype,
                                     0 if tolerance is None else 1, 0 if tolerance is None else int(tolerance),
                                     ctypes.byref(res)))
    return _rows(L, "orc", res)


def join_count_sum(pkey, pval, bkey):
    L = orc()
    a, b, c = pkey.orc(), pval.orc(), bkey.orc()
    n, s, ok = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    _check(L, "orc", L.orc_join_count_sum(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), 2048,
                                          ctypes.byref(n), ctypes.byref(s), ctypes.byref(ok)))
    return n.value, (s.value if ok.value else None)


def parallel_join_count_sum(pkey, pval, bkey, bval, threads=0, morsel_rows=1024):
    L = orc()
    a, b, c, d = pkey.orc(), pval.orc(), bkey.orc(), bval.orc()
    n, s, ok = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    _check(L, "orc", L.orc_parallel_join_count_sum(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                   ctypes.byref(d), threads, morsel_rows, ctypes.byref(n),
                                                   ctypes.byref(s), ctypes.byref(ok)))
    return n.value, (s.value if ok.value else None)


def ref_groupby(cols, keys, aggs, batch_rows=2048, mode=0, threads=0):
    """The reference engine's own GROUP BY (mode 0 operator tree, 1 its
    independent reference oracle, 2 its morsel-parallel engine)."""
    L = ref()
    arr = _cols(cols)
    k, f, c = _agg_arrays(keys, aggs)
    res = ctypes.c_void_p()
    _check(L, "ref", L.ref_groupby(arr, len(cols), k, len(keys), f, c, len(aggs), batch_rows, mode, threads,
                                   ctypes.byref(res)))
    return _rows(L, "ref", res)


def ref_join(probe, build_, pkeys, bkeys, jtype=INNER, batch_rows=2048, mode=0):
    L = ref()
    pa, ba = _cols(probe), _cols(build_)
    pk = (ctypes.c_uint32 * len(pkeys))(*pkeys)
    bk = (ctypes.c_uint32 * len(bkeys))(*bkeys)
    res = ctypes.c_void_p()
    _check(L, "ref", L.ref_join(pa, len(probe), ba, len(build_), pk, bk, len(pkeys), jtype, batch_rows, mode,
                                ctypes.byref(res)))
    return _rows(L, "ref", res)


def ref_window_tumbling(cols, keys, time_col, width, aggs, batch_rows=2048, mode=0):
    """The reference's tumbling Window (mode 0 operator tree, 1 its
    independent reference oracle)."""
    L = ref()
    arr = _cols(cols)
    k, f, c = _agg_arrays(keys, aggs)
    res = ctypes.c_void_p()
    _check(L, "ref", L.ref_window_tumbling(arr, len(cols), k, len(keys), time_col, width, f, c, len(aggs),
                                           batch_rows, mode, ctypes.byref(res)))
    return _rows(L, "ref", res)


def ref_asof_join(probe, build_, pkeys, bkeys, ptime, btime, jtype=INNER, tolerance=None, batch_rows=2048,
                  mode=0):
    """The reference's AsofJoin (mode 0 operator tree, 1 its independent
    reference oracle)."""
    L = ref()
    pa, ba = _cols(probe), _cols(build_)
    pk = (ctypes.c_uint32 * max(1, len(pkeys)))(*pkeys)
    bk = (ctypes.c_uint32 * max(1, len(bkeys)))(*bkeys)
    res = ctypes.c_void_p()
    _check(L, "ref", L.ref_asof_join(pa, len(probe), ba, len(build_), pk, bk, len(pkeys), ptime, btime, jtype,
                                     0 if tolerance is None else 1, 0 if tolerance is None else int(tolerance),
                                     batch_rows, mode, ctypes.byref(res)))
    return _rows(L, "ref", res)


# ---------------------------------------------------------------------------
# Comparator (restates the reference's compare_result_sets)
# ---------------------------------------------------------------------------
def _cell_key(v, t):
    if v is None:
        return (0,)
    if t == F64:
        if math.isnan(v):
            return (1, 1, 0.0)
        return (1, 0, v)
    return (1, v)


def canonical(types, rows):
    return sorted(rows, key=lambda r: tuple(_cell_key(v, t) for v, t in zip(r, types)))


def float_eq(a, b):
    if math.isnan(a) and math.isnan(b):
        return True
    if a == b:
        return True
    return abs(a - b) <= ABS_EPS + REL_EPS * max(abs(a), abs(b))


def compare(types_a, rows_a, types_b, rows_b):
    """Returns None when equal under the reference's rules, else a message."""
    if list(types_a) != list(types_b):
        return "column type/shape mismatch: %s vs %s" % (types_a, types_b)
    if len(rows_a) != len(rows_b):
        return "row count mismatch: %d vs %d" % (len(rows_a), len(rows_b))
    ca, cb = canonical(types_a, rows_a), canonical(types_b, rows_b)
    for i, (ra, rb) in enumerate(zip(ca, cb)):
        for c, t in enumerate(types_a):
            a, b = ra[c], rb[c]
            if (a is None) != (b is None):
                return "null mismatch at canonical row %d col %d: %r vs %r" % (i, c, a, b)
            if a is None:
                continue
            same = float_eq(a, b) if t == F64 else a == b
            if not same:
                return "value mismatch at canonical row %d col %d: %r vs %r" % (i, c, a, b)
    return None
