"""Python binding of the qeg C ABI (include/qeg.h) through ctypes.

Columns are numpy arrays (host memory: copied to the GPU inside each call) or
torch CUDA tensors (device memory: used in place). The library is loaded from
query-engine_gb300/libqeg.so; a missing library raises, there is no fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "libqeg.so")

I32, I64, F64, BOOL, TS, STR = 0, 1, 2, 3, 4, 5
COUNT_STAR, COUNT, SUM, MIN, MAX, AVG = 0, 1, 2, 3, 4, 5
INNER, LEFT = 0, 1
AGG_AUTO, AGG_SMEM, AGG_GLOBAL, AGG_PARTITIONED = 0, 1, 2, 3
SIZE_LEARNED, SIZE_FIXED = 0, 1
JOIN_AUTO, JOIN_HASH, JOIN_PARTITIONED, JOIN_DENSE = 0, 1, 2, 3

WIDTH = {I32: 4, I64: 8, F64: 8, BOOL: 1, TS: 8, STR: 4}
NP_DTYPE = {I32: np.int32, I64: np.int64, F64: np.float64, BOOL: np.uint8, TS: np.int64, STR: np.int32}

STATUS = {0: "OK", -1: "INVALID", -2: "OVERFLOW", -3: "OOM", -4: "CUDA", -5: "TIMEOUT",
          -6: "UNSUPPORTED", -7: "NO_DEVICE"}


class QegError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class Column(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("all_valid", ctypes.c_int32), ("len", ctypes.c_uint64),
                ("data", ctypes.c_void_p), ("validity", ctypes.c_void_p),
                ("code_map", ctypes.c_void_p), ("code_map_len", ctypes.c_uint64)]


class OutColumn(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("validity", ctypes.c_void_p), ("all_valid", ctypes.c_void_p)]


class AggSpec(ctypes.Structure):
    _fields_ = [("func", ctypes.c_int32), ("input_col", ctypes.c_uint32)]


class AggConfig(ctypes.Structure):
    _fields_ = [("strategy", ctypes.c_int32), ("sizing", ctypes.c_int32),
                ("initial_capacity", ctypes.c_uint64), ("expected_groups", ctypes.c_uint64),
                ("block_threads", ctypes.c_int32), ("rows_per_thread", ctypes.c_int32),
                ("smem_slots", ctypes.c_int32), ("hot_keys", ctypes.c_int32)]


class JoinConfig(ctypes.Structure):
    _fields_ = [("strategy", ctypes.c_int32), ("partition_bits", ctypes.c_int32), ("sizing", ctypes.c_int32)]


_lib = None


def lib():
    """Loads libqeg.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libqeg.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, i32, c = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int
        P = ctypes.POINTER
        sig = {
            "qeg_ctx_create": (i32, [c, P(vp)]),
            "qeg_ctx_destroy": (None, [vp]),
            "qeg_last_error": (ctypes.c_char_p, [vp]),
            "qeg_ctx_stream": (vp, [vp]),
            "qeg_ctx_synchronize": (i32, [vp]),
            "qeg_ctx_kernel_launches": (u64, [vp]),
            "qeg_agg_create": (i32, [vp, vp, c, vp, c, vp, c, vp, P(vp)]),
            "qeg_agg_consume": (i32, [vp, vp, c, vp, u64]),
            "qeg_agg_finish": (i32, [vp, P(u64)]),
            "qeg_agg_result_types": (i32, [vp, vp]),
            "qeg_agg_fetch": (i32, [vp, u64, u64, vp]),
            "qeg_agg_stats": (i32, [vp, P(u64), P(ctypes.c_uint32), P(i32), P(i32), P(ctypes.c_double)]),
            "qeg_agg_destroy": (None, [vp]),
        }
        optional = {
            "qeg_join_create": (i32, [vp, vp, c, vp, c, vp, vp, c, i32, vp, P(vp)]),
            "qeg_asof_create": (i32, [vp, vp, c, vp, c, vp, vp, c, ctypes.c_uint32, ctypes.c_uint32, i32, i32,
                                      ctypes.c_int64, P(vp)]),
            "qeg_window_create": (i32, [vp, vp, c, vp, c, ctypes.c_uint32, ctypes.c_int64, vp, c, vp, P(vp)]),
            "qeg_join_build": (i32, [vp, vp, c]),
            "qeg_join_build_finish": (i32, [vp]),
            "qeg_join_probe": (i32, [vp, vp, c, P(u64)]),
            "qeg_join_fetch": (i32, [vp, u64, u64, vp]),
            "qeg_join_probe_count_sum": (i32, [vp, vp, vp]),
            "qeg_join_count_sum_result": (i32, [vp, P(ctypes.c_int64), P(ctypes.c_int64), P(i32)]),
            "qeg_join_stats": (i32, [vp, P(i32), P(i32), P(u64)]),
            "qeg_join_sizing_stats": (i32, [vp, P(u64), P(ctypes.c_double), P(i32)]),
            "qeg_join_destroy": (None, [vp]),
            "qeg_join_count_sum_noalloc": (i32, [vp, vp, vp, vp, vp]),
            "qeg_ctx_check_bounded_wait": (i32, [vp, i32]),
            "qeg_filter_join_agg": (i32, [vp, vp, c, vp, c, vp, u64, vp, P(u64)]),
            "qeg_sketch": (i32, [vp, vp, u64, vp, P(ctypes.c_double), P(ctypes.c_double)]),
            "qeg_sketch_batch": (i32, [vp, vp, ctypes.c_uint32, vp, u64, vp, vp]),
            "qeg_estimator_init": (i32, [vp, u64]),
            "qeg_estimator_set_weights": (i32, [vp, vp]),
            "qeg_estimator_get_weights": (i32, [vp, vp]),
            "qeg_estimator_set_deadband": (i32, [vp, ctypes.c_double]),
            "qeg_estimator_get_deadband": (i32, [vp, P(ctypes.c_double)]),
            "qeg_estimator_predict": (i32, [vp, vp, ctypes.c_uint32, vp]),
            "qeg_estimator_grad": (i32, [vp, vp, vp, ctypes.c_uint32, P(ctypes.c_float), vp]),
            "qeg_estimator_train": (i32, [vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_float, u64, P(ctypes.c_float)]),
            "qeg_batch_create": (i32, [vp, ctypes.c_uint32, vp, vp, vp, vp, c, vp, c, c, P(vp)]),
            "qeg_batch_run": (i32, [vp]),
            "qeg_batch_finish": (i32, [vp, vp]),
            "qeg_batch_fetch": (i32, [vp, ctypes.c_uint32, vp]),
            "qeg_batch_stats": (i32, [vp, ctypes.c_uint32, P(ctypes.c_double), P(ctypes.c_float), P(i32),
                                      P(ctypes.c_uint32)]),
            "qeg_batch_destroy": (None, [vp]),
        }
        for name, (res, args) in list(sig.items()) + list(optional.items()):
            if not hasattr(L, name):
                if name in sig:
                    raise RuntimeError("libqeg.so lacks %s" % name)
                continue
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status, ctx_ptr):
    if status != 0:
        msg = lib().qeg_last_error(ctx_ptr)
        raise QegError(status, msg.decode() if msg else "")


def _ptr(a):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _len(a):
    return a.shape[0] if isinstance(a, np.ndarray) else a.numel()


def pack_validity(valid):
    """Packs a boolean mask (True = valid) into 64-bit LSB-first words."""
    valid = np.asarray(valid, dtype=bool)
    n = len(valid)
    nw = (n + 63) // 64
    padded = np.ones(nw * 64, dtype=bool)
    padded[:n] = valid
    return np.packbits(padded, bitorder="little").view(np.uint64).copy()


def unpack_validity(words, n):
    words = np.ascontiguousarray(words, dtype=np.uint64)
    b = words.view(np.uint8).reshape(-1, 8)
    bits = np.unpackbits(b, axis=1, bitorder="little").reshape(-1)
    return bits[:n].astype(bool)


class Col:
    """A column view: values (numpy or torch CUDA), optional validity words,
    optional STR code map. Keeps the referenced buffers alive."""

    def __init__(self, values, validity=None, type=None, code_map=None):
        self.values = values
        self.validity = validity
        self.code_map = code_map
        if type is None:
            dt = str(values.dtype)
            type = {"int32": I32, "torch.int32": I32, "int64": I64, "torch.int64": I64,
                    "float64": F64, "torch.float64": F64, "uint8": BOOL, "torch.uint8": BOOL,
                    "bool": BOOL, "torch.bool": BOOL}[dt]
        self.type = type
        self.n = _len(values)

    def c(self):
        cm = self.code_map
        return Column(self.type, 1 if self.validity is None else 0, self.n, _ptr(self.values),
                      _ptr(self.validity), _ptr(cm), 0 if cm is None else _len(cm))


def _cols(cols):
    arr = (Column * max(1, len(cols)))()
    for i, c in enumerate(cols):
        arr[i] = c.c()
    return arr


class Context:
    def __init__(self, device=0):
        p = ctypes.c_void_p()
        st = lib().qeg_ctx_create(device, ctypes.byref(p))
        if st != 0:
            msg = lib().qeg_last_error(None)
            raise QegError(st, msg.decode() if msg else "")
        self.p = p

    @property
    def stream(self):
        return lib().qeg_ctx_stream(self.p)

    def synchronize(self):
        _check(lib().qeg_ctx_synchronize(self.p), self.p)

    def check_bounded_wait(self, polls):
        """Runs the composite-key tables' bounded wait on a row that stays
        claimed (qeg_ctx_check_bounded_wait); raises QegError(TIMEOUT)."""
        _check(lib().qeg_ctx_check_bounded_wait(self.p, polls), self.p)

    @property
    def launches(self):
        return lib().qeg_ctx_kernel_launches(self.p)

    def close(self):
        if self.p:
            lib().qeg_ctx_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def agg_config(strategy=AGG_AUTO, sizing=SIZE_LEARNED, initial_capacity=0, expected_groups=0,
               block_threads=0, rows_per_thread=0, smem_slots=0, hot_keys=0):
    return AggConfig(strategy, sizing, initial_capacity, expected_groups, block_threads,
                     rows_per_thread, smem_slots, hot_keys)


class Aggregate:
    """The GPU GROUP BY operator state behind one qeg_agg."""

    def __init__(self, ctx, col_types, key_cols, aggs, config=None):
        self.ctx = ctx
        self.ncols = len(col_types)
        self.nkeys = len(key_cols)
        self.naggs = len(aggs)
        types = (ctypes.c_int32 * len(col_types))(*col_types)
        keys = (ctypes.c_uint32 * max(1, len(key_cols)))(*key_cols)
        specs = (AggSpec * max(1, len(aggs)))()
        for i, (f, c) in enumerate(aggs):
            specs[i] = AggSpec(f, c)
        cfg = config if config is not None else agg_config()
        p = ctypes.c_void_p()
        _check(lib().qeg_agg_create(ctx.p, types, len(col_types), keys, len(key_cols), specs,
                                    len(aggs), ctypes.byref(cfg), ctypes.byref(p)), ctx.p)
        self.p = p
        rt = (ctypes.c_int32 * (self.nkeys + self.naggs))()
        _check(lib().qeg_agg_result_types(p, rt), ctx.p)
        self.result_types = list(rt)
        self.rows = None

    def consume(self, cols, sel=None):
        arr = _cols(cols)
        _check(lib().qeg_agg_consume(self.p, arr, len(cols), _ptr(sel), 0 if sel is None else _len(sel)),
               self.ctx.p)

    def finish(self):
        n = ctypes.c_uint64()
        _check(lib().qeg_agg_finish(self.p, ctypes.byref(n)), self.ctx.p)
        self.rows = n.value
        return self.rows

    def fetch(self, first=0, count=None):
        """Returns [(values ndarray, valid bool ndarray)] for keys then aggregates."""
        if count is None:
            count = self.rows - first
        outs = (OutColumn * len(self.result_types))()
        keep = []
        for i, t in enumerate(self.result_types):
            v = np.zeros(max(count, 1), dtype=NP_DTYPE[t])
            w = np.zeros(max(1, (count + 63) // 64), dtype=np.uint64)
            av = np.zeros(1, dtype=np.int32)
            keep.append((v, w, av))
            outs[i] = OutColumn(v.ctypes.data, w.ctypes.data, av.ctypes.data)
        _check(lib().qeg_agg_fetch(self.p, first, count, outs), self.ctx.p)
        return [(v[:count], unpack_validity(w, count)) for v, w, _ in keep]

    def fetch_pinned(self, first=0, count=None, bufs=None):
        """Like fetch(), into page-locked host tensors (copied at the host
        link's speed): [(values, validity words)]. `bufs` (a previous result,
        large enough) is reused when given: pinning memory is slow."""
        import torch

        if count is None:
            count = self.rows - first
        tdt = {I32: torch.int32, I64: torch.int64, F64: torch.float64, BOOL: torch.uint8, TS: torch.int64,
               STR: torch.int32}
        if bufs is None or any(v.numel() < count for v, _ in bufs):
            bufs = [(torch.empty(max(count, 1), dtype=tdt[t], pin_memory=True),
                     torch.empty(max(1, (count + 63) // 64), dtype=torch.int64, pin_memory=True))
                    for t in self.result_types]
        outs = (OutColumn * len(self.result_types))()
        for i, (v, w) in enumerate(bufs):
            outs[i] = OutColumn(v.data_ptr(), w.data_ptr(), None)
        _check(lib().qeg_agg_fetch(self.p, first, count, outs), self.ctx.p)
        return bufs

    def fetch_torch(self, first=0, count=None):
        """Like fetch(), into torch CUDA tensors: [(values, validity words)]."""
        import torch

        if count is None:
            count = self.rows - first
        tdt = {I32: torch.int32, I64: torch.int64, F64: torch.float64, BOOL: torch.uint8, TS: torch.int64,
               STR: torch.int32}
        outs = (OutColumn * len(self.result_types))()
        keep = []
        for i, t in enumerate(self.result_types):
            v = torch.empty(max(count, 1), dtype=tdt[t], device="cuda")
            w = torch.empty(max(1, (count + 63) // 64), dtype=torch.int64, device="cuda")
            keep.append((v, w))
            outs[i] = OutColumn(v.data_ptr(), w.data_ptr(), None)
        # The library writes on its own stream: the new tensors' memory may
        # still be in use by torch's stream until it drains.
        torch.cuda.synchronize()
        _check(lib().qeg_agg_fetch(self.p, first, count, outs), self.ctx.p)
        return [(v[:count], w) for v, w in keep]

    def stats(self):
        cap, rs, st, hk, est = (ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_int32(),
                                ctypes.c_double())
        _check(lib().qeg_agg_stats(self.p, ctypes.byref(cap), ctypes.byref(rs), ctypes.byref(st),
                                   ctypes.byref(hk), ctypes.byref(est)), self.ctx.p)
        return {"capacity": cap.value, "resizes": rs.value, "strategy": st.value, "hot_keys": hk.value,
                "est_groups": est.value}

    def close(self):
        if self.p:
            lib().qeg_agg_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def groupby(ctx, cols, key_cols, aggs, config=None, batch_rows=None, sel=None):
    """Runs a whole GROUP BY: create, consume (in batches of batch_rows when
    given), finish, fetch. Returns [(values, valid)] keys then aggregates."""
    a = Aggregate(ctx, [c.type for c in cols], key_cols, aggs, config)
    try:
        n = cols[0].n if cols else 0
        if batch_rows is None or batch_rows >= n:
            a.consume(cols, sel)
        else:
            for s in range(0, n, batch_rows):
                e = min(n, s + batch_rows)
                part = []
                for c in cols:
                    v = c.values[s:e]
                    w = None
                    if c.validity is not None:
                        assert s % 64 == 0
                        w = c.validity[s // 64:(e + 63) // 64]
                    part.append(Col(v, w, c.type, c.code_map))
                a.consume(part)
        a.finish()
        return a.fetch()
    finally:
        a.close()


class Window(Aggregate):
    """Tumbling window (qeg_window_create): GROUP BY (key_cols..., bucket
    start of time_col with bucket width `width`); results are keys, the bucket
    start (typed as the time column), then the aggregates."""

    def __init__(self, ctx, col_types, key_cols, time_col, width, aggs, config=None):
        self.ctx = ctx
        self.ncols = len(col_types)
        self.nkeys = len(key_cols) + 1
        self.naggs = len(aggs)
        types = (ctypes.c_int32 * len(col_types))(*col_types)
        keys = (ctypes.c_uint32 * max(1, len(key_cols)))(*key_cols)
        specs = (AggSpec * max(1, len(aggs)))()
        for i, (f, c) in enumerate(aggs):
            specs[i] = AggSpec(f, c)
        cfg = config if config is not None else agg_config()
        p = ctypes.c_void_p()
        _check(lib().qeg_window_create(ctx.p, types, len(col_types), keys, len(key_cols), time_col, width, specs,
                                       len(aggs), ctypes.byref(cfg), ctypes.byref(p)), ctx.p)
        self.p = p
        rt = (ctypes.c_int32 * (self.nkeys + self.naggs))()
        _check(lib().qeg_agg_result_types(p, rt), ctx.p)
        self.result_types = list(rt)
        self.rows = None


class Join:
    """The GPU hash-join operator state behind one qeg_join."""

    def __init__(self, ctx, probe_types, build_types, probe_keys, build_keys, join_type=INNER,
                 strategy=JOIN_AUTO, partition_bits=0, sizing=SIZE_LEARNED):
        self.ctx = ctx
        self.probe_types = list(probe_types)
        self.build_types = list(build_types)
        pt = (ctypes.c_int32 * max(1, len(probe_types)))(*probe_types)
        bt = (ctypes.c_int32 * max(1, len(build_types)))(*build_types)
        pk = (ctypes.c_uint32 * len(probe_keys))(*probe_keys)
        bk = (ctypes.c_uint32 * len(build_keys))(*build_keys)
        cfg = JoinConfig(strategy, partition_bits, sizing)
        p = ctypes.c_void_p()
        _check(lib().qeg_join_create(ctx.p, pt, len(probe_types), bt, len(build_types), pk, bk,
                                     len(probe_keys), join_type, ctypes.byref(cfg), ctypes.byref(p)), ctx.p)
        self.p = p
        self.rows = 0

    def build(self, cols):
        _check(lib().qeg_join_build(self.p, _cols(cols), len(cols)), self.ctx.p)

    def build_finish(self):
        _check(lib().qeg_join_build_finish(self.p), self.ctx.p)

    def probe(self, cols):
        n = ctypes.c_uint64()
        _check(lib().qeg_join_probe(self.p, _cols(cols), len(cols), ctypes.byref(n)), self.ctx.p)
        self.rows = n.value
        return self.rows

    def fetch(self, first=0, count=None):
        if count is None:
            count = self.rows - first
        types = self.probe_types + self.build_types
        outs = (OutColumn * len(types))()
        keep = []
        for i, t in enumerate(types):
            v = np.zeros(max(count, 1), dtype=NP_DTYPE[t])
            w = np.zeros(max(1, (count + 63) // 64), dtype=np.uint64)
            av = np.zeros(1, dtype=np.int32)
            keep.append((v, w, av))
            outs[i] = OutColumn(v.ctypes.data, w.ctypes.data, av.ctypes.data)
        _check(lib().qeg_join_fetch(self.p, first, count, outs), self.ctx.p)
        return [(v[:count], unpack_validity(w, count)) for v, w, _ in keep]

    def fetch_pinned(self, first=0, count=None, bufs=None):
        """Like fetch(), into page-locked host tensors [(values, validity
        words)]: gathered on the device in row chunks, copied at the host
        link's speed. `bufs` (a previous result, large enough) is reused when
        given: pinning memory is slow."""
        import torch

        if count is None:
            count = self.rows - first
        types = self.probe_types + self.build_types
        tdt = {I32: torch.int32, I64: torch.int64, F64: torch.float64, BOOL: torch.uint8, TS: torch.int64,
               STR: torch.int32}
        if bufs is None or any(v.numel() < count for v, _ in bufs):
            bufs = [(torch.empty(max(count, 1), dtype=tdt[t], pin_memory=True),
                     torch.empty(max(1, (count + 63) // 64), dtype=torch.int64, pin_memory=True)) for t in types]
        outs = (OutColumn * len(types))()
        for i, (v, w) in enumerate(bufs):
            outs[i] = OutColumn(v.data_ptr(), w.data_ptr(), None)
        _check(lib().qeg_join_fetch(self.p, first, count, outs), self.ctx.p)
        return bufs

    def fetch_device(self, first=0, count=None, bufs=None, flags=None):
        """Like fetch(), into torch CUDA tensors [(values, validity words)]:
        one gather pass per column straight into them. `bufs` (a previous
        result, large enough) is reused when given; a validity entry of None
        asks for no words. `flags` (a list) receives each column's all-valid
        flag."""
        import torch

        if count is None:
            count = self.rows - first
        types = self.probe_types + self.build_types
        tdt = {I32: torch.int32, I64: torch.int64, F64: torch.float64, BOOL: torch.uint8, TS: torch.int64,
               STR: torch.int32}
        if bufs is None:
            bufs = [(torch.empty(max(count, 1), dtype=tdt[t], device="cuda"),
                     torch.empty(max(1, (count + 63) // 64), dtype=torch.int64, device="cuda")) for t in types]
            torch.cuda.synchronize()  # the library writes them on its own stream
        outs = (OutColumn * len(types))()
        av = (ctypes.c_int32 * len(types))()
        for i, (v, w) in enumerate(bufs):
            outs[i] = OutColumn(v.data_ptr(), None if w is None else w.data_ptr(),
                                ctypes.addressof(av) + 4 * i)
        _check(lib().qeg_join_fetch(self.p, first, count, outs), self.ctx.p)
        if flags is not None:
            flags[:] = [bool(x) for x in av]
        return bufs

    def probe_count_sum(self, key, val):
        k, v = Column(), Column()
        k, v = key.c(), val.c()
        _check(lib().qeg_join_probe_count_sum(self.p, ctypes.byref(k), ctypes.byref(v)), self.ctx.p)

    def count_sum(self):
        c, s, ok = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        _check(lib().qeg_join_count_sum_result(self.p, ctypes.byref(c), ctypes.byref(s), ctypes.byref(ok)),
               self.ctx.p)
        return c.value, (s.value if ok.value else None)

    def stats(self):
        st, pb, dk = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint64()
        _check(lib().qeg_join_stats(self.p, ctypes.byref(st), ctypes.byref(pb), ctypes.byref(dk)), self.ctx.p)
        out = {"strategy": st.value, "partition_bits": pb.value, "distinct_keys": dk.value}
        slots, est, rb = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_int32()
        _check(lib().qeg_join_sizing_stats(self.p, ctypes.byref(slots), ctypes.byref(est), ctypes.byref(rb)),
               self.ctx.p)
        out.update({"slots": slots.value, "est_distinct": est.value, "rebuilds": rb.value})
        return out

    def close(self):
        if self.p:
            lib().qeg_join_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AsofJoin(Join):
    """Backward as-of join (qeg_asof_create): per probe row the build row of
    the same key with the greatest time <= the probe's time (within
    `tolerance` when given). build / build_finish / probe / fetch as Join."""

    def __init__(self, ctx, probe_types, build_types, probe_keys, build_keys, probe_time, build_time,
                 asof_type=INNER, tolerance=None):
        self.ctx = ctx
        self.probe_types = list(probe_types)
        self.build_types = list(build_types)
        pt = (ctypes.c_int32 * max(1, len(probe_types)))(*probe_types)
        bt = (ctypes.c_int32 * max(1, len(build_types)))(*build_types)
        pk = (ctypes.c_uint32 * max(1, len(probe_keys)))(*probe_keys)
        bk = (ctypes.c_uint32 * max(1, len(build_keys)))(*build_keys)
        p = ctypes.c_void_p()
        self.p = None
        _check(lib().qeg_asof_create(ctx.p, pt, len(probe_types), bt, len(build_types), pk, bk, len(probe_keys),
                                     probe_time, build_time, asof_type, 0 if tolerance is None else 1,
                                     0 if tolerance is None else int(tolerance), ctypes.byref(p)), ctx.p)
        self.p = p
        self.rows = 0


def join_count_sum_noalloc(stream, build_key, probe_key, probe_val, out):
    """The join COUNT/SUM sink without device allocation (see include/qeg.h).
    All columns and `out` (4 int64 on the device) must be device tensors; the
    work is enqueued on `stream` (a cudaStream_t handle) without a sync."""
    b, k, v = build_key.c(), probe_key.c(), probe_val.c()
    st = lib().qeg_join_count_sum_noalloc(stream, ctypes.byref(b), ctypes.byref(k), ctypes.byref(v), _ptr(out))
    if st != 0:
        msg = lib().qeg_last_error(None)
        raise QegError(st, msg.decode() if msg else "")


# ---- fused filter -> join -> GROUP BY ---------------------------------------
CMP_LT, CMP_LE, CMP_GT, CMP_GE, CMP_EQ, CMP_NE = 0, 1, 2, 3, 4, 5


class PipelineDesc(ctypes.Structure):
    _fields_ = [("filter_col", ctypes.c_int32), ("filter_op", ctypes.c_int32), ("filter_value", ctypes.c_double),
                ("probe_key", ctypes.c_uint32), ("build_key", ctypes.c_uint32), ("group_col", ctypes.c_uint32),
                ("naggs", ctypes.c_int32), ("aggs", AggSpec * 16)]


def filter_join_agg(ctx, probe, build, probe_key, build_key, group_col, aggs, filter_col=-1, filter_op=CMP_GT,
                    filter_value=0.0, capacity=None):
    """scan(probe).filter(...).join(scan(build)).aggregate({group_col}, aggs)
    in one fused pass; returns [(values, valid)] group column then aggregates."""
    d = PipelineDesc()
    d.filter_col, d.filter_op, d.filter_value = filter_col, filter_op, filter_value
    d.probe_key, d.build_key, d.group_col, d.naggs = probe_key, build_key, group_col, len(aggs)
    for i, (f, c) in enumerate(aggs):
        d.aggs[i] = AggSpec(f, c)
    gtype = build[group_col - len(probe)].type
    types = [gtype]
    for f, c in aggs:
        t = probe[c].type if f not in (COUNT_STAR, COUNT) else I64
        types.append(I64 if f in (COUNT_STAR, COUNT) else F64 if f == AVG else
                     (F64 if t == F64 else I64) if f == SUM else t)
    cap = capacity or (build[0].n + 1)
    outs = (OutColumn * len(types))()
    keep = []
    for i, t in enumerate(types):
        v = np.zeros(max(cap, 1), dtype=NP_DTYPE[t])
        w = np.zeros(max(1, (cap + 63) // 64), dtype=np.uint64)
        keep.append((v, w))
        outs[i] = OutColumn(v.ctypes.data, w.ctypes.data, None)
    n = ctypes.c_uint64()
    _check(lib().qeg_filter_join_agg(ctx.p, _cols(probe), len(probe), _cols(build), len(build), ctypes.byref(d),
                                     cap, outs, ctypes.byref(n)), ctx.p)
    return types, [(v[:n.value], unpack_validity(w, n.value)) for v, w in keep]


# ---- sketch and learned estimator -------------------------------------------
SKETCH_FEATURES = 80
MLP_PARAMS = 9474


def sketch(ctx, col, sample_rows=0):
    """80 sketch features of a key column, the classic (non-learned) distinct
    estimate, and the sampled share of rows in the top-2048 candidates."""
    f = np.zeros(SKETCH_FEATURES, dtype=np.float32)
    g, s = ctypes.c_double(), ctypes.c_double()
    c = col.c()
    _check(lib().qeg_sketch(ctx.p, ctypes.byref(c), sample_rows, f.ctypes.data, ctypes.byref(g), ctypes.byref(s)),
           ctx.p)
    return f, g.value, s.value


def sketch_batch(ctx, col, row_offsets, sample_rows=0):
    """The batch planner's per-range sketch: (features [n, 80], classic [n])."""
    offs = np.ascontiguousarray(np.asarray(row_offsets, dtype=np.uint64))
    n = len(offs) - 1
    f = np.zeros((n, SKETCH_FEATURES), np.float32)
    c = np.zeros(n, np.float64)
    cc = col.c()
    _check(lib().qeg_sketch_batch(ctx.p, ctypes.byref(cc), n, offs.ctypes.data, sample_rows, f.ctypes.data,
                                  c.ctypes.data), ctx.p)
    return f, c


# The library's dead band on the network's log2 correction (kCorrectionDeadband
# in csrc/qeg_mlp.h).
CORRECTION_DEADBAND = 0.125


def learned_groups(classic, out0, deadband=CORRECTION_DEADBAND):
    """Group count from the classic estimate of a null-free key column and the
    network's first output, as the library computes it: log2(1 + g) =
    log2(1 + classic) + c, where c is 32 * out0 moved toward zero by the dead
    band (and 0 inside it)."""
    import math

    c = 32.0 * out0
    c = c - deadband if c > deadband else (c + deadband if c < -deadband else 0.0)
    return 2.0 ** min(40.0, max(0.0, math.log2(1.0 + max(classic, 0.0)) + c)) - 1.0


def estimator_init(ctx, seed):
    _check(lib().qeg_estimator_init(ctx.p, seed), ctx.p)


def estimator_set_weights(ctx, params):
    p = np.ascontiguousarray(params, dtype=np.float32)
    assert p.size == MLP_PARAMS
    _check(lib().qeg_estimator_set_weights(ctx.p, p.ctypes.data), ctx.p)


def estimator_set_deadband(ctx, band):
    _check(lib().qeg_estimator_set_deadband(ctx.p, band), ctx.p)


def estimator_get_deadband(ctx):
    b = ctypes.c_double(0)
    _check(lib().qeg_estimator_get_deadband(ctx.p, ctypes.byref(b)), ctx.p)
    return b.value


def estimator_get_weights(ctx):
    p = np.zeros(MLP_PARAMS, dtype=np.float32)
    _check(lib().qeg_estimator_get_weights(ctx.p, p.ctypes.data), ctx.p)
    return p


def estimator_predict(ctx, features):
    x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, SKETCH_FEATURES)
    y = np.zeros((x.shape[0], 2), dtype=np.float32)
    _check(lib().qeg_estimator_predict(ctx.p, x.ctypes.data, x.shape[0], y.ctypes.data), ctx.p)
    return y


def estimator_grad(ctx, x, t):
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, SKETCH_FEATURES)
    t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, 2)
    g = np.zeros(MLP_PARAMS, dtype=np.float32)
    loss = ctypes.c_float()
    _check(lib().qeg_estimator_grad(ctx.p, x.ctypes.data, t.ctypes.data, x.shape[0], ctypes.byref(loss),
                                    g.ctypes.data), ctx.p)
    return loss.value, g


def estimator_train(ctx, x, t, epochs, batch, lr, seed):
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, SKETCH_FEATURES)
    t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, 2)
    loss = ctypes.c_float()
    _check(lib().qeg_estimator_train(ctx.p, x.ctypes.data, t.ctypes.data, x.shape[0], epochs, batch, lr, seed,
                                     ctypes.byref(loss)), ctx.p)
    return loss.value


class BatchTuning(ctypes.Structure):
    _fields_ = [("max_log2_groups", ctypes.c_double), ("skewed", ctypes.c_int32), ("smem_slots", ctypes.c_int32),
                ("rows_per_item", ctypes.c_uint64), ("peer_rows", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Batch:
    """Many GROUP BY queries over slices of one (key, value) column pair, run
    by one persistent kernel from a captured CUDA graph (qeg_batch_*).
    `row_offsets` has nqueries + 1 ascending entries; `tuning` is a list of
    (max_log2_groups, skewed, smem_slots, rows_per_item[, peer_rows]) buckets."""

    def __init__(self, ctx, row_offsets, key, val, aggs, tuning=(), block_threads=0):
        self.ctx = ctx
        offs = np.ascontiguousarray(np.asarray(row_offsets, dtype=np.uint64))
        self.nq = len(offs) - 1
        specs = (AggSpec * max(1, len(aggs)))()
        for i, (f, c) in enumerate(aggs):
            specs[i] = AggSpec(f, c)
        tun = (BatchTuning * max(1, len(tuning)))()
        for i, t in enumerate(tuning):
            t = tuple(t) + (-1,) * (5 - len(t))  # peer_rows defaults to "decide from the estimate"
            tun[i] = BatchTuning(*t[:5], 0)
        self._keep = (key, val)  # the batch reads these buffers on every run
        kc, vc = key.c(), val.c()
        p = ctypes.c_void_p()
        _check(lib().qeg_batch_create(ctx.p, self.nq, offs.ctypes.data, ctypes.byref(kc), ctypes.byref(vc), specs,
                                      len(aggs), tun, len(tuning), block_threads, ctypes.byref(p)), ctx.p)
        self.p = p
        a = Aggregate(ctx, [key.type, val.type], [0], aggs)
        self.result_types = a.result_types
        a.close()
        self.aggs = list(aggs)
        self.groups = None

    def run(self):
        _check(lib().qeg_batch_run(self.p), self.ctx.p)

    def finish(self):
        g = np.zeros(self.nq, dtype=np.uint64)
        _check(lib().qeg_batch_finish(self.p, g.ctypes.data), self.ctx.p)
        self.groups = g
        return g

    def fetch(self, query):
        """Result of one query: [(values, valid)] for the key then the aggregates."""
        count = int(self.groups[query])
        outs = (OutColumn * len(self.result_types))()
        keep = []
        for i, t in enumerate(self.result_types):
            v = np.zeros(max(count, 1), dtype=NP_DTYPE[t])
            w = np.zeros(max(1, (count + 63) // 64), dtype=np.uint64)
            av = np.zeros(1, dtype=np.int32)
            keep.append((v, w, av))
            outs[i] = OutColumn(v.ctypes.data, w.ctypes.data, av.ctypes.data)
        _check(lib().qeg_batch_fetch(self.p, query, outs), self.ctx.p)
        return [(v[:count], unpack_validity(w, count)) for v, w, _ in keep]

    def stats(self, query):
        est, hot, st, fb = ctypes.c_double(), ctypes.c_float(), ctypes.c_int32(), ctypes.c_uint32()
        _check(lib().qeg_batch_stats(self.p, query, ctypes.byref(est), ctypes.byref(hot), ctypes.byref(st),
                                     ctypes.byref(fb)), self.ctx.p)
        return {"est_groups": est.value, "hot_share": hot.value, "strategy": st.value, "fell_back": fb.value}

    def close(self):
        if self.p:
            lib().qeg_batch_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
