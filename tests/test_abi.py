"""CPU-side checks of the drop-in boundary: libqeg.so loads and exports every
entry point include/qeg.h declares; the host-side validity packing matches
the reference's bitmap layout (core/validity.h:21-40 of the reference)."""
import ctypes
import os
import re
import subprocess

import numpy as np

import qeg

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(REPO, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(REPO, "include", h)).read()
            names |= set(re.findall(r"\b(qeg_[a-z0-9_]+)\s*\(", src))
    return names


def _ensure_built():
    if not os.path.exists(qeg.LIB_PATH):
        import build as qbuild

        qbuild.build()


def test_library_exports_every_declared_symbol():
    _ensure_built()
    L = ctypes.CDLL(qeg.LIB_PATH)
    missing = [n for n in sorted(_declared()) if not hasattr(L, n)]
    assert not missing, "declared in include/*.h but not exported: %s" % missing
    out = subprocess.run(["nm", "-D", "--defined-only", qeg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (qeg_[a-z0-9_]+)", out))
    assert _declared() <= exported


def test_context_without_gpu_reports_no_device():
    _ensure_built()
    try:
        import torch

        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    try:
        qeg.Context(0)
    except qeg.QegError as e:
        assert e.code == -7  # QEG_ERR_NO_DEVICE
    else:
        raise AssertionError("context creation without a GPU must fail loudly")


def test_validity_packing_layout():
    rng = np.random.default_rng(3)
    for n in (0, 1, 63, 64, 65, 200, 2048):
        v = rng.random(n) > 0.3
        w = qeg.pack_validity(v)
        assert len(w) == (n + 63) // 64
        for i in range(n):
            assert bool((int(w[i >> 6]) >> (i & 63)) & 1) == v[i]
        assert (qeg.unpack_validity(w, n) == v).all()
        if n % 64:
            assert int(w[-1]) >> (n % 64) == (1 << (64 - n % 64)) - 1  # padding bits set


def test_python_structs_match_the_c_layouts(tmp_path):
    """Every parameter struct the Python binding passes across the C ABI has
    the size and field offsets the C compiler gives include/qeg.h."""
    structs = {"qeg_column": qeg.Column, "qeg_out_column": qeg.OutColumn, "qeg_agg_spec": qeg.AggSpec,
               "qeg_agg_config": qeg.AggConfig, "qeg_join_config": qeg.JoinConfig,
               "qeg_pipeline_desc": qeg.PipelineDesc, "qeg_batch_tuning": qeg.BatchTuning}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qeg.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_device_table_entry_points_reject_a_null_context():
    """qeg_dev_alloc / qeg_dev_upload / qeg_dev_download check their arguments
    before any CUDA call: a NULL context is QEG_ERR_INVALID with the message in
    the thread's error slot, *out is left alone, and qeg_dev_free(NULL) is a
    no-op. (Runs without a GPU.)"""
    _ensure_built()
    L = ctypes.CDLL(qeg.LIB_PATH)
    L.qeg_last_error.restype = ctypes.c_char_p
    out = ctypes.c_void_p(1234)
    assert L.qeg_dev_alloc(None, ctypes.c_uint64(64), ctypes.byref(out)) == -1  # QEG_ERR_INVALID
    assert b"NULL" in L.qeg_last_error(None)
    assert out.value == 1234
    buf = ctypes.create_string_buffer(16)
    assert L.qeg_dev_upload(None, None, buf, ctypes.c_uint64(16)) == -1
    assert L.qeg_dev_download(None, buf, None, ctypes.c_uint64(16)) == -1
    L.qeg_dev_free(None)
