"""The GPU operators compiled and linked inside the reference tree.

tests/cpp/test_reference_lowering.cpp is built with QEG_WITH_REFERENCE_HEADERS
against the reference's own headers, linked with the reference engine compiled
from its sources (oracle/_ref/libqe_ref.so) and with libqeg.so, and run: it
lowers 60 plans of the reference's own plan generator both with the
reference's Plan::lower and with a lowering that puts the GPU operators in the
Aggregate / Join / tumbling Window / AsofJoin nodes, drains both with the
reference's drain_operator and compares them with its compare_result_sets.
Where no CUDA device is present the GPU trees are built (constructors, schema
checks) but not drained. Skipped where the reference's source tree or its
compiled library is absent.
"""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "query-engine_gb300")
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")
REF_LIB = os.path.join(REPO, "oracle", "_ref")


def _build():
    if not os.path.isdir(os.path.join(REF_ROOT, "plan")) or not os.path.exists(os.path.join(REF_LIB, "libqe_ref.so")):
        pytest.skip("the reference source tree or its compiled library is not present")
    if not os.path.exists(os.path.join(PKG, "libqeg.so")):
        pytest.skip("libqeg.so is not built")
    out = os.path.join(PKG, "_build", "test_reference_lowering")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++", "-std=c++20", "-O1", "-DQEG_WITH_REFERENCE_HEADERS",
           "-I" + REF_ROOT, "-I" + os.path.join(REF_ROOT, "third_party", "highway"),
           "-I" + os.path.join(REF_ROOT, "third_party"), "-I" + REPO, "-I" + os.path.join(REPO, "include"),
           "-o", out, os.path.join(REPO, "tests", "cpp", "test_reference_lowering.cpp"),
           os.path.join(PKG, "host", "gpu_operators.cpp"),
           "-L" + REF_LIB, "-lqe_ref", "-L" + PKG, "-lqeg", "-Wl,-rpath," + REF_LIB, "-Wl,-rpath," + PKG, "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_operators_build_and_lower_inside_the_reference_tree():
    exe = _build()
    r = subprocess.run([exe, "60"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "0 failures" in r.stdout
