"""Compiles tests/cpp/test_operators.cpp against the C++ host operators
(query-engine_gb300/host/) and libqeg.so, and runs it on the GPU: the
GpuAggregate / GpuHashJoin drop-ins driven through the reference's Operator
pull interface (open/next/close, Batch/Column views, selection vectors,
STR dictionaries, <= 2048-row output batches)."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "query-engine_gb300")


def build_test_binary():
    out = os.path.join(PKG, "_build", "test_operators")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-o", out,
           os.path.join(REPO, "tests", "cpp", "test_operators.cpp"), os.path.join(PKG, "host", "gpu_operators.cpp"),
           "-I" + os.path.join(REPO, "include"), "-L" + PKG, "-lqeg", "-Wl,-rpath," + PKG]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_host_operators_compile():
    build_test_binary()


@pytest.mark.gpu
def test_host_operators_on_gpu():
    exe = build_test_binary()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
