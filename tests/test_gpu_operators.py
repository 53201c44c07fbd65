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
           "-I" + os.path.join(REPO, "include"), "-L" + PKG, "-lqeg", "-Wl,-rpath," + PKG, "-pthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_host_operators_compile():
    build_test_binary()


@pytest.mark.gpu
def test_host_operators_on_gpu():
    exe = build_test_binary()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


def test_string_dict_contract(tmp_path):
    """The host contract's StringDict (used when the operators are built
    without the reference's headers) keeps the reference's semantics: dense
    codes in first-seen order, a repeated string gets its first code, at()
    returns the interned bytes (empty strings and embedded NULs included), and
    copies and moves keep every code and string."""
    src = tmp_path / "dict.cpp"
    src.write_text(r'''
#include <cassert>
#include <string>
#include <utility>
#include "host/qe_contract.h"
int main() {
  qe::StringDict d;
  assert(d.size() == 0);
  assert(d.intern("b") == 0 && d.intern("a") == 1 && d.intern("b") == 0);
  assert(d.intern("") == 2 && d.intern(std::string("x\0y", 3)) == 3);
  for (int i = 0; i < 1000; ++i) assert(d.intern("k" + std::to_string(i)) == 4 + i);
  assert(d.size() == 1004 && d.at(1) == "a" && d.at(2).empty() && d.at(3) == std::string("x\0y", 3));
  qe::StringDict c = d;
  assert(c.size() == d.size() && c.intern("a") == 1 && c.intern("k999") == 1003 && c.intern("new") == 1004);
  assert(d.size() == 1004);
  qe::StringDict m = std::move(c);
  assert(m.intern("k5") == 9 && m.at(1004) == "new" && m.size() == 1005);
  qe::StringDict e;
  e = m;
  assert(e.intern("b") == 0 && e.size() == 1005);
  return 0;
}
''')
    exe = tmp_path / "dict"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", PKG, str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    subprocess.run([str(exe)], check=True)


def test_host_staging_without_a_gpu():
    """tests/cpp/test_staging.cpp: the operators' host staging (values and
    validity words across random batches and selection vectors, STR codes to
    canonical ids by value, the invalid-code error, output column views)
    checked on the CPU; page-locked allocation falls back to the heap."""
    out = os.path.join(PKG, "_build", "test_staging")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-o", out,
           os.path.join(REPO, "tests", "cpp", "test_staging.cpp"), os.path.join(PKG, "host", "gpu_operators.cpp"),
           "-I" + os.path.join(REPO, "include"), "-L" + PKG, "-lqeg", "-Wl,-rpath," + PKG, "-pthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
