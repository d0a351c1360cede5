"""The C++ drop-in header (include/graphalgo_gb300.hpp) used with the
reference's call shapes, checked against the oracle (tests/cpp/test_dropin.cpp)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out):
    lib = os.path.join(ROOT, "graphalgo_gb300", "_lib")
    orc = os.path.join(ROOT, "oracle", "_build")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), "-L" + lib, "-lgraphalgo_gb300",
           "-L" + orc, "-loracle", "-Wl,-rpath," + lib, "-Wl,-rpath," + orc, "-o", out]
    subprocess.check_call(cmd)


def test_dropin_header_compiles(built, tmp_path):
    _compile(str(tmp_path / "test_dropin"))


@pytest.mark.gpu
def test_dropin_on_gpu(built, tmp_path):
    exe = str(tmp_path / "test_dropin")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "drop-in ok" in r.stdout
