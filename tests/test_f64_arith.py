"""The float64 kernels quantize and dequantize in integer arithmetic
(szp_gb300/csrc/szp_f64.h).  The header is plain C++ too: compiled here with
g++ it must agree bit for bit with this CPU's binary64 multiply and
truncating conversion on random, subnormal, tie and range-edge operands."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("f64") / "f64_arith_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "szp_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "f64_arith_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2024])
def test_integer_f64_arith_matches_cpu(checker, seed):
    r = subprocess.run([checker, "1000000", str(seed)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
