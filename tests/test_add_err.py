"""The integer rounding-error routine the compensated aggregations use
(pythia_gb300/csrc/pg_add_err.h) equals Knuth's TwoSum bit for bit on the host,
over random operand pairs and the edge cases: subnormals, cancellation,
powers of two, ties to even."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_add_error_equals_two_sum(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "add_err_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I" + os.path.join(ROOT, "pythia_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "add_err_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
