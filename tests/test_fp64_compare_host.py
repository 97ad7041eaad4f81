"""The integer-pipe FP64 comparisons of the plain kernels (de_plain.cuh:
dlt, dle, dgt, dge, dmax, dmin and the tests against zero) give the IEEE
comparison's outcome for every non-NaN pair: checked on the host by
tests/cpp/check_dcompare.cpp over special values and 2M random pairs."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_comparisons_match_ieee(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "check_dcompare")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "cpp", "check_dcompare.cpp")],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
