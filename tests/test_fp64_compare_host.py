"""Exactness of the plain kernels' restructured arithmetic, checked on the
host from the same source (de_plain.cuh compiled by g++):

* tests/cpp/check_dcompare.cpp: the integer-pipe FP64 comparisons (dlt, dle,
  dgt, dge, dmax, dmin, the tests against zero) give the IEEE comparison's
  outcome for every non-NaN pair (special values and 2M random pairs);
* tests/cpp/check_limiter.cpp: the limiter (margin tests, failing ratios
  only, one division per call) and the wet/dry factor equal the reference's
  formulas bit for bit on 4M and 2M random and adversarial inputs;
* tests/cpp/check_bits.cpp: the mixed update's integer-pipe conversions
  (bits.cuh: f2d_bits, d2f_bits) and RK2 halving (half_sum) equal the
  operations they replace;
* tests/cpp/check_soft64.cpp: the integer-only binary64 add, sub, mul, div
  and sqrt (soft64.cuh) equal the processor's IEEE operations bit for bit
  on special values, significands at the ends of their range and 1M random
  cases of each class."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(tmp_path, name):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / name)
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "cpp", name + ".cpp")], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_integer_comparisons_match_ieee(tmp_path):
    assert "mismatches 0" in _run(tmp_path, "check_dcompare")


def test_limiter_and_wet_dry_factor_match_reference_formulas(tmp_path):
    out = _run(tmp_path, "check_limiter")
    assert "mismatches 0" in out and "wet/dry mismatches 0" in out


def test_mixed_update_bit_conversions(tmp_path):
    assert "mismatches 0" in _run(tmp_path, "check_bits")


def test_integer_binary64_arithmetic_matches_ieee(tmp_path):
    out = _run(tmp_path, "check_soft64")
    assert "mismatches 0" in out.splitlines()[-1], out
