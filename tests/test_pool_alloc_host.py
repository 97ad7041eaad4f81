"""The device pool's free-extent bookkeeping (anuga_core_gb300/csrc/
free_runs.h, compiled by g++ on the host): first-fit placement, the largest
free run and the end of the used range agree with a scan of an owner array
over random admissions and releases (tests/cpp/check_free_runs.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_free_runs_match_owner_array_scan(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "check_free_runs")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "cpp", "check_free_runs.cpp")],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "mismatches 0" in r.stdout, r.stdout + r.stderr
