"""The integer-instruction binary64 operations the FP64 kernels use for
division and square root (anuga_core_gb300/csrc/soft64.cuh) against the GPU's
own IEEE FP64 pipe, on the device build: bit for bit on drawn cases of every
class (any bit pattern, close exponents, exact and tie quotients, results
near and below the normal range)."""
import pytest

from anuga_core_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261204])
def test_device_soft64_matches_fp64_pipe(seed):
    mism = _lib.soft64_check(1 << 24, seed)
    assert mism == {"add": 0, "sub": 0, "mul": 0, "div": 0, "sqrt": 0}


def test_soft64_throughput_probe_runs():
    r = _lib.soft64_throughput()
    assert all(v > 0 for v in r.values()), r
