"""Checkpoint and resume on the device (shallow_water_domain.py:1123-1157,
:2376-2397; shallow_water/checkpoint.py): a run restarted from a checkpoint
file continues bitwise as the uninterrupted run (plain FP64 form; the mixed
form to its own rounding), and the operator's applied volume carries over."""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300 import workloads

pytestmark = pytest.mark.gpu


def _domain(precision, tmp_path=None):
    d = workloads.dam_break(m=20, flow_algorithm="DE1", precision=precision)
    d.set_name("cp_" + precision)
    idx = np.arange(0, len(d), 4)
    agx.Rate_operator(d, rate=2.0e-4, indices=idx)
    if tmp_path is not None:
        d.set_checkpointing(checkpoint_dir=str(tmp_path), checkpoint_step=2)
    return d


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_resume_continues_the_run(tmp_path, precision):
    ref = _domain(precision)
    for _ in ref.evolve(yieldstep=1.0, finaltime=6.0):
        pass
    d = _domain(precision, tmp_path)
    for t in d.evolve(yieldstep=1.0, finaltime=3.0):
        pass
    # checkpoints at the yields 0, 2 (every second yieldstep)
    r = agx.load_checkpoint_file("cp_" + precision, str(tmp_path))
    assert r.get_time() == 2.0
    for _ in r.evolve(yieldstep=1.0, finaltime=6.0):
        pass
    a = r.quantities["stage"].centroid_values
    b = ref.quantities["stage"].centroid_values
    if precision == "fp64":
        assert np.array_equal(a, b)
        assert np.array_equal(r.quantities["xmomentum"].centroid_values, ref.quantities["xmomentum"].centroid_values)
    else:
        assert np.abs(a - b).max() <= 1.0e-6
    qa = r.fractional_step_operators[1].get_Q()
    qb = ref.fractional_step_operators[1].get_Q()
    assert abs(qa - qb) <= 1e-9 * abs(qb)
