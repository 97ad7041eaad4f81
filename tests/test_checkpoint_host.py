"""Checkpoint files (shallow_water/checkpoint.py): a pickled domain keeps its
host state and leaves the device handle out; load_checkpoint_file picks the
latest time that opens."""
import os
import pickle

import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300 import workloads


def test_pickle_round_trip_keeps_the_state(tmp_path):
    d = workloads.dam_break(m=6, flow_algorithm="DE1")
    d.set_name("cp")
    agx.Rate_operator(d, rate=1.0e-3, indices=np.arange(5))
    d2 = pickle.loads(pickle.dumps(d))
    for q in ("stage", "xmomentum", "ymomentum", "elevation", "friction"):
        assert np.array_equal(d2.quantities[q].centroid_values, d.quantities[q].centroid_values)
    assert d2._scn is None and d2.get_flow_algorithm() == "DE1"
    assert len(d2.fractional_step_operators) == 2      # the boundary flux integral, the rate
    assert d2.fractional_step_operators[1].domain is d2
    assert d2.fractional_step_operators[0] is d2.boundary_flux_integral


def test_load_picks_the_latest_time(tmp_path):
    d = workloads.dam_break(m=4, flow_algorithm="DE0")
    d.set_name("run")
    for t, marker in ((1.0, 1.0), (2.5, 2.0), (10.0, 3.0)):
        d.relative_time = t
        d.quantities["friction"].centroid_values[:] = marker
        with open(os.path.join(str(tmp_path), "run_%s.pickle" % str(t)), "wb") as fh:
            pickle.dump(d, fh)
    with open(os.path.join(str(tmp_path), "run_20.0.pickle"), "wb") as fh:
        fh.write(b"truncated")                   # an unreadable newest file is skipped
    r = agx.load_checkpoint_file("run", str(tmp_path))
    assert r.relative_time == 10.0 and r.quantities["friction"].centroid_values[0] == 3.0
    r = agx.load_checkpoint_file("run", str(tmp_path), time=2.5)
    assert r.relative_time == 2.5
    with pytest.raises(Exception, match="Unable to open checkpoint file"):
        agx.load_checkpoint_file("other", str(tmp_path))
