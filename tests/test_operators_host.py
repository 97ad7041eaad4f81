"""Operator set-up on the host (no GPU): the Inlet_operator regions select the
same triangles as the reference's Region for a polygon and for a line."""
import numpy as np

import anuga_core_gb300 as agx
from anuga_core_gb300.mesh import rectangular_cross

REGIONS = {"a": [[10.0, 20.0], [30.0, 20.0], [30.0, 60.0], [10.0, 60.0]],
           "b": [[90.0, 10.0], [110.0, 10.0], [110.0, 30.0], [90.0, 30.0]],
           "c": [[50.0, 70.0], [70.0, 70.0]]}


def test_inlet_regions_match_reference(golden):
    f = golden("traj_inlets_de1.npz")
    p, e, b = rectangular_cross(12, 8, 120.0, 80.0)
    d = agx.Domain(p, e, b)
    for k, region in REGIONS.items():
        op = agx.Inlet_operator(d, region, Q=float(f["inlet_%s.Q" % k]))
        assert np.array_equal(op.indices, np.sort(f["inlet_%s.indices" % k])), k
        assert op.area == float(np.sum(d.mesh.areas[op.indices]))
    assert [o.device_loop for o in d.fractional_step_operators] == [True, True, True, True]
    assert d.fractional_step_operators[0] is d.boundary_flux_integral
    q = agx.Inlet_operator(d, REGIONS["a"], Q=lambda t: 1.0 + t)
    assert not q.device_loop and q.update_Q(2.0) == 3.0
