"""Riverwall tables (anuga_core_gb300/riverwall.py) against the reference's
create_riverwalls on the same mesh and walls (tests/golden/traj_riverwall_de1.npz,
written by the reference's structures/riverwall.py), and its input checks."""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300.mesh import rectangular_cross

RIVERWALLS = {"south": [[50.0, 0.0, -2.2], [50.0, 50.0, -2.0]],
              "north": [[50.0, 50.0, -2.0], [50.0, 80.0, -1.7], [50.0, 100.0, -1.9]]}
RIVERWALL_PAR = {"north": {"Qfactor": 0.8, "s1": 0.85}}


def _domain(f):
    m = int(f["mesh.m"])
    p, e, b = rectangular_cross(m, m, 100.0, 100.0)
    assert np.array_equal(p, f["mesh.points"]) and np.array_equal(e, f["mesh.elements"])
    d = agx.Domain(p, e, b)
    d.set_flow_algorithm("DE1")
    return d


def test_tables_equal_the_reference(golden):
    f = golden("traj_riverwall_de1.npz")
    d = _domain(f)
    d.create_riverwalls(RIVERWALLS, RIVERWALL_PAR)
    rw = d.riverwallData
    assert np.array_equal(d.edge_flux_type, f["rw.edge_flux_type"])
    assert np.array_equal(d.edge_river_wall_counter, f["rw.edge_river_wall_counter"])
    assert np.array_equal(rw.riverwall_elevation, f["rw.riverwall_elevation"])
    assert np.array_equal(rw.hydraulic_properties_rowIndex, f["rw.hydraulic_properties_rowIndex"])
    assert np.array_equal(rw.hydraulic_properties, f["rw.hydraulic_properties"])
    assert np.array_equal(rw.riverwall_edges, f["rw.riverwall_edges"])
    assert d.number_of_riverwall_edges == len(f["rw.riverwall_edges"]) == 40
    # both slots of every interior wall edge are marked
    nb = d.mesh.neighbours.reshape(-1, 3)
    ne = d.mesh.neighbour_edges.reshape(-1, 3)
    for s in rw.riverwall_edges:
        k, i = divmod(int(s), 3)
        if nb[k, i] >= 0:
            assert d.edge_flux_type[3 * nb[k, i] + ne[k, i]] == 1


def test_input_checks(golden):
    f = golden("traj_riverwall_de1.npz")
    d = _domain(f)
    with pytest.raises(Exception, match="no corresponding key"):
        d.create_riverwalls(RIVERWALLS, {"east": {"Qfactor": 1.0}})
    with pytest.raises(Exception, match="not recognised"):
        d.create_riverwalls(RIVERWALLS, {"north": {"Cd": 1.0}})
    with pytest.raises(Exception, match="s1"):
        d.create_riverwalls(RIVERWALLS, {"north": {"s1": 0.99}})
    with pytest.raises(Exception, match="h1"):
        d.create_riverwalls(RIVERWALLS, {"south": {"h1": 2.0}})
    # a wall away from every edge marks nothing
    d.create_riverwalls({"off": [[52.3, 10.0, 0.0], [52.3, 20.0, 0.0]]})
    assert d.number_of_riverwall_edges == 0 and not d.riverwallData.active
