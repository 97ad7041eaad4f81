"""The CPU oracle is pinned to the reference: every phase output and three
full trajectories from the reference ANUGA (tests/golden/, written by
tests/golden/make_golden.py) are reproduced bit for bit."""
import numpy as np
import pytest

from anuga_core_gb300.mesh import Mesh, rectangular_cross

KINDS = {"left": ("dirichlet", (1.3, 0.05, -0.02)), "right": ("transmissive", None),
         "top": ("reflective", None), "bottom": ("reflective", None)}


@pytest.mark.parametrize("alg", ["de0", "de1"])
def test_oracle_phases_bit_exact(golden, oracle_mod, alg):
    f = golden("phases_%s.npz" % alg)
    m, n, L1, L2 = f["params"]
    p, e, b = rectangular_cross(int(m), int(n), L1, L2)
    assert np.array_equal(p, f["mesh.points"])
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, alg.upper())
    od.set_centroid_state(f["in.stage.centroid_values"], f["in.xmomentum.centroid_values"],
                          f["in.ymomentum.centroid_values"], f["in.elevation.centroid_values"],
                          f["in.friction.centroid_values"])
    od.set_boundaries([(M.tag_boundary_cells[t], KINDS[t][0], KINDS[t][1]) for t in M.tag_boundary_cells])
    od.protect()
    assert np.array_equal(od.stage_c, f["protect.stage.centroid_values"])
    assert np.array_equal(od.xmom_c, f["protect.xmomentum.centroid_values"])
    od.extrapolate()
    for q, a in [("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom"), ("elevation", "bed"),
                 ("height", "height")]:
        assert np.array_equal(getattr(od, a + "_e"), f["extrap.%s.edge_values" % q].ravel())
        assert np.array_equal(getattr(od, a + "_v"), f["extrap.%s.vertex_values" % q].ravel())
    od.update_boundary()
    for q, a in [("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")]:
        assert np.array_equal(getattr(od, a + "_b"), f["bc.%s.boundary_values" % q])
    assert od.compute_fluxes(0) == float(f["flux.flux_timestep"])
    assert np.array_equal(od.max_speed, f["flux.max_speed"])
    # an OpenMP sum in both the reference and the oracle: its last place
    # follows the host's thread count
    np.testing.assert_allclose(od.boundary_flux_sum, f["flux.boundary_flux_sum"], rtol=1e-13, atol=0)
    for q, a in [("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")]:
        assert np.array_equal(getattr(od, a + "_x"), f["flux.%s.explicit_update" % q])
    od.compute_forcing_terms()
    for q, a in [("xmomentum", "xmom"), ("ymomentum", "ymom")]:
        assert np.array_equal(getattr(od, a + "_s"), f["forcing.%s.semi_implicit_update" % q])
    od.timestep = float(f["update.timestep"])
    od.update_conserved_quantities()
    for q, a in [("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")]:
        assert np.array_equal(getattr(od, a + "_c"), f["update.%s.centroid_values" % q])


R = ("reflective", None)
TRAJ = {
    "traj_dambreak_de0": ("DE0", {"left": R, "right": R, "top": R, "bottom": R}, False),
    "traj_inflow_de1": ("DE1", {"left": ("dirichlet", (2.0, 0, 0)), "right": ("transmissive", None),
                                "top": R, "bottom": R}, False),
    "traj_delaunay_rain_de1": ("DE1", {"exterior": R}, True),
    "traj_dambreak_de2": ("DE2", {"left": R, "right": R, "top": R, "bottom": R}, False),
    "traj_inflow_de2": ("DE2", {"left": ("dirichlet", (2.0, 0, 0)), "right": ("transmissive", None),
                                "top": R, "bottom": R}, False),
    "traj_inflow_de0_7": ("DE0_7", {"left": ("dirichlet", (2.0, 0, 0)), "right": ("transmissive", None),
                                    "top": R, "bottom": R}, False),
    "traj_inflow_de1_7": ("DE1_7", {"left": ("dirichlet", (2.0, 0, 0)), "right": ("transmissive", None),
                                    "top": R, "bottom": R}, False),
}


@pytest.mark.parametrize("name", sorted(TRAJ))
def test_oracle_trajectories_bit_exact(golden, oracle_mod, name):
    alg, kinds, rain = TRAJ[name]
    f = golden(name + ".npz")
    p, e = f["mesh.points"], f["mesh.elements"]
    b = None
    if "mesh.m" in f:
        m = int(f["mesh.m"])
        L = float(p[:, 0].max())
        p2, e2, b = rectangular_cross(m, m, L, L)
        assert np.array_equal(p, p2) and np.array_equal(e, e2)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, alg)
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    od.set_boundaries([(M.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in M.tag_boundary_cells])
    if rain:
        od.add_rate(f["rain.indices"], float(f["rain.rate"]))
    res = [(t, od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["times"])
    assert [r[1] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[2], f["stage"][i])
        assert np.array_equal(r[3], f["xmom"][i])
        assert np.array_equal(r[4], f["ymom"][i])


INLETS = {"a": dict(), "b": dict(zero_velocity=True), "c": dict(velocity=(0.2, 0.0))}


def test_oracle_inlets_bit_exact(golden, oracle_mod):
    """Inlet_operator (inflow over a polygon, extraction with zero velocity, a
    line inlet with an imposed velocity) against the reference's trajectory."""
    f = golden("traj_inlets_de1.npz")
    p, e = f["mesh.points"], f["mesh.elements"]
    p2, e2, b = rectangular_cross(12, 8, 120.0, 80.0)
    assert np.array_equal(p, p2) and np.array_equal(e, e2)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, "DE1")
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    od.set_boundaries([(M.tag_boundary_cells[t], "reflective", None) for t in M.tag_boundary_cells])
    for k, kw in INLETS.items():
        od.add_inlet(f["inlet_%s.indices" % k], float(f["inlet_%s.Q" % k]), **kw)
    res = [(t, od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["times"])
    assert [r[1] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[2], f["stage"][i]), i
        assert np.array_equal(r[3], f["xmom"][i]), i
        assert np.array_equal(r[4], f["ymom"][i]), i


def test_oracle_riverwall_trajectory_bit_exact(golden, oracle_mod):
    """The weir branch of the flux (sw_domain_openmp.c:324-426, 581-650) on a
    dam break whose dam line carries two riverwalls, against the reference."""
    f = golden("traj_riverwall_de1.npz")
    m = int(f["mesh.m"])
    p, e, b = rectangular_cross(m, m, 100.0, 100.0)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, "DE1")
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    od.set_boundaries([(M.tag_boundary_cells[t], "reflective", None) for t in M.tag_boundary_cells])
    od.set_riverwalls(f["rw.edge_flux_type"], f["rw.edge_river_wall_counter"], f["rw.riverwall_elevation"],
                      f["rw.hydraulic_properties_rowIndex"], f["rw.hydraulic_properties"])
    res = [(t, od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["times"])
    assert [r[1] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[2], f["stage"][i]), i
        assert np.array_equal(r[3], f["xmom"][i]), i
        assert np.array_equal(r[4], f["ymom"][i]), i


CHANNEL = {"left": ("transmissive_set_stage", lambda t: 0.6 + 0.03 * np.sin(0.3 * t)),
           "right": ("flather", lambda t: 0.56 + 0.0 * t),
           "top": ("dirichlet_discharge", (0.6, 0.01)),
           "bottom": ("transmissive_zero_momentum", None)}


@pytest.mark.parametrize("alg", ["DE1", "DE0"])
def test_oracle_channel_boundaries_bit_exact(golden, oracle_mod, alg):
    """Transmissive_momentum_set_stage, Flather_external_stage_zero_velocity
    (its wet branch), Dirichlet_discharge and Transmissive_stage_zero_momentum
    boundaries, one per side of a channel, against the reference."""
    f = golden("traj_channel_boundaries_%s.npz" % alg.lower())
    m, n = int(f["mesh.m"]), int(f["mesh.n"])
    p, e, b = rectangular_cross(m, n, 160.0, 80.0)
    assert np.array_equal(p, f["mesh.points"])
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, alg)
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    od.set_boundaries([(M.tag_boundary_cells[t], CHANNEL[t][0], CHANNEL[t][1]) for t in M.tag_boundary_cells])
    res = [(t, od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[1] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[2], f["stage"][i]), i
        assert np.array_equal(r[3], f["xmom"][i]), i
        assert np.array_equal(r[4], f["ymom"][i]), i


def test_oracle_characteristic_boundary_bit_exact(golden, oracle_mod):
    """Characteristic_stage_boundary (shallow_water/boundaries.py:639-848)."""
    f = golden("traj_channel_characteristic_de1.npz")
    p, e, b = rectangular_cross(int(f["mesh.m"]), int(f["mesh.n"]), 160.0, 80.0)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, "DE1")
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    kinds = {"left": ("characteristic", lambda t: 0.6 + 0.03 * np.sin(0.3 * t)), "right": ("transmissive", None),
             "top": R, "bottom": R}
    od.set_boundaries([(M.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in M.tag_boundary_cells])
    res = [(od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[1], f["stage"][i]), i
        assert np.array_equal(r[2], f["xmom"][i]), i
        assert np.array_equal(r[3], f["ymom"][i]), i


def _time_space(t, x, y):
    return [0.6 + 0.02 * np.sin(0.3 * t) * np.cos(y / 20.0), 0.0, 0.0]


def test_oracle_time_space_boundary_bit_exact(golden, oracle_mod):
    """Time_space_boundary (generic_boundary_conditions.py:419-517)."""
    f = golden("traj_channel_time_space_de1.npz")
    p, e, b = rectangular_cross(int(f["mesh.m"]), int(f["mesh.n"]), 160.0, 80.0)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, "DE1")
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    kinds = {"left": ("time_space", _time_space), "right": ("transmissive", None), "top": R, "bottom": R}
    od.set_boundaries([(M.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in M.tag_boundary_cells])
    res = [(od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[1], f["stage"][i]), i
        assert np.array_equal(r[2], f["xmom"][i]), i


def test_oracle_inflow_boundary_bit_exact(golden, oracle_mod):
    """Inflow_boundary (shallow_water/boundaries.py:902-992)."""
    f = golden("traj_channel_inflow_de1.npz")
    p, e, b = rectangular_cross(int(f["mesh.m"]), int(f["mesh.n"]), 160.0, 80.0)
    M = Mesh(p, e, b)
    od = oracle_mod.OracleDomain(M, "DE1")
    od.set_centroid_state(f["init.stage"], f["init.xmom"], f["init.ymom"], f["init.elevation_c"], f["init.friction"])
    od.set_bed_vertex_values(f["init.elevation_v"])
    kinds = {"left": ("inflow", 2.0), "right": ("transmissive", None), "top": R, "bottom": R}
    od.set_boundaries([(M.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in M.tag_boundary_cells])
    res = [(od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy())
           for t in od.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))]
    assert [r[0] for r in res] == list(f["steps"])
    for i, r in enumerate(res):
        assert np.array_equal(r[1], f["stage"][i]), i
        assert np.array_equal(r[2], f["xmom"][i]), i
