"""Generates the golden fixtures in tests/golden/ from the reference ANUGA.

Run once in a container that has the reference source tree:

    bash tests/golden/build_reference_pkg.sh /path/to/anuga_core
    OMP_NUM_THREADS=1 python tests/golden/make_golden.py

The reference package is imported from baseline/_ref (built by the script
above with -ffp-contract=off); the DE kernels run in multiprocessor mode 2
(OpenMP) with one thread.  Each fixture is a small compressed .npz.
"""
import os
import sys

os.environ.setdefault("OMP_NUM_THREADS", "1")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "baseline", "_ref", "_shims"), os.path.join(ROOT, "baseline", "_ref")]

import numpy as np  # noqa: E402
import anuga  # noqa: E402

MESH_KEYS = ["vertex_coordinates", "edge_midpoint_coordinates", "centroid_coordinates", "normals",
             "edgelengths", "areas", "radii", "neighbours", "neighbour_edges", "number_of_boundaries",
             "surrogate_neighbours", "boundary_cells", "boundary_edges"]


def delaunay_case(npts=300, seed=3, size=100.0):
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, size, (npts, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    return pts, tri


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def mesh_fixture(name, points, elements, boundary):
    d = anuga.Domain(points, elements, boundary)
    out = {k: np.asarray(getattr(d.mesh, k)) for k in MESH_KEYS}
    keys = sorted(d.boundary.keys())
    out["boundary_keys"] = np.array(keys, np.int64).reshape(-1, 2)
    out["points"] = np.asarray(points, float)
    out["elements"] = np.asarray(elements, np.int64)
    save(name, **out)


def bumpy_bed(x, y, L):
    return 0.02 * x - 0.01 * y + 0.6 * np.exp(-((x - 0.4 * L) ** 2 + (y - 0.5 * L) ** 2) / (0.02 * L * L)) \
        - 0.4 * np.exp(-((x - 0.7 * L) ** 2 + (y - 0.3 * L) ** 2) / (0.01 * L * L))


def phase_fixture(name, flow_algorithm, m=8, n=6, L=60.0):
    """One full set of per-phase outputs from an identical, non-trivial state."""
    pts, elem, bnd = anuga.rectangular_cross(m, n, L, L * n / m)
    d = anuga.Domain(pts, elem, bnd)
    d.set_flow_algorithm(flow_algorithm)
    d.set_multiprocessor_mode(2)
    d.set_store(False)
    d.set_quantity("elevation", lambda x, y: bumpy_bed(x, y, L))
    d.set_quantity("stage", lambda x, y: np.where(x < 0.45 * L, 1.1, 0.3 + 0.0 * x))
    rng = np.random.default_rng(11)
    N = len(d)
    d.set_quantity("xmomentum", rng.normal(0, 0.05, N), location="centroids")
    d.set_quantity("ymomentum", rng.normal(0, 0.05, N), location="centroids")
    d.set_quantity("friction", rng.uniform(0.02, 0.05, N), location="centroids")
    Br = anuga.Reflective_boundary(d)
    Bt = anuga.Transmissive_boundary(d)
    Bd = anuga.Dirichlet_boundary([1.3, 0.05, -0.02])
    d.set_boundary({"left": Bd, "right": Bt, "top": Br, "bottom": Br})
    Q = d.quantities
    out = {}

    def snap(prefix, names):
        for nm in names:
            out[prefix + nm] = np.array(nm_arr(nm))

    def nm_arr(nm):
        q, loc = nm.split(".")
        return getattr(Q[q], loc)

    cen = ["stage.centroid_values", "xmomentum.centroid_values", "ymomentum.centroid_values",
           "elevation.centroid_values", "friction.centroid_values", "height.centroid_values"]
    snap("in.", cen + ["elevation.vertex_values", "elevation.edge_values"])
    out["in.mass_error"] = np.array(d.protect_against_infinitesimal_and_negative_heights() or 0.0)
    snap("protect.", cen)
    from anuga.shallow_water.sw_domain_openmp_ext import extrapolate_second_order_edge_sw
    extrapolate_second_order_edge_sw(d)
    edge = [f"{q}.edge_values" for q in ("stage", "xmomentum", "ymomentum", "elevation", "height")]
    vert = [f"{q}.vertex_values" for q in ("stage", "xmomentum", "ymomentum", "elevation", "height")]
    snap("extrap.", cen + edge + vert)
    d.update_boundary()
    snap("bc.", [f"{q}.boundary_values" for q in ("stage", "xmomentum", "ymomentum")])
    d.compute_fluxes()
    out["flux.flux_timestep"] = np.array(d.flux_timestep)
    out["flux.max_speed"] = np.array(d.max_speed)
    out["flux.boundary_flux_sum"] = np.array(d.boundary_flux_sum)
    snap("flux.", [f"{q}.explicit_update" for q in ("stage", "xmomentum", "ymomentum")])
    d.compute_forcing_terms()
    snap("forcing.", [f"{q}.semi_implicit_update" for q in ("stage", "xmomentum", "ymomentum")])
    d.timestep = 0.9 * d.flux_timestep
    out["update.timestep"] = np.array(d.timestep)
    d.update_conserved_quantities()
    snap("update.", cen)
    out["mesh.points"] = pts
    out["mesh.elements"] = elem
    out["params"] = np.array([m, n, L, L * n / m])
    save(name, **out)


def trajectory_fixture(name, build, flow_algorithm, yieldstep, finaltime):
    d, extra = build()
    d.set_flow_algorithm(flow_algorithm)
    d.set_multiprocessor_mode(2)
    d.set_store(False)
    out = dict(extra)
    Q = d.quantities
    out["init.stage"] = Q["stage"].centroid_values.copy()
    out["init.xmom"] = Q["xmomentum"].centroid_values.copy()
    out["init.ymom"] = Q["ymomentum"].centroid_values.copy()
    out["init.elevation_c"] = Q["elevation"].centroid_values.copy()
    out["init.elevation_v"] = Q["elevation"].vertex_values.copy()
    out["init.friction"] = Q["friction"].centroid_values.copy()
    times, steps, st, xm, ym = [], [], [], [], []
    for t in d.evolve(yieldstep=yieldstep, finaltime=finaltime):
        times.append(t)
        steps.append(d.number_of_steps)
        st.append(Q["stage"].centroid_values.copy())
        xm.append(Q["xmomentum"].centroid_values.copy())
        ym.append(Q["ymomentum"].centroid_values.copy())
    out["times"] = np.array(times)
    out["steps"] = np.array(steps)
    out["stage"] = np.array(st)
    out["xmom"] = np.array(xm)
    out["ymom"] = np.array(ym)
    out["final.stage_edge"] = Q["stage"].edge_values.copy()
    out["final.stage_vertex"] = Q["stage"].vertex_values.copy()
    out["yieldstep"] = np.array(yieldstep)
    out["finaltime"] = np.array(finaltime)
    if hasattr(d, "_degenerate_calls"):
        out["degenerate_zeroed"] = np.array(d._degenerate_calls["zeroed"])
    save(name, **out)


def build_dam_break(m=20):
    # the small form of the 40,000-triangle dam break (same geometry, coarser mesh)
    pts, elem, bnd = anuga.rectangular_cross(m, m, 100.0, 100.0)
    d = anuga.Domain(pts, elem, bnd)
    d.set_quantity("elevation", lambda x, y: -x / 20)
    d.set_quantity("stage", lambda x, y: -x / 20 + np.where(x < 50, 1.0, 0.1))
    d.set_quantity("friction", 0.03)
    Br = anuga.Reflective_boundary(d)
    d.set_boundary({"left": Br, "right": Br, "top": Br, "bottom": Br})
    return d, {"mesh.points": pts, "mesh.elements": elem, "mesh.m": np.array(m)}


def build_inflow_bumps(m=16, L=800.0):
    # the small form of the slope + Gaussian bumps inflow case
    pts, elem, bnd = anuga.rectangular_cross(m, m, L, L)
    d = anuga.Domain(pts, elem, bnd)
    rng = np.random.default_rng(1234)
    cx = rng.uniform(0, L, 8)
    cy = rng.uniform(0, L, 8)
    A = rng.uniform(-5, 5, 8)
    s = rng.uniform(0.1 * L, 0.4 * L, 8)

    def bed(x, y):
        z = -0.004 * (x - 0.4 * L)
        for i in range(8):
            z = z + A[i] * np.exp(-((x - cx[i]) ** 2 + (y - cy[i]) ** 2) / (2 * s[i] ** 2))
        return z
    d.set_quantity("elevation", bed)
    d.set_quantity("stage", 0.0)
    N = len(d)
    d.set_quantity("friction", rng.uniform(0.02, 0.06, N), location="centroids")
    Br = anuga.Reflective_boundary(d)
    Bt = anuga.Transmissive_boundary(d)
    Bd = anuga.Dirichlet_boundary([2.0, 0.0, 0.0])
    d.set_boundary({"left": Bd, "right": Bt, "top": Br, "bottom": Br})
    return d, {"mesh.points": pts, "mesh.elements": elem, "mesh.m": np.array(m),
               "bed.params": np.stack([cx, cy, A, s])}


def build_delaunay_rain():
    pts, tri = delaunay_case(400, seed=5, size=200.0)
    d = anuga.Domain(pts, tri, None)
    d.set_quantity("elevation", lambda x, y: 0.01 * x + 0.5 * np.sin(y / 20.0))
    d.set_quantity("stage", lambda x, y: np.maximum(0.01 * x + 0.5 * np.sin(y / 20.0), 0.3))
    d.set_quantity("friction", 0.025)
    Br = anuga.Reflective_boundary(d)
    d.set_boundary({"exterior": Br})
    c = d.centroid_coordinates
    idx = np.nonzero((c[:, 0] > 50) & (c[:, 0] < 150) & (c[:, 1] > 50) & (c[:, 1] < 150))[0]
    anuga.Rate_operator(d, rate=0.01, indices=idx)
    return d, {"mesh.points": pts, "mesh.elements": tri, "rain.indices": idx, "rain.rate": np.array(0.01)}


def build_inlets(m=12, n=8):
    # Inlet_operator: inflow over a polygon, extraction with zero velocity,
    # and a line inlet with an imposed velocity
    pts, elem, bnd = anuga.rectangular_cross(m, n, 120.0, 80.0)
    d = anuga.Domain(pts, elem, bnd)
    d.set_quantity("elevation", lambda x, y: -0.02 * x + 0.1 * np.sin(y / 10.0))
    d.set_quantity("stage", lambda x, y: np.maximum(-0.02 * x + 0.1 * np.sin(y / 10.0), -1.5))
    d.set_quantity("friction", 0.02)
    Br = anuga.Reflective_boundary(d)
    d.set_boundary({"left": Br, "right": Br, "top": Br, "bottom": Br})
    a = anuga.Inlet_operator(d, [[10.0, 20.0], [30.0, 20.0], [30.0, 60.0], [10.0, 60.0]], Q=1.5)
    b = anuga.Inlet_operator(d, [[90.0, 10.0], [110.0, 10.0], [110.0, 30.0], [90.0, 30.0]], Q=-0.4,
                             zero_velocity=True)
    c = anuga.Inlet_operator(d, [[50.0, 70.0], [70.0, 70.0]], Q=0.8, velocity=[0.2, 0.0])
    extra = {"mesh.points": pts, "mesh.elements": elem}
    for name, op, q in (("a", a, 1.5), ("b", b, -0.4), ("c", c, 0.8)):
        extra["inlet_%s.indices" % name] = np.asarray(op.inlet.triangle_indices, np.int64)
        extra["inlet_%s.Q" % name] = np.array(q)
    d._inlets = (a, b, c)
    return d, extra


RIVERWALLS = {"south": [[50.0, 0.0, -2.2], [50.0, 50.0, -2.0]],
              "north": [[50.0, 50.0, -2.0], [50.0, 80.0, -1.7], [50.0, 100.0, -1.9]]}
RIVERWALL_PAR = {"north": {"Qfactor": 0.8, "s1": 0.85}}


def build_dam_break_riverwall(m=20):
    # the dam break with a levee on the dam line, overtopped along part of it
    d, extra = build_dam_break(m)
    d.set_flow_algorithm("DE1")
    d.riverwallData.create_riverwalls(RIVERWALLS, RIVERWALL_PAR, verbose=False)
    rw = d.riverwallData
    extra = dict(extra)
    extra["rw.edge_flux_type"] = np.asarray(d.edge_flux_type).copy()
    extra["rw.edge_river_wall_counter"] = np.asarray(d.edge_river_wall_counter).copy()
    extra["rw.riverwall_elevation"] = np.asarray(rw.riverwall_elevation).copy()
    extra["rw.hydraulic_properties_rowIndex"] = np.asarray(rw.hydraulic_properties_rowIndex).copy()
    extra["rw.hydraulic_properties"] = np.asarray(rw.hydraulic_properties).copy()
    extra["rw.riverwall_edges"] = np.asarray(rw.riverwall_edges).copy()
    return d, extra


def build_open_channel(m=16, n=8, L=160.0, W=80.0):
    # a channel whose bed rises to the right under a 0.6 m water level; each
    # side carries another of the stage/momentum boundaries of
    # shallow_water/boundaries.py (Flather's outside stage below the bed at
    # the right end, so that its wet branch is taken)
    pts, elem, bnd = anuga.rectangular_cross(m, n, L, W)
    d = anuga.Domain(pts, elem, bnd)
    bed = lambda x, y: 0.55 * x / L + 0.02 * np.sin(y / 9.0)
    d.set_quantity("elevation", bed)
    d.set_quantity("stage", lambda x, y: np.maximum(0.6 + 0.0 * x, bed(x, y)))
    d.set_quantity("friction", 0.025)
    from anuga.shallow_water.boundaries import Dirichlet_discharge_boundary
    d.set_boundary({
        "left": anuga.Transmissive_momentum_set_stage_boundary(d, function=lambda t: 0.6 + 0.03 * np.sin(0.3 * t)),
        "right": anuga.Flather_external_stage_zero_velocity_boundary(d, function=lambda t: 0.56 + 0.0 * t),
        "top": Dirichlet_discharge_boundary(d, stage0=0.6, wh0=0.01),
        "bottom": anuga.Transmissive_stage_zero_momentum_boundary(d)})
    return d, {"mesh.points": pts, "mesh.elements": elem, "mesh.m": np.array(m), "mesh.n": np.array(n)}


def build_characteristic_channel(m=16, n=8, L=160.0, W=80.0):
    d, extra = build_open_channel(m, n, L, W)
    d.set_boundary({"left": anuga.Characteristic_stage_boundary(d, function=lambda t: 0.6 + 0.03 * np.sin(0.3 * t)),
                    "right": anuga.Transmissive_boundary(d), "top": anuga.Reflective_boundary(d),
                    "bottom": anuga.Reflective_boundary(d)})
    return d, extra


def _time_space(t, x, y):
    return [0.6 + 0.02 * np.sin(0.3 * t) * np.cos(y / 20.0), 0.0, 0.0]


def build_time_space_channel(m=16, n=8, L=160.0, W=80.0):
    d, extra = build_open_channel(m, n, L, W)
    d.set_boundary({"left": anuga.Time_space_boundary(d, function=_time_space),
                    "right": anuga.Transmissive_boundary(d), "top": anuga.Reflective_boundary(d),
                    "bottom": anuga.Reflective_boundary(d)})
    return d, extra


def build_inflow_channel(m=16, n=8, L=160.0, W=80.0):
    d, extra = build_open_channel(m, n, L, W)
    from anuga.shallow_water.boundaries import Inflow_boundary
    d.set_boundary({"left": Inflow_boundary(d, rate=2.0), "right": anuga.Transmissive_boundary(d),
                    "top": anuga.Reflective_boundary(d), "bottom": anuga.Reflective_boundary(d)})
    return d, extra


def boundary_fixtures():
    trajectory_fixture("traj_channel_inflow_de1.npz", build_inflow_channel, "DE1", 2.0, 12.0)
    trajectory_fixture("traj_channel_time_space_de1.npz", build_time_space_channel, "DE1", 2.0, 12.0)
    trajectory_fixture("traj_channel_characteristic_de1.npz", build_characteristic_channel, "DE1", 2.0, 12.0)
    trajectory_fixture("traj_channel_boundaries_de1.npz", build_open_channel, "DE1", 2.0, 12.0)
    trajectory_fixture("traj_channel_boundaries_de0.npz", build_open_channel, "DE0", 2.0, 8.0)


def flow_algorithm_fixtures():
    # the other flow algorithms of the DE family (shallow_water_domain.py:708-877):
    # DE2 (rk3 time stepping), DE0_7 and DE1_7 (other betas, minimum height)
    trajectory_fixture("traj_dambreak_de2.npz", build_dam_break, "DE2", 1.0, 3.0)
    trajectory_fixture("traj_inflow_de2.npz", build_inflow_bumps, "DE2", 10.0, 30.0)
    trajectory_fixture("traj_inflow_de0_7.npz", build_inflow_bumps, "DE0_7", 10.0, 30.0)
    trajectory_fixture("traj_inflow_de1_7.npz", build_inflow_bumps, "DE1_7", 10.0, 30.0)


def integral_fixture(name, build, flow_algorithm, yieldstep, finaltime, rain=None):
    """Boundary flux integral, water volume and fractional-step volume at
    every yield (shallow_water_domain.py:1630-1745, 2749-2781)."""
    d, extra = build()
    d.set_flow_algorithm(flow_algorithm)
    d.set_multiprocessor_mode(2)
    d.set_store(False)
    out = dict(extra)
    if rain is not None:
        c = d.centroid_coordinates
        L = float(c[:, 0].max())
        idx = np.nonzero((c[:, 0] > 0.5 * L) & (c[:, 1] < 0.5 * L))[0]
        anuga.Rate_operator(d, rate=rain, indices=idx)
        out["rain.indices"] = idx
        out["rain.rate"] = np.array(rain)
    Q = d.quantities
    out["init.stage"] = Q["stage"].centroid_values.copy()
    out["init.xmom"] = Q["xmomentum"].centroid_values.copy()
    out["init.ymom"] = Q["ymomentum"].centroid_values.copy()
    out["init.elevation_c"] = Q["elevation"].centroid_values.copy()
    out["init.friction"] = Q["friction"].centroid_values.copy()
    v0 = d.get_water_volume()
    times, steps, st, bfi, vol, frac = [], [], [], [], [], []
    for t in d.evolve(yieldstep=yieldstep, finaltime=finaltime):
        times.append(t)
        steps.append(d.number_of_steps)
        st.append(Q["stage"].centroid_values.copy())
        V, BF, FS = d.report_water_volume_statistics(verbose=False, returnStats=True)
        vol.append(V)
        bfi.append(BF)
        frac.append(FS)
    out["volume0"] = np.array(v0)
    out["times"] = np.array(times)
    out["steps"] = np.array(steps)
    out["stage"] = np.array(st)
    out["boundary_flux_integral"] = np.array(bfi)
    out["volume"] = np.array(vol)
    out["fractional_step_volume"] = np.array(frac)
    out["yieldstep"] = np.array(yieldstep)
    out["finaltime"] = np.array(finaltime)
    save(name, **out)


def integral_fixtures():
    # the inflow case (Dirichlet 2 m west, transmissive east): water enters
    # and leaves through the boundaries; one stage per step (DE0), two (DE1,
    # with rain on a quarter of the domain) and three (DE2)
    integral_fixture("bfi_inflow_de0.npz", build_inflow_bumps, "DE0", 10.0, 30.0)
    integral_fixture("bfi_inflow_de1_rain.npz", build_inflow_bumps, "DE1", 10.0, 30.0, rain=2.0e-4)
    integral_fixture("bfi_inflow_de2.npz", build_inflow_bumps, "DE2", 10.0, 30.0)


def build_inflow_fixed_dt():
    # the inflow case with a fixed flux timestep (generic_domain.py:2332-2359)
    d, extra = build_inflow_bumps()
    d.set_fixed_flux_timestep(0.4)
    extra = dict(extra)
    extra["fixed_flux_timestep"] = np.array(0.4)
    return d, extra


def build_isolated_fast_cell(m=12):
    # a lake at rest with one cell given a large momentum: its speed sits
    # alone in the top bin of the speed histogram, so the protection against
    # isolated degenerate timesteps (generic_domain.py:2520-2560) zeroes it
    pts, elem, bnd = anuga.rectangular_cross(m, m, 120.0, 120.0)
    d = anuga.Domain(pts, elem, bnd)
    d.set_quantity("elevation", lambda x, y: -0.01 * x)
    d.set_quantity("stage", 0.5)
    d.set_quantity("friction", 0.02)
    N = len(d)
    xm = np.zeros(N)
    xm[N // 2 + 7] = 60.0
    d.set_quantity("xmomentum", xm, location="centroids")
    Br = anuga.Reflective_boundary(d)
    d.set_boundary({"left": Br, "right": Br, "top": Br, "bottom": Br})
    d.protect_against_isolated_degenerate_timesteps = True
    calls = {"zeroed": 0}
    orig = d.get_quantity("xmomentum").set_values

    def counting(*a, **k):
        if k.get("indices") is not None:
            calls["zeroed"] += 1
        return orig(*a, **k)
    d.get_quantity("xmomentum").set_values = counting
    d._degenerate_calls = calls
    return d, {"mesh.points": pts, "mesh.elements": elem, "mesh.m": np.array(m)}


def sww_fixture(name, build, flow_algorithm, yieldstep, finaltime, minimum_storable_height):
    """The .sww file the reference writes at every yield (file/sww.py:260-435
    store_timestep through the netCDF stand-in), read back as arrays."""
    import tempfile
    from scipy.io import netcdf_file
    d, extra = build()
    d.set_flow_algorithm(flow_algorithm)
    d.set_multiprocessor_mode(2)
    out = dict(extra)
    Q = d.quantities
    out["init.stage"] = Q["stage"].centroid_values.copy()
    out["init.xmom"] = Q["xmomentum"].centroid_values.copy()
    out["init.ymom"] = Q["ymomentum"].centroid_values.copy()
    out["init.elevation_c"] = Q["elevation"].centroid_values.copy()
    out["init.elevation_v"] = Q["elevation"].vertex_values.copy()
    out["init.friction"] = Q["friction"].centroid_values.copy()
    with tempfile.TemporaryDirectory() as tmp:
        d.set_datadir(tmp)
        d.set_name("ref")
        d.set_minimum_storable_height(minimum_storable_height)
        d.set_store(True)
        for t in d.evolve(yieldstep=yieldstep, finaltime=finaltime):
            pass
        f = netcdf_file(os.path.join(tmp, "ref.sww"), "r", mmap=False)
        for k, v in f.variables.items():
            out["sww." + k] = np.array(v[:])
        f.close()
    out["minimum_storable_height"] = np.array(minimum_storable_height)
    out["yieldstep"] = np.array(yieldstep)
    out["finaltime"] = np.array(finaltime)
    save(name, **out)


def option_fixtures():
    trajectory_fixture("traj_inflow_fixed_dt_de1.npz", build_inflow_fixed_dt, "DE1", 10.0, 30.0)
    trajectory_fixture("traj_isolated_fast_cell_de0.npz", build_isolated_fast_cell, "DE0", 0.5, 1.5)


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "sww":
    # the inflow case: partly dry, so the storable-height mask takes effect
    sww_fixture("sww_inflow_de1.npz", build_inflow_bumps, "DE1", 10.0, 30.0, 0.05)
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "options":
    option_fixtures()
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "integrals":
    integral_fixtures()
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "inlets":
    trajectory_fixture("traj_inlets_de1.npz", build_inlets, "DE1", 1.0, 6.0)
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "flows":
    flow_algorithm_fixtures()
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "boundaries":
    boundary_fixtures()
    integral_fixtures()
    option_fixtures()
    sww_fixture("sww_inflow_de1.npz", build_inflow_bumps, "DE1", 10.0, 30.0, 0.05)
elif __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "riverwall":
    trajectory_fixture("traj_riverwall_de1.npz", build_dam_break_riverwall, "DE1", 1.0, 6.0)
elif __name__ == "__main__":
    p, e, b = anuga.rectangular_cross(3, 2, 3.0, 2.0)
    mesh_fixture("mesh_rect_3x2.npz", p, e, b)
    p, e = delaunay_case()
    mesh_fixture("mesh_delaunay_300.npz", p, e, None)
    phase_fixture("phases_de0.npz", "DE0")
    phase_fixture("phases_de1.npz", "DE1")
    trajectory_fixture("traj_dambreak_de0.npz", build_dam_break, "DE0", 1.0, 4.0)
    trajectory_fixture("traj_inflow_de1.npz", build_inflow_bumps, "DE1", 10.0, 40.0)
    trajectory_fixture("traj_delaunay_rain_de1.npz", build_delaunay_rain, "DE1", 2.0, 6.0)
    trajectory_fixture("traj_inlets_de1.npz", build_inlets, "DE1", 1.0, 6.0)
    flow_algorithm_fixtures()
    trajectory_fixture("traj_riverwall_de1.npz", build_dam_break_riverwall, "DE1", 1.0, 6.0)
    boundary_fixtures()
    integral_fixtures()
    option_fixtures()
    sww_fixture("sww_inflow_de1.npz", build_inflow_bumps, "DE1", 10.0, 30.0, 0.05)
