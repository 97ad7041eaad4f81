"""Parity of the plain FP64 GPU path against the reference and the oracle.

Bar: bit-exact for every phase output from an identical input state (the
reference's own cross-implementation test pattern, shallow_water/tests/
test_DE_openmp.py:31-170), except Manning's semi-implicit terms, where CUDA's
pow may differ from the C library's in the last place (tolerance 1e-14
normwise).  Trajectories: flux timesteps bit-exact per step until the first
pow rounding difference, states within 1e-12 normwise per step.
"""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300.mesh import Mesh, rectangular_cross
from helpers import make_domain, make_oracle, random_state, normwise

pytestmark = pytest.mark.gpu

POW_TOL = 1e-14
STATE_TOL = 1e-12


def _phase_domain(f, alg):
    m, n, L1, L2 = f["params"]
    p, e, b = rectangular_cross(int(m), int(n), L1, L2)
    state = dict(stage=f["in.stage.centroid_values"], xmom=f["in.xmomentum.centroid_values"],
                 ymom=f["in.ymomentum.centroid_values"], elevation=f["in.elevation.centroid_values"],
                 friction=f["in.friction.centroid_values"])
    kinds = {"left": ("dirichlet", (1.3, 0.05, -0.02)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    return make_domain(p, e, b, alg, state, kinds)


@pytest.mark.parametrize("alg", ["de0", "de1"])
def test_phases_match_reference(golden, alg):
    f = golden("phases_%s.npz" % alg)
    d = _phase_domain(f, alg.upper())
    Q = d.quantities
    d.protect_against_infinitesimal_and_negative_heights()
    assert np.array_equal(Q["stage"].centroid_values, f["protect.stage.centroid_values"])
    assert np.array_equal(Q["xmomentum"].centroid_values, f["protect.xmomentum.centroid_values"])
    assert np.array_equal(Q["ymomentum"].centroid_values, f["protect.ymomentum.centroid_values"])
    d.distribute_to_vertices_and_edges()
    for q in ("stage", "xmomentum", "ymomentum", "elevation", "height"):
        assert np.array_equal(Q[q].edge_values, f["extrap.%s.edge_values" % q]), q
        assert np.array_equal(Q[q].vertex_values, f["extrap.%s.vertex_values" % q]), q
    for q in ("stage", "xmomentum", "ymomentum", "height"):
        assert np.array_equal(Q[q].centroid_values, f["extrap.%s.centroid_values" % q]), q
    d.update_boundary()
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(Q[q].boundary_values, f["bc.%s.boundary_values" % q]), q
    d.compute_fluxes()
    assert d.flux_timestep == float(f["flux.flux_timestep"])
    assert np.array_equal(d.max_speed, f["flux.max_speed"])
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(Q[q].explicit_update, f["flux.%s.explicit_update" % q]), q
    d.compute_forcing_terms()
    for q in ("xmomentum", "ymomentum"):
        assert normwise(Q[q].semi_implicit_update, f["forcing.%s.semi_implicit_update" % q]) <= POW_TOL
    d.timestep = float(f["update.timestep"])
    d.update_conserved_quantities()
    for q in ("stage", "xmomentum", "ymomentum"):
        assert normwise(Q[q].centroid_values, f["update.%s.centroid_values" % q]) <= POW_TOL, q


TRAJ = {
    "traj_dambreak_de0": ("DE0", {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}, False),
    "traj_inflow_de1": ("DE1", {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                                "top": ("reflective", None), "bottom": ("reflective", None)}, False),
    "traj_delaunay_rain_de1": ("DE1", {"exterior": ("reflective", None)}, True),
    "traj_dambreak_de2": ("DE2", {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}, False),
    "traj_inflow_de2": ("DE2", {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                                "top": ("reflective", None), "bottom": ("reflective", None)}, False),
    "traj_inflow_de0_7": ("DE0_7", {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                                    "top": ("reflective", None), "bottom": ("reflective", None)}, False),
    "traj_inflow_de1_7": ("DE1_7", {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                                    "top": ("reflective", None), "bottom": ("reflective", None)}, False),
}


@pytest.mark.parametrize("name", sorted(TRAJ))
def test_trajectory_matches_reference(golden, name):
    alg, kinds, rain = TRAJ[name]
    f = golden(name + ".npz")
    p, e = f["mesh.points"], f["mesh.elements"]
    if "mesh.m" in f:
        m = int(f["mesh.m"])
        L = float(p[:, 0].max())
        p2, e2, b = rectangular_cross(m, m, L, L)
        assert np.array_equal(p2, p)
    else:
        b = None
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    rates = [(f["rain.indices"], float(f["rain.rate"]))] if rain else []
    d = make_domain(p, e, b, alg, state, kinds, rates=rates)
    times, steps = [], []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        times.append(t)
        steps.append(d.number_of_steps)
        Q = d.quantities
        assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, (name, i)
        assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, (name, i)
        assert normwise(Q["ymomentum"].centroid_values, f["ymom"][i]) <= 1e-10, (name, i)
    assert np.allclose(times, f["times"], rtol=0, atol=1e-12)
    assert steps == list(f["steps"])


def _rect_case(m, n, seed, alg):
    p, e, b = rectangular_cross(m, n, 10.0 * m, 10.0 * n)
    mesh = Mesh(p, e, b)
    st = random_state(mesh, seed)
    kinds = {"left": ("dirichlet", (float(np.max(st["stage"])) + 0.2, 0.1, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    return p, e, b, mesh, st, kinds


def _delaunay_case(npts, seed):
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 300, (npts, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    mesh = Mesh(pts, tri, None)
    st = random_state(mesh, seed + 1)
    return pts, tri, None, mesh, st, {"exterior": ("reflective", None)}


CASES = [("rect", 40, 30, 5, "DE0"), ("rect", 40, 30, 6, "DE1"), ("delaunay", 3000, 0, 7, "DE1"),
         ("delaunay", 2000, 0, 8, "DE0")]


@pytest.mark.parametrize("kind,a,b_,seed,alg", CASES)
def test_one_step_from_identical_state(oracle_mod, kind, a, b_, seed, alg):
    """flux timestep bit-exact and every phase output equal for one step."""
    p, e, b, mesh, st, kinds = _rect_case(a, b_, seed, alg) if kind == "rect" else _delaunay_case(a, seed)
    d = make_domain(p, e, b, alg, st, kinds)
    od = make_oracle(oracle_mod, mesh, alg, st, kinds)
    d.distribute_to_vertices_and_edges()
    od.distribute_to_vertices_and_edges()
    Q = d.quantities
    assert np.array_equal(Q["stage"].edge_values.ravel(), od.stage_e)
    assert np.array_equal(Q["xmomentum"].edge_values.ravel(), od.xmom_e)
    assert np.array_equal(Q["height"].edge_values.ravel(), od.height_e)
    d.update_boundary()
    od.update_boundary()
    d.compute_fluxes()
    dt = od.compute_fluxes(0)
    assert d.flux_timestep == dt
    assert np.array_equal(Q["stage"].explicit_update, od.stage_x)
    assert np.array_equal(Q["xmomentum"].explicit_update, od.xmom_x)
    assert np.array_equal(Q["ymomentum"].explicit_update, od.ymom_x)
    assert np.array_equal(d.max_speed, od.max_speed)


@pytest.mark.parametrize("kind,a,b_,seed,alg", CASES)
def test_frictionless_trajectory_bit_exact(oracle_mod, kind, a, b_, seed, alg):
    """Without Manning friction every operation is +,-,*,/,sqrt (correctly
    rounded on both sides), so whole trajectories must be bit-identical."""
    p, e, b, mesh, st, kinds = _rect_case(a, b_, seed, alg) if kind == "rect" else _delaunay_case(a, seed)
    st = dict(st, friction=np.zeros_like(st["friction"]))
    d = make_domain(p, e, b, alg, st, kinds)
    od = make_oracle(oracle_mod, mesh, alg, st, kinds)
    ys, ft = 0.5, 2.0
    got, ref, err_g, err_r = [], [], None, None
    try:
        for t in d.evolve(yieldstep=ys, finaltime=ft):
            got.append((t, d.number_of_steps, d.quantities["stage"].centroid_values.copy(),
                        d.quantities["xmomentum"].centroid_values.copy(),
                        d.quantities["ymomentum"].centroid_values.copy()))
    except agx._lib.AgxError as e:
        err_g = e
    try:
        for t in od.evolve(yieldstep=ys, finaltime=ft):
            ref.append((t, od.number_of_steps, od.stage_c.copy(), od.xmom_c.copy(), od.ymom_c.copy()))
    except RuntimeError as e:
        err_r = e
    # the reference aborts on a too-small timestep at first order
    # (generic_domain.py:2369-2395); both sides must stop at the same point
    assert (err_g is None) == (err_r is None), (err_g, err_r)
    if err_g is not None:
        assert err_g.code == -6 and "Too small timestep" in str(err_r)
    assert len(got) == len(ref)
    for g, r in zip(got, ref):
        assert g[0] == r[0] and g[1] == r[1]
        for a1, a2 in zip(g[2:], r[2:]):
            assert np.array_equal(a1, a2)


@pytest.mark.parametrize("kind,a,b_,seed,alg", CASES[:3])
def test_each_step_with_friction_within_1e12(oracle_mod, kind, a, b_, seed, alg):
    """With friction, each step from an identical state agrees to 1e-12
    (normwise) and the flux timestep is bit-exact; the state is re-synced
    from the oracle before every step.  The drift over a free run is
    reported by test_friction_trajectory_drift."""
    p, e, b, mesh, st, kinds = _rect_case(a, b_, seed, alg) if kind == "rect" else _delaunay_case(a, seed)
    d = make_domain(p, e, b, alg, st, kinds)
    od = make_oracle(oracle_mod, mesh, alg, st, kinds)
    gen = od.evolve(yieldstep=1e300, finaltime=None)
    next(gen)
    od.relative_yieldtime = 1e300
    Q = d.quantities
    for step in range(12):
        Q["stage"].set_values(od.stage_c.copy(), location="centroids")
        Q["xmomentum"].set_values(od.xmom_c.copy(), location="centroids")
        Q["ymomentum"].set_values(od.ymom_c.copy(), location="centroids")
        st_ = d.advance_steps(1)
        if od.timestepping_method == "euler":
            od.euler_step(1e300, None)
        else:
            od.rk2_step(1e300, None)
        od.relative_time += od.timestep
        assert st_.flux_timestep == od.flux_timestep or alg == "DE1", step   # DE1 reports stage-2's value
        assert st_.last_timestep == od.timestep, step
        assert normwise(Q["stage"].centroid_values, od.stage_c) <= STATE_TOL, step
        assert normwise(Q["xmomentum"].centroid_values, od.xmom_c) <= STATE_TOL, step
        assert normwise(Q["ymomentum"].centroid_values, od.ymom_c) <= STATE_TOL, step


def test_friction_trajectory_drift(oracle_mod):
    """Free-running drift with friction (CUDA pow vs C library pow): stated
    bound 1e-5 m in stage after 2 s of a wet/dry DE1 run."""
    p, e, b, mesh, st, kinds = _delaunay_case(3000, 7)
    d = make_domain(p, e, b, "DE1", st, kinds)
    od = make_oracle(oracle_mod, mesh, "DE1", st, kinds)
    for _ in d.evolve(yieldstep=2.0, finaltime=2.0):
        pass
    for _ in od.evolve(yieldstep=2.0, finaltime=2.0):
        pass
    err = np.abs(d.quantities["stage"].centroid_values - od.stage_c).max()
    assert err <= 1e-5, err


def test_lake_at_rest_stays_at_rest():
    p, e, b = rectangular_cross(20, 20, 100.0, 100.0)
    mesh = Mesh(p, e, b)
    C = mesh.centroid_coordinates
    z = 0.5 * np.sin(C[:, 0] / 10.0) * np.cos(C[:, 1] / 13.0)
    st = dict(elevation=z, stage=np.full(len(z), 1.0), xmom=np.zeros(len(z)), ymom=np.zeros(len(z)),
              friction=np.full(len(z), 0.03))
    kinds = {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}
    for alg in ("DE0", "DE1"):
        d = make_domain(p, e, b, alg, st, kinds)
        for _ in d.evolve(yieldstep=1.0, finaltime=3.0):
            pass
        assert np.abs(d.quantities["stage"].centroid_values - 1.0).max() < 1e-12
        assert np.abs(d.quantities["xmomentum"].centroid_values).max() < 1e-12


def test_single_triangle_and_dry_domain(oracle_mod):
    # one triangle: three boundary edges (number_of_boundaries == 3 branch)
    p = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    e = np.array([[0, 1, 2]])
    mesh = Mesh(p, e, None)
    st = dict(elevation=np.zeros(1), stage=np.full(1, 0.5), xmom=np.full(1, 0.1), ymom=np.zeros(1),
              friction=np.zeros(1))
    kinds = {"exterior": ("reflective", None)}
    d = make_domain(p, e, None, "DE0", st, kinds)
    od = make_oracle(oracle_mod, mesh, "DE0", st, kinds)
    for _ in d.evolve(yieldstep=0.1, finaltime=0.3):
        pass
    for _ in od.evolve(yieldstep=0.1, finaltime=0.3):
        pass
    assert np.array_equal(d.quantities["stage"].centroid_values, od.stage_c)
    # completely dry domain: nothing moves, timestep is the maximum
    p, e, b = rectangular_cross(5, 5, 10.0, 10.0)
    mesh = Mesh(p, e, b)
    z = mesh.centroid_coordinates[:, 0] * 0.1
    st = dict(elevation=z, stage=z.copy(), xmom=np.zeros_like(z), ymom=np.zeros_like(z), friction=np.zeros_like(z))
    d = make_domain(p, e, b, "DE1", st, {t: ("reflective", None) for t in mesh.tag_boundary_cells})
    for _ in d.evolve(yieldstep=5.0, finaltime=5.0):
        pass
    assert np.array_equal(d.quantities["stage"].centroid_values, z)
    assert d.total_steps == 1


def test_fp64_throughput_probe():
    """The FP64 ceiling the plain path is reported against: positive, and DFMA
    faster than the IEEE division and square root."""
    from anuga_core_gb300 import _lib
    r = _lib.fp64_throughput()
    assert 10.0 < r["dfma_gops"] < 1.0e5
    assert 0.0 < r["ddiv_gops"] < r["dfma_gops"]
    assert 0.0 < r["dsqrt_gops"] < r["dfma_gops"]


def test_state_exchange_in_one_call_matches_per_field():
    from anuga_core_gb300 import workloads
    d = workloads.dam_break(m=20)
    for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
        pass
    scn = d._scn
    w, uh, vh = scn.get_state()
    assert np.array_equal(w, scn.get("stage_c")) and np.array_equal(vh, scn.get("ymom_c"))
    scn.set_state(w * 1.001, uh, vh * 0.5)
    assert np.array_equal(scn.get("stage_c"), w * 1.001) and np.array_equal(scn.get("ymom_c"), vh * 0.5)


def test_rate_given_as_a_function_runs_on_the_device():
    """A Rate_operator whose rate is a Python function makes the domain step
    from the host, phase by phase; the rate is still applied by the device.
    With a function that returns a constant, the result is bit-identical to
    the device step loop with that constant."""
    from anuga_core_gb300 import workloads
    out = []
    for rate in (2.0e-4, lambda t: 2.0e-4):
        d = workloads.dam_break(m=20, flow_algorithm="DE1")
        idx = np.arange(0, len(d), 3)
        op = agx.Rate_operator(d, rate=rate, indices=idx)
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        assert d._device_loop_ok() == (not callable(rate))
        out.append((d.quantities["stage"].centroid_values.copy(), d.total_steps, op.get_Q()))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][2] > 0 and abs(out[0][2] - out[1][2]) <= 1e-12 * out[0][2]


RIVERWALLS = {"south": [[50.0, 0.0, -2.2], [50.0, 50.0, -2.0]],
              "north": [[50.0, 50.0, -2.0], [50.0, 80.0, -1.7], [50.0, 100.0, -1.9]]}


def test_riverwall_trajectory_matches_reference(golden):
    """Two riverwalls on the dam line (weir flux, per-side evaluation of the
    wall edges) against the reference's trajectory."""
    f = golden("traj_riverwall_de1.npz")
    m = int(f["mesh.m"])
    p, e, b = rectangular_cross(m, m, 100.0, 100.0)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")})
    d.create_riverwalls(RIVERWALLS, {"north": {"Qfactor": 0.8, "s1": 0.85}})
    assert np.array_equal(d.edge_river_wall_counter, f["rw.edge_river_wall_counter"])
    steps = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        steps.append(d.number_of_steps)
        Q = d.quantities
        assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, i
        assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        assert normwise(Q["ymomentum"].centroid_values, f["ymom"][i]) <= 1e-10, i
    assert steps == list(f["steps"])
    # the walls hold part of the water back: the run differs from one without them
    d2 = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")})
    for _ in d2.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"])):
        pass
    assert np.abs(d2.quantities["stage"].centroid_values - f["stage"][-1]).max() > 1e-3


def _channel_domain(f, alg, precision="fp64", constant=False):
    m, n = int(f["mesh.m"]), int(f["mesh.n"])
    p, e, b = rectangular_cross(m, n, 160.0, 80.0)
    assert np.array_equal(p, f["mesh.points"])
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p, e, b, alg, state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")},
                    precision=precision)
    left = 0.6 if constant else (lambda t: 0.6 + 0.03 * np.sin(0.3 * t))
    right = 0.56 if constant else (lambda t: 0.56 + 0.0 * t)
    d.set_boundary({"left": agx.Transmissive_momentum_set_stage_boundary(d, function=left),
                    "right": agx.Flather_external_stage_zero_velocity_boundary(d, function=right),
                    "top": agx.Dirichlet_discharge_boundary(d, stage0=0.6, wh0=0.01),
                    "bottom": agx.Transmissive_stage_zero_momentum_boundary(d)})
    return d


@pytest.mark.parametrize("alg", ["DE1", "DE0"])
def test_channel_boundaries_match_reference(golden, alg):
    """Transmissive_momentum_set_stage, Flather (wet branch), Dirichlet_discharge
    and Transmissive_stage_zero_momentum boundaries against the reference."""
    f = golden("traj_channel_boundaries_%s.npz" % alg.lower())
    d = _channel_domain(f, alg)
    steps = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        steps.append(d.number_of_steps)
        Q = d.quantities
        assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, i
        assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        assert normwise(Q["ymomentum"].centroid_values, f["ymom"][i]) <= 1e-10, i
    assert steps == list(f["steps"])


def test_channel_boundaries_in_the_device_loop(golden):
    """Constant stages run in the device step loop; the same constants given
    as functions run the host-driven step: bitwise the same."""
    f = golden("traj_channel_boundaries_de1.npz")
    out = []
    for constant in (True, False):
        d = _channel_domain(f, "DE1", constant=constant)
        if not constant:   # functions returning the constants
            d.boundary_map["left"].function = lambda t: 0.6
            d.boundary_map["right"].function = lambda t: 0.56
            d.boundary_map["left"].device_loop = d.boundary_map["right"].device_loop = False
        for _ in d.evolve(yieldstep=2.0, finaltime=8.0):
            pass
        assert d._device_loop_ok() == constant
        out.append((d.quantities["stage"].centroid_values.copy(), d.total_steps))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_characteristic_boundary_matches_reference(golden, precision):
    """Characteristic_stage_boundary on the inflow side: plain FP64 to the
    trajectory tolerance, mixed within 1 mm of depth."""
    f = golden("traj_channel_characteristic_de1.npz")
    d = _channel_domain(f, "DE1", precision=precision)
    d.set_boundary({"left": agx.Characteristic_stage_boundary(d, function=lambda t: 0.6 + 0.03 * np.sin(0.3 * t)),
                    "right": agx.Transmissive_boundary(d), "top": agx.Reflective_boundary(d),
                    "bottom": agx.Reflective_boundary(d)})
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        Q = d.quantities
        if precision == "fp64":
            assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, i
            assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        else:
            err = np.abs(np.maximum(Q["stage"].centroid_values - z, 0) - np.maximum(f["stage"][i] - z, 0)).max()
            assert err <= 1.0e-3, (i, err)


def test_time_space_boundary_matches_reference(golden):
    f = golden("traj_channel_time_space_de1.npz")
    d = _channel_domain(f, "DE1")
    fn = lambda t, x, y: [0.6 + 0.02 * np.sin(0.3 * t) * np.cos(y / 20.0), 0.0, 0.0]
    d.set_boundary({"left": agx.Time_space_boundary(d, function=fn), "right": agx.Transmissive_boundary(d),
                    "top": agx.Reflective_boundary(d), "bottom": agx.Reflective_boundary(d)})
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        Q = d.quantities
        assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, i
        assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_inflow_boundary_matches_reference(golden, precision):
    f = golden("traj_channel_inflow_de1.npz")
    d = _channel_domain(f, "DE1", precision=precision)
    d.set_boundary({"left": agx.Inflow_boundary(d, rate=2.0), "right": agx.Transmissive_boundary(d),
                    "top": agx.Reflective_boundary(d), "bottom": agx.Compute_fluxes_boundary()})
    d.set_boundary({"bottom": agx.Reflective_boundary(d)})
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        Q = d.quantities
        if precision == "fp64":
            assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= STATE_TOL, i
            assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        else:
            err = np.abs(np.maximum(Q["stage"].centroid_values - z, 0) - np.maximum(f["stage"][i] - z, 0)).max()
            assert err <= 1.0e-3, (i, err)


def test_time_stage_zero_momentum_matches_oracle(oracle_mod, golden):
    f = golden("traj_channel_boundaries_de1.npz")
    fn = lambda t: 0.6 + 0.05 * np.sin(0.2 * t)
    d = _channel_domain(f, "DE1")
    Br = agx.Reflective_boundary(d)
    d.set_boundary({"left": agx.Time_stage_zero_momentum_boundary(d, function=fn), "right": Br, "top": Br,
                    "bottom": Br})
    kinds = {"left": ("time_stage_zero_momentum", fn), "right": ("reflective", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    st = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"], elevation=f["init.elevation_c"],
              friction=f["init.friction"])
    od = make_oracle(oracle_mod, d.mesh, "DE1", st, kinds)
    od.set_bed_vertex_values(f["init.elevation_v"])
    for _ in d.evolve(yieldstep=2.0, finaltime=10.0):
        pass
    for _ in od.evolve(yieldstep=2.0, finaltime=10.0):
        pass
    assert d.total_steps == od.total_steps
    assert normwise(d.quantities["stage"].centroid_values, od.stage_c) <= STATE_TOL


def test_rk3_host_steps_equal_the_device_loop():
    """DE2 (rk3) through the per-phase host step (a rate given as a function
    of time) and through the device step loop (the same constant rate):
    bitwise the same states and step counts."""
    from anuga_core_gb300 import workloads
    out = []
    for rate in (1.0e-4, lambda t: 1.0e-4):
        d = workloads.dam_break(m=16, flow_algorithm="DE2")
        assert d.get_timestepping_method() == "rk3"
        idx = np.arange(0, len(d), 2)
        op = agx.Rate_operator(d, rate=rate, indices=idx)
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        assert d._device_loop_ok() == (not callable(rate))
        out.append((d.quantities["stage"].centroid_values.copy(), d.quantities["xmomentum"].centroid_values.copy(),
                    d.total_steps, op.get_Q()))
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert abs(out[0][3] - out[1][3]) <= 1e-12 * abs(out[0][3])


INLET_REGIONS = {"a": ([[10.0, 20.0], [30.0, 20.0], [30.0, 60.0], [10.0, 60.0]], {}),
                 "b": ([[90.0, 10.0], [110.0, 10.0], [110.0, 30.0], [90.0, 30.0]], dict(zero_velocity=True)),
                 "c": ([[50.0, 70.0], [70.0, 70.0]], dict(velocity=[0.2, 0.0]))}


def _inlet_domain(f, callable_q=False):
    p, e, b = rectangular_cross(12, 8, 120.0, 80.0)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")})
    ops = []
    for k, (region, kw) in INLET_REGIONS.items():
        q = float(f["inlet_%s.Q" % k])
        ops.append(agx.Inlet_operator(d, region, Q=(lambda t, q=q: q) if callable_q else q, **kw))
    return d, ops


def test_inlets_match_reference(golden):
    """Inlet_operator on the device (inflow, extraction with zero velocity, a
    line inlet with imposed velocity) against the reference trajectory: the
    device sums the inlet volume and the cumulative areas in another order
    than numpy, so the states agree to 1e-12 normwise, not bitwise."""
    f = golden("traj_inlets_de1.npz")
    d, ops = _inlet_domain(f)
    for k, op in zip(INLET_REGIONS, ops):
        assert np.array_equal(op.indices, np.sort(f["inlet_%s.indices" % k]))
    steps = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        steps.append(d.number_of_steps)
        Q = d.quantities
        assert normwise(Q["stage"].centroid_values, f["stage"][i]) <= 1e-12, i
        assert normwise(Q["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        assert normwise(Q["ymomentum"].centroid_values, f["ymom"][i]) <= 1e-10, i
    assert steps == list(f["steps"])
    T = float(f["finaltime"])
    assert abs(ops[0].get_total_applied_volume() - 1.5 * T) <= 1e-9
    assert abs(ops[2].get_total_applied_volume() - 0.8 * T) <= 1e-9


def test_inlet_q_as_a_function_runs_on_the_device(golden):
    f = golden("traj_inlets_de1.npz")
    out = []
    for callable_q in (False, True):
        d, ops = _inlet_domain(f, callable_q)
        for _ in d.evolve(yieldstep=1.0, finaltime=3.0):
            pass
        assert d._device_loop_ok() == (not callable_q)
        out.append(d.quantities["stage"].centroid_values.copy())
    assert np.array_equal(out[0], out[1])
