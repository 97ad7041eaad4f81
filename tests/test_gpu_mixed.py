"""Mixed-precision form (FP32 reconstruction and flux, FP64 accumulation,
FP64 depth and timestep reduction) against the FP64 oracle.

Stated bars: max depth error <= 1 mm against the FP64 oracle over the run;
water volume of a closed domain conserved to 5e-8 relative; a scenario gives
bitwise the same result alone and batched with others in one pool.
"""
import numpy as np
import pytest

from anuga_core_gb300 import workloads
from anuga_core_gb300.mesh import Mesh, rectangular_cross
from anuga_core_gb300.mixed import Pool
from helpers import make_domain, make_oracle, random_state

pytestmark = pytest.mark.gpu

DEPTH_TOL = 1.0e-3   # metres


def _oracle_for(oracle_mod, d, alg, kinds):
    Q = d.quantities
    st = dict(stage=Q["stage"].centroid_values.copy(), xmom=Q["xmomentum"].centroid_values.copy(),
              ymom=Q["ymomentum"].centroid_values.copy(), elevation=Q["elevation"].centroid_values.copy(),
              friction=Q["friction"].centroid_values.copy())
    return make_oracle(oracle_mod, d.mesh, alg, st, kinds), st


def test_inflow_bumps_depth_error_within_1mm(oracle_mod):
    d = workloads.inflow_bumps(m=60, L=600.0, precision="mixed")
    kinds = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    od, _ = _oracle_for(oracle_mod, d, "DE1", kinds)
    for _ in d.evolve(yieldstep=10.0, finaltime=60.0):
        pass
    for _ in od.evolve(yieldstep=10.0, finaltime=60.0):
        pass
    z = d.quantities["elevation"].centroid_values
    h_gpu = np.maximum(d.quantities["stage"].centroid_values - z, 0)
    h_ref = np.maximum(od.stage_c - od.bed_c, 0)
    err = np.abs(h_gpu - h_ref).max()
    assert err <= DEPTH_TOL, err
    assert abs(d.total_steps - od.total_steps) <= max(2, od.total_steps // 50)


@pytest.mark.parametrize("alg", ["DE0_7", "DE1_7"])
def test_other_flow_algorithms_depth_error_within_1mm(oracle_mod, alg):
    """DE0_7 and DE1_7 (other betas and minimum height) on the mixed form."""
    d = workloads.inflow_bumps(m=40, L=400.0, flow_algorithm=alg, precision="mixed")
    kinds = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    od, _ = _oracle_for(oracle_mod, d, alg, kinds)
    for _ in d.evolve(yieldstep=10.0, finaltime=40.0):
        pass
    for _ in od.evolve(yieldstep=10.0, finaltime=40.0):
        pass
    z = d.quantities["elevation"].centroid_values
    err = np.abs(np.maximum(d.quantities["stage"].centroid_values - z, 0) - np.maximum(od.stage_c - od.bed_c, 0)).max()
    assert err <= DEPTH_TOL, err


def test_riverwall_depth_error_within_1mm(golden):
    """Two riverwalls on the dam line (FP32 weir branch of the pool's flux
    kernels) against the reference's trajectory."""
    from anuga_core_gb300.mesh import rectangular_cross as rc
    f = golden("traj_riverwall_de1.npz")
    m = int(f["mesh.m"])
    p, e, b = rc(m, m, 100.0, 100.0)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    walls = {"south": [[50.0, 0.0, -2.2], [50.0, 50.0, -2.0]],
             "north": [[50.0, 50.0, -2.0], [50.0, 80.0, -1.7], [50.0, 100.0, -1.9]]}
    d = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")},
                    precision="mixed")
    d.create_riverwalls(walls, {"north": {"Qfactor": 0.8, "s1": 0.85}})
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        h = np.maximum(d.quantities["stage"].centroid_values - z, 0.0)
        h_ref = np.maximum(f["stage"][i] - z, 0.0)
        assert np.abs(h - h_ref).max() <= DEPTH_TOL, (i, np.abs(h - h_ref).max())


def test_channel_boundaries_depth_error_within_1mm(golden):
    """The four stage/momentum boundaries of the channel case (Flather in its
    wet branch) on the mixed form against the reference's trajectory."""
    from anuga_core_gb300.mesh import rectangular_cross as rc
    import anuga_core_gb300 as agx
    f = golden("traj_channel_boundaries_de1.npz")
    p, e, b = rc(int(f["mesh.m"]), int(f["mesh.n"]), 160.0, 80.0)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")},
                    precision="mixed")
    d.set_boundary({"left": agx.Transmissive_momentum_set_stage_boundary(d, function=lambda t: 0.6 + 0.03 * np.sin(0.3 * t)),
                    "right": agx.Flather_external_stage_zero_velocity_boundary(d, function=lambda t: 0.56 + 0.0 * t),
                    "top": agx.Dirichlet_discharge_boundary(d, stage0=0.6, wh0=0.01),
                    "bottom": agx.Transmissive_stage_zero_momentum_boundary(d)})
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        h = np.maximum(d.quantities["stage"].centroid_values - z, 0.0)
        h_ref = np.maximum(f["stage"][i] - z, 0.0)
        assert np.abs(h - h_ref).max() <= DEPTH_TOL, (i, np.abs(h - h_ref).max())


@pytest.mark.parametrize("name", ["traj_dambreak_de2", "traj_inflow_de2"])
def test_rk3_depth_error_within_1mm(golden, name):
    """DE2 (rk3: a third stage in the pool's step) against the reference's
    trajectory."""
    from anuga_core_gb300.mesh import rectangular_cross as rc
    f = golden(name + ".npz")
    m = int(f["mesh.m"])
    L = float(f["mesh.points"][:, 0].max())
    p, e, b = rc(m, m, L, L)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    if "dambreak" in name:
        kinds = {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}
    else:
        kinds = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                 "top": ("reflective", None), "bottom": ("reflective", None)}
    d = make_domain(p, e, b, "DE2", state, kinds, precision="mixed")
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        h = np.maximum(d.quantities["stage"].centroid_values - z, 0.0)
        h_ref = np.maximum(f["stage"][i] - z, 0.0)
        assert np.abs(h - h_ref).max() <= DEPTH_TOL, (i, np.abs(h - h_ref).max())


def test_dam_break_de0_depth_error_within_1mm(oracle_mod):
    d = workloads.dam_break(m=40, precision="mixed")
    kinds = {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}
    od, _ = _oracle_for(oracle_mod, d, "DE0", kinds)
    for _ in d.evolve(yieldstep=1.0, finaltime=5.0):
        pass
    for _ in od.evolve(yieldstep=1.0, finaltime=5.0):
        pass
    z = d.quantities["elevation"].centroid_values
    err = np.abs(np.maximum(d.quantities["stage"].centroid_values - z, 0) - np.maximum(od.stage_c - od.bed_c, 0)).max()
    assert err <= DEPTH_TOL, err


def test_delaunay_dry_start_inflow_depth_error_within_1mm(oracle_mod):
    """Unstructured mesh (jittered-lattice Delaunay), dry start, Dirichlet
    inflow on the west side and Manning friction: the serving workload's
    scenario form."""
    from anuga_core_gb300.serve import Request, delaunay_mesh, scenario_state
    mesh = delaunay_mesh(8000, seed=3)
    req = Request(rid=0, arrival=0.0, kind="delaunay", cells=8000, seed=41, finaltime=20.0, inflow_stage=2.0)
    z, stage, eta = scenario_state(mesh, req)
    st = dict(elevation=z, stage=stage, xmom=0 * z, ymom=0 * z, friction=eta)
    kinds = {"inflow": ("dirichlet", (2.0, 0.0, 0.0)), "wall": ("reflective", None)}
    d = make_domain(mesh.nodes, mesh.triangles, mesh.boundary, "DE1", st, kinds, precision="mixed")
    od = make_oracle(oracle_mod, mesh, "DE1", st, kinds)
    for _ in d.evolve(yieldstep=5.0, finaltime=20.0):
        pass
    for _ in od.evolve(yieldstep=5.0, finaltime=20.0):
        pass
    h_gpu = np.maximum(d.quantities["stage"].centroid_values - z, 0)
    h_ref = np.maximum(od.stage_c - od.bed_c, 0)
    assert h_ref.max() > 0.1                       # the inflow has entered
    err = np.abs(h_gpu - h_ref).max()
    assert err <= DEPTH_TOL, err


def test_rain_polygon_depth_error_within_1mm(oracle_mod):
    """The unstructured rain-and-inflow workload (random polygon, refined
    region, value-noise bed, rain patch, inflow segment) at 20k triangles."""
    d = workloads.rain_polygon(target_cells=2.0e4, precision="mixed")
    op = d.fractional_step_operators[1]
    kinds = {"inflow": ("dirichlet", (3.0, 0.0, 0.0)), "wall": ("reflective", None)}
    Q = d.quantities
    st = dict(stage=Q["stage"].centroid_values.copy(), xmom=Q["xmomentum"].centroid_values.copy(),
              ymom=Q["ymomentum"].centroid_values.copy(), elevation=Q["elevation"].centroid_values.copy(),
              friction=Q["friction"].centroid_values.copy())
    od = make_oracle(oracle_mod, d.mesh, "DE1", st, kinds, rates=[(op.indices, op.rate)])
    for _ in d.evolve(yieldstep=30.0, finaltime=120.0):
        pass
    for _ in od.evolve(yieldstep=30.0, finaltime=120.0):
        pass
    z = Q["elevation"].centroid_values
    h_gpu = np.maximum(Q["stage"].centroid_values - z, 0)
    h_ref = np.maximum(od.stage_c - od.bed_c, 0)
    err = np.abs(h_gpu - h_ref).max()
    assert err <= DEPTH_TOL, err
    A = d.mesh.areas
    vol_gpu, vol_ref = float(np.sum(h_gpu * A)), float(np.sum(h_ref * A))
    assert abs(vol_gpu - vol_ref) <= 1e-5 * vol_ref, (vol_gpu, vol_ref)


@pytest.mark.parametrize("m,alg", [(40, "DE0"), (40, "DE1"), (100, "DE1"), (40, "DE2")])
def test_closed_domain_conserves_volume(m, alg):
    """A dam break between walls (no cell dries): the FP64 depth update of
    FP32 edge fluxes, each edge evaluated from both sides, keeps the water
    volume to a few 1e-9 relative over the run (measured up to 6.9e-9)."""
    d = workloads.dam_break(m=m, flow_algorithm=alg, precision="mixed")
    v0 = d.get_water_volume()
    for _ in d.evolve(yieldstep=2.0, finaltime=10.0):
        pass
    v1 = d.get_water_volume()
    assert abs(v1 - v0) / v0 <= 5e-8, (v0, v1)


def test_rain_adds_the_expected_volume():
    d = workloads.dam_break(m=30, flow_algorithm="DE1", precision="mixed")
    import anuga_core_gb300 as agx
    c = d.get_centroid_coordinates()
    idx = np.nonzero((c[:, 0] > 20) & (c[:, 0] < 60))[0]
    rate = 0.002
    agx.Rate_operator(d, rate=rate, indices=idx)
    v0 = d.get_water_volume()
    for _ in d.evolve(yieldstep=1.0, finaltime=4.0):
        pass
    v1 = d.get_water_volume()
    expect = rate * 4.0 * d.mesh.areas[idx].sum()
    assert abs((v1 - v0) - expect) / expect <= 1e-5


def _pool_case(seed, m):
    p, e, b = rectangular_cross(m, m, 10.0 * m, 10.0 * m)
    mesh = Mesh(p, e, b)
    st = random_state(mesh, seed)
    kinds = {"left": ("dirichlet", (float(np.max(st["stage"])) + 0.1, 0.0, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    return p, e, b, st, kinds


def test_scenario_same_alone_and_batched():
    cases = [_pool_case(s, m) for s, m in ((1, 12), (2, 30), (3, 7), (4, 21))]
    alone = []
    for p, e, b, st, kinds in cases:
        d = make_domain(p, e, b, "DE1", st, kinds, precision="mixed")
        d.advance_steps(25)
        alone.append(d.quantities["stage"].centroid_values.copy())
    # batched: all four in one pool, advanced by the same graph launches
    doms = [make_domain(p, e, b, "DE1", st, kinds, precision="mixed") for p, e, b, st, kinds in cases]
    from anuga_core_gb300.batch import Batch
    B = Batch(doms)
    B.advance_steps(25)
    for i, d in enumerate(doms):
        got = B.get_centroids(i)["stage_c"]
        assert np.array_equal(got, alone[i]), i


def test_snapshot_restore_and_autotune_leave_state_unchanged():
    p, e, b, st, kinds = _pool_case(9, 24)
    d1 = make_domain(p, e, b, "DE1", st, kinds, precision="mixed")
    d1.advance_steps(10)
    ref = d1.quantities["stage"].centroid_values.copy()
    d2 = make_domain(p, e, b, "DE1", st, kinds, precision="mixed")
    d2._ensure_device()
    from anuga_core_gb300.autotune import tune_pool, VARIANTS, NAMES
    pool = d2._scn.pool
    res, best = tune_pool(pool, steps=3, reps=1)
    assert set(NAMES.values()) <= set(res) and best in res      # every form timed, the fastest kept
    d2.advance_steps(10)
    got = d2.quantities["stage"].centroid_values
    assert np.array_equal(got, ref)
    # every kernel variant computes the same result
    outs = []
    for v in VARIANTS:
        d3 = make_domain(p, e, b, "DE1", st, kinds, precision="mixed")
        d3._ensure_device()
        d3._scn.pool.set_variant(*v)
        d3.advance_steps(10)
        outs.append(d3.quantities["stage"].centroid_values.copy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def _same_state(got, want, d, name):
    """Momenta come back bitwise; the stage is stored as depth (stage - bed),
    so it comes back to within one rounding of the bed's magnitude."""
    if name != "stage_c":
        assert np.array_equal(got, want), name
        return
    z = d.quantities["elevation"].centroid_values
    tol = 2.0 * np.finfo(float).eps * max(np.abs(want).max(), np.abs(z).max(), 1.0)
    assert np.abs(got - want).max() <= tol, name


def test_state_exchange_in_one_call_matches_per_field():
    d = workloads.dam_break(m=30, flow_algorithm="DE1", precision="mixed")
    for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
        pass
    scn = d._scn
    w, uh, vh = scn.get_state()
    assert np.array_equal(w, scn.get("stage_c")) and np.array_equal(uh, scn.get("xmom_c"))
    assert np.array_equal(vh, scn.get("ymom_c"))
    rng = np.random.default_rng(3)
    w2, uh2, vh2 = w + 0.01 * rng.uniform(size=w.size), uh * 0.5, vh * 0.25
    scn.set_state(w2, uh2, vh2)
    for name, ref in (("stage_c", w2), ("xmom_c", uh2), ("ymom_c", vh2)):
        _same_state(scn.get(name), ref, d, name)


def test_state_exchange_with_page_locked_buffers():
    """Page-locked host buffers are read and written by the device directly;
    the values are the same as through the copying path."""
    import torch
    d = workloads.dam_break(m=30, flow_algorithm="DE1", precision="mixed")
    for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
        pass
    scn = d._scn
    N = len(d)
    pin = [torch.empty(N, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    scn.get_state(*pin)
    ref = scn.get_state()                      # pageable numpy arrays: the copying path
    for a, b in zip(pin, ref):
        assert np.array_equal(a, b)
    rng = np.random.default_rng(4)
    new = [ref[0] + 0.01 * rng.uniform(size=N), ref[1] * 0.5, ref[2] * 0.25]
    for a, b in zip(pin, new):
        a[:] = b
    scn.set_state(*pin)
    for name, b in zip(("stage_c", "xmom_c", "ymom_c"), new):
        _same_state(scn.get(name), b, d, name)


def test_full_size_mixed_against_plain_fp64():
    """The benchmark's own workload at full size (inflow over bumps, 4.0M
    triangles, DE1): 150 steps of the mixed form against the bit-exact plain
    FP64 form on the same GPU; max depth difference within 1 mm."""
    out = []
    for prec in ("fp64", "mixed"):
        d = workloads.inflow_bumps(m=1000, precision=prec)
        d.distribute_to_vertices_and_edges()
        d.advance_steps(150)
        Q = d.quantities
        out.append((np.maximum(Q["stage"].centroid_values - Q["elevation"].centroid_values, 0.0), d.relative_time))
        del d
    (h64, t64), (h32, t32) = out
    assert abs(t64 - t32) <= 1e-3 * t64                  # the same simulated time within 0.1%
    assert h64.max() > 1.0 and (h64 == 0.0).any()        # wet and dry cells
    err = float(np.abs(h32 - h64).max())
    assert err <= DEPTH_TOL, err
