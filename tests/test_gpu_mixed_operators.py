"""Operators and time-dependent boundaries on the mixed-precision form.

Inlet_operator and Rate_operator run in the pool's step loop when their
values are constants; when a rate, a discharge or a boundary value is a
Python function of time, the domain steps one device step at a time and
applies the operators after each step (agx_pool_apply_operator).

Bars: depths within 1 mm of the reference's trajectory (inlets, from the
golden fixture) or of the plain FP64 form (time-function boundary); a
function that returns a constant gives bitwise the state of the step loop
with that constant; applied inlet volumes equal Q x elapsed time.
"""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300 import workloads
from anuga_core_gb300.mesh import rectangular_cross
from helpers import make_domain

pytestmark = pytest.mark.gpu

DEPTH_TOL = 1.0e-3   # metres

INLET_REGIONS = {"a": ([[10.0, 20.0], [30.0, 20.0], [30.0, 60.0], [10.0, 60.0]], {}),
                 "b": ([[90.0, 10.0], [110.0, 10.0], [110.0, 30.0], [90.0, 30.0]], dict(zero_velocity=True)),
                 "c": ([[50.0, 70.0], [70.0, 70.0]], dict(velocity=[0.2, 0.0]))}


def _inlet_domain(f, callable_q=False):
    p, e, b = rectangular_cross(12, 8, 120.0, 80.0)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p, e, b, "DE1", state, {t: ("reflective", None) for t in ("left", "right", "top", "bottom")},
                    precision="mixed")
    ops = []
    for k, (region, kw) in INLET_REGIONS.items():
        q = float(f["inlet_%s.Q" % k])
        ops.append(agx.Inlet_operator(d, region, Q=(lambda t, q=q: q) if callable_q else q, **kw))
    return d, ops


def test_inlets_match_reference_within_1mm(golden):
    """Inflow, extraction with zero velocity and a line inlet with imposed
    velocity, in the pool's step loop, against the reference's trajectory."""
    f = golden("traj_inlets_de1.npz")
    d, ops = _inlet_domain(f)
    assert d._device_loop_ok()
    z = f["init.elevation_c"]
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        h = np.maximum(d.quantities["stage"].centroid_values - z, 0.0)
        h_ref = np.maximum(f["stage"][i] - z, 0.0)
        assert np.abs(h - h_ref).max() <= DEPTH_TOL, (i, np.abs(h - h_ref).max())
    T = float(f["finaltime"])
    assert abs(ops[0].get_total_applied_volume() - 1.5 * T) <= 1e-9
    assert abs(ops[2].get_total_applied_volume() - 0.8 * T) <= 1e-9
    assert ops[1].get_total_applied_volume() < 0.0


def test_inlet_q_as_a_function_gives_the_step_loop_result(golden):
    f = golden("traj_inlets_de1.npz")
    out = []
    for callable_q in (False, True):
        d, ops = _inlet_domain(f, callable_q)
        for _ in d.evolve(yieldstep=1.0, finaltime=3.0):
            pass
        assert d._device_loop_ok() == (not callable_q)
        out.append((d.quantities["stage"].centroid_values.copy(), d.total_steps,
                    [op.get_total_applied_volume() for op in ops]))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][2] == out[1][2]


def test_rate_given_as_a_function_gives_the_step_loop_result():
    out = []
    for rate in (2.0e-4, lambda t: 2.0e-4):
        d = workloads.dam_break(m=20, flow_algorithm="DE1", precision="mixed")
        idx = np.arange(0, len(d), 3)
        op = agx.Rate_operator(d, rate=rate, indices=idx)
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        assert d._device_loop_ok() == (not callable(rate))
        out.append((d.quantities["stage"].centroid_values.copy(), d.total_steps, op.get_Q()))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][2] > 0 and abs(out[0][2] - out[1][2]) <= 1e-12 * out[0][2]


def test_rate_varying_in_time_matches_plain_within_1mm():
    """A rate that changes sign over the run (rain, then extraction) on the
    host-driven mixed step against the plain FP64 form."""
    res = {}
    for precision in ("fp64", "mixed"):
        d = workloads.dam_break(m=24, flow_algorithm="DE1", precision=precision)
        c = d.get_centroid_coordinates()
        idx = np.nonzero((c[:, 0] > 30) & (c[:, 0] < 70))[0]
        op = agx.Rate_operator(d, rate=lambda t: 3.0e-3 * np.cos(0.8 * t), indices=idx)
        for _ in d.evolve(yieldstep=1.0, finaltime=4.0):
            pass
        z = d.quantities["elevation"].centroid_values
        res[precision] = (np.maximum(d.quantities["stage"].centroid_values - z, 0.0), op.get_Q())
    err = np.abs(res["mixed"][0] - res["fp64"][0]).max()
    assert err <= DEPTH_TOL, err
    assert abs(res["mixed"][1] - res["fp64"][1]) <= 1e-3 * abs(res["fp64"][1]) + 1e-9


@pytest.mark.parametrize("alg", ["DE1", "DE2"])
def test_time_function_boundary_matches_plain_within_1mm(alg):
    """Time_boundary given as a function of time on the inflow edge: both
    forms evaluate it at the step's start for the first stage, at t + dt for
    the second and (rk3) at t + dt/2 for the third (the mixed form between
    agx_pool_step_begin, agx_pool_step_stage and agx_pool_step_end)."""
    res = {}
    for precision in ("fp64", "mixed"):
        d = workloads.dam_break(m=24, flow_algorithm=alg, precision=precision)
        Br = agx.Reflective_boundary(d)
        Bt = agx.Time_boundary(d, function=lambda t: [0.8 + 0.2 * np.sin(0.5 * t), 0.0, 0.0])
        d.set_boundary({"left": Bt, "right": Br, "top": Br, "bottom": Br})
        for _ in d.evolve(yieldstep=1.0, finaltime=4.0):
            pass
        assert not d._device_loop_ok()
        z = d.quantities["elevation"].centroid_values
        res[precision] = np.maximum(d.quantities["stage"].centroid_values - z, 0.0)
    err = np.abs(res["mixed"] - res["fp64"]).max()
    assert err <= DEPTH_TOL, err
