"""update_timestep options against trajectories the reference wrote:
set_fixed_flux_timestep (generic_domain.py:2332-2359; device step loop and
host-driven steps) and the protection against isolated degenerate timesteps
(generic_domain.py:2520-2560; host-driven steps of the plain form)."""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300.mesh import rectangular_cross
from helpers import make_domain, normwise

pytestmark = pytest.mark.gpu

INFLOW = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
          "top": ("reflective", None), "bottom": ("reflective", None)}
WALLS = {t: ("reflective", None) for t in ("left", "right", "top", "bottom")}


def _domain(f, alg, kinds, precision="fp64"):
    m = int(f["mesh.m"])
    p = f["mesh.points"]
    L = float(p[:, 0].max())
    p2, e, b = rectangular_cross(m, m, L, L)
    assert np.array_equal(p2, p)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    return make_domain(p2, e, b, alg, state, kinds, precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fixed_flux_timestep_matches_reference(golden, precision):
    f = golden("traj_inflow_fixed_dt_de1.npz")
    d = _domain(f, "DE1", INFLOW, precision)
    d.set_fixed_flux_timestep(float(f["fixed_flux_timestep"]))
    z = f["init.elevation_c"]
    steps = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        steps.append(d.number_of_steps)
        w = d.quantities["stage"].centroid_values
        if precision == "fp64":
            assert normwise(w, f["stage"][i]) <= 1e-12, i
            assert normwise(d.quantities["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
        else:
            assert np.abs(np.maximum(w - z, 0) - np.maximum(f["stage"][i] - z, 0)).max() <= 1.0e-3, i
    assert steps == list(f["steps"])          # fixed steps: the same count in both forms
    assert d.flux_timestep == float(f["fixed_flux_timestep"])


def test_fixed_flux_timestep_host_steps_equal_device_loop(golden):
    f = golden("traj_inflow_fixed_dt_de1.npz")
    out = []
    for host in (False, True):
        d = _domain(f, "DE1", INFLOW)
        d.set_fixed_flux_timestep(0.4)
        if host:
            d.set_boundary({"left": agx.Time_boundary(d, function=lambda t: [2.0, 0.0, 0.0])})
        for _ in d.evolve(yieldstep=10.0, finaltime=20.0):
            pass
        assert d._device_loop_ok() == (not host)
        out.append((d.total_steps, d.quantities["stage"].centroid_values.copy()))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    d.set_fixed_flux_timestep(None)           # variable timestepping again
    assert d.fixed_flux_timestep is None
    with pytest.raises(Exception):
        d.set_fixed_flux_timestep(-1.0)


def test_isolated_degenerate_timestep_protection_matches_reference(golden):
    f = golden("traj_isolated_fast_cell_de0.npz")
    assert int(f["degenerate_zeroed"]) > 0        # the reference's protection acted on this run
    d = _domain(f, "DE0", WALLS)
    d.protect_against_isolated_degenerate_timesteps = True
    assert not d._device_loop_ok()
    steps = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        steps.append(d.number_of_steps)
        assert normwise(d.quantities["stage"].centroid_values, f["stage"][i]) <= 1e-12, i
        assert normwise(d.quantities["xmomentum"].centroid_values, f["xmom"][i]) <= 1e-10, i
    assert steps == list(f["steps"])
    # without the protection the run differs
    d2 = _domain(f, "DE0", WALLS)
    for _ in d2.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"])):
        pass
    assert not np.allclose(d2.quantities["xmomentum"].centroid_values, f["xmom"][-1], rtol=0, atol=1e-6)
