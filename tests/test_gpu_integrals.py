"""Boundary flux integral, volume bookkeeping and the mixed form's FP64 timestep.

The boundary flux integral (operators/boundary_flux_integral_operator.py,
shallow_water_domain.py:1677-1745, 2749-2781) is checked against values the
reference wrote on the inflow case for one-, two- and three-stage time
stepping (tests/golden/bfi_*.npz).  Plain FP64: within 1e-9 of the largest
integral (the device sums each stage's boundary fluxes in another order);
mixed: within 2e-3 relative, with the volume balance V - BF - FS held to
1e-5 of the volume.
"""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300 import workloads
from anuga_core_gb300.mesh import rectangular_cross
from helpers import make_domain

pytestmark = pytest.mark.gpu

KINDS = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
         "top": ("reflective", None), "bottom": ("reflective", None)}
CASES = [("bfi_inflow_de0.npz", "DE0"), ("bfi_inflow_de1_rain.npz", "DE1"), ("bfi_inflow_de2.npz", "DE2")]


def _domain(f, alg, precision):
    m = int(f["mesh.m"])
    p = f["mesh.points"]
    L = float(p[:, 0].max())
    p2, e, b = rectangular_cross(m, m, L, L)
    assert np.array_equal(p2, p)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    rates = [(f["rain.indices"], float(f["rain.rate"]))] if "rain.rate" in f else []
    return make_domain(p2, e, b, alg, state, KINDS, precision=precision, rates=rates)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name,alg", CASES)
def test_boundary_flux_integral_matches_reference(golden, name, alg, precision):
    f = golden(name)
    d = _domain(f, alg, precision)
    ref_bf = f["boundary_flux_integral"]
    scale = float(np.abs(ref_bf).max())
    assert scale > 1000.0                       # water enters and leaves through the boundaries
    area = float(np.sum(d.mesh.areas))
    got = []
    for i, t in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        V, BF, FS = d.report_water_volume_statistics(verbose=False, returnStats=True) if i else \
            (d.get_water_volume(), d.get_boundary_flux_integral(), d.get_fractional_step_volume_integral())
        got.append((V, BF, FS))
        if precision == "fp64":
            assert abs(BF - ref_bf[i]) <= 1e-9 * scale, (i, BF, ref_bf[i])
            assert abs(FS - f["fractional_step_volume"][i]) <= 1e-9 * max(f["fractional_step_volume"][i], 1.0)
            assert abs(V - f["volume"][i]) <= 1e-12 * f["volume"][i], (i, V, f["volume"][i])
        else:
            assert abs(BF - ref_bf[i]) <= 2e-3 * scale, (i, BF, ref_bf[i])
            assert abs(FS - f["fractional_step_volume"][i]) <= 1e-6 * max(f["fractional_step_volume"][i], 1.0)
            assert abs(V - f["volume"][i]) <= 1e-3 * area, (i, V, f["volume"][i])
    # volume balance: V - BF - FS stays the initial volume
    bal = np.array([v - bf - fs for v, bf, fs in got])
    tol = 1e-10 if precision == "fp64" else 1e-5
    assert np.abs(bal - bal[0]).max() <= tol * got[0][0], bal - bal[0]


def test_boundary_flux_integral_host_steps_equal_device_loop():
    """The same Dirichlet values given as a Time_boundary function (steps
    driven by the host phase by phase, integrated by the operator on the
    host) and as a Dirichlet_boundary (device step loop, integrated by the
    device clock): bitwise the same integral."""
    out = []
    for host in (False, True):
        d = workloads.dam_break(m=16, flow_algorithm="DE1")
        Br = agx.Reflective_boundary(d)
        left = agx.Time_boundary(d, function=lambda t: [1.2, 0.0, 0.0]) if host else agx.Dirichlet_boundary([1.2, 0.0, 0.0])
        d.set_boundary({"left": left, "right": Br, "top": Br, "bottom": Br})
        for _ in d.evolve(yieldstep=1.0, finaltime=3.0):
            pass
        assert d._device_loop_ok() == (not host)
        out.append((d.get_boundary_flux_integral(), d.total_steps, d.quantities["stage"].centroid_values.copy()))
    assert out[0][1] == out[1][1] and np.array_equal(out[0][2], out[1][2])
    assert out[0][0] == out[1][0] and out[0][0] > 0.0


def test_boundary_flux_integral_survives_device_rebuild_and_checkpoint(tmp_path):
    import pickle
    d = workloads.dam_break(m=12, flow_algorithm="DE1")
    Br = agx.Reflective_boundary(d)
    d.set_boundary({"left": agx.Dirichlet_boundary([1.2, 0.0, 0.0]), "right": Br, "top": Br, "bottom": Br})
    for _ in d.evolve(yieldstep=1.0, finaltime=1.0):
        pass
    a = d.get_boundary_flux_integral()
    d.set_CFL(d.CFL)                              # destroys and rebuilds the device scenario
    assert d.get_boundary_flux_integral() == a
    d2 = pickle.loads(pickle.dumps(d))
    assert d2.get_boundary_flux_integral() == a
    for _ in d.evolve(yieldstep=1.0, finaltime=2.0):
        pass
    assert d.get_boundary_flux_integral() > a


def test_mixed_timestep_is_an_fp64_quotient():
    """The mixed form's flux timestep is radius / speed in FP64 for the cell
    with the smallest FP32 quotient: equal to r_c / s_c (FP64 radius, the
    stored FP32 speed) for some cell c, within FP32 rounding of the minimum
    over all cells, and within the FP32 speed error of the plain form's."""
    out = {}
    for prec in ("fp64", "mixed"):
        d = workloads.inflow_bumps(m=60, L=600.0, precision=prec)
        d.distribute_to_vertices_and_edges()
        d.advance_steps(40)
        out[prec] = d
    dm, dp = out["mixed"], out["fp64"]
    st = dm.advance_steps(1)
    r = dm.mesh.radii
    s = dm.max_speed
    ok = s > 0
    q = np.full(len(r), np.inf)
    q[ok] = r[ok] / s[ok]
    assert np.any(q == st.flux_timestep)                      # an exact FP64 quotient of one cell
    assert abs(st.flux_timestep - q.min()) <= 2e-7 * q.min()  # the FP32 selection of the minimum
    # the same state in the plain form gives the timestep to the FP32 speed error
    w, uh, vh = dm.get_conserved_state()
    dp.set_conserved_state(w, uh, vh)
    dp.distribute_to_vertices_and_edges()
    dp.update_boundary()
    dp.compute_fluxes()
    assert abs(dp.flux_timestep - st.flux_timestep) <= 1e-4 * dp.flux_timestep
    # the clock advances by the FP64 timestep it applies
    t0 = st.time
    st2 = dm.advance_steps(1)
    assert st2.time == t0 + st2.last_timestep
