"""The multiprocessor-mode adapter (anuga_core_gb300.plugin.AGX_interface)
driven phase by phase the way the reference's Domain drives its
gpu_interface in mode 4 (shallow_water_domain.py:1872, 1912, 2037, 2146;
friction.py:125-147), on the reference's own per-phase fixtures: every
phase output equal to what the reference wrote (bit for bit; Manning's
semi-implicit terms and the update within the pow tolerance)."""
import numpy as np
import pytest

from anuga_core_gb300.mesh import rectangular_cross
from anuga_core_gb300.plugin import AGX_interface
from helpers import make_domain, normwise

pytestmark = pytest.mark.gpu
POW_TOL = 1e-14


@pytest.mark.parametrize("alg", ["de0", "de1"])
def test_adapter_phases_match_reference(golden, alg):
    f = golden("phases_%s.npz" % alg)
    m, n, L1, L2 = f["params"]
    p, e, b = rectangular_cross(int(m), int(n), L1, L2)
    state = dict(stage=f["in.stage.centroid_values"], xmom=f["in.xmomentum.centroid_values"],
                 ymom=f["in.ymomentum.centroid_values"], elevation=f["in.elevation.centroid_values"],
                 friction=f["in.friction.centroid_values"])
    kinds = {"left": ("dirichlet", (1.3, 0.05, -0.02)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    d = make_domain(p, e, b, alg.upper(), state, kinds)
    assert d._scn is None                      # the domain's own arrays are the storage here
    gpu = AGX_interface(d)
    Q = d.quantities
    gpu.protect_against_infinitesimal_and_negative_heights_kernal(d)
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(Q[q].centroid_values, f["protect.%s.centroid_values" % q]), q
    gpu.extrapolate_second_order_edge_sw_kernel(d)
    for q in ("stage", "xmomentum", "ymomentum", "elevation", "height"):
        assert np.array_equal(Q[q].edge_values, f["extrap.%s.edge_values" % q]), q
        assert np.array_equal(Q[q].vertex_values, f["extrap.%s.vertex_values" % q]), q
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(Q[q].centroid_values, f["extrap.%s.centroid_values" % q]), q
    for q in ("stage", "xmomentum", "ymomentum"):          # the host's boundary objects' values
        Q[q].boundary_values[:] = f["bc.%s.boundary_values" % q]
    d.boundary_flux_sum = np.zeros(3)
    dt = gpu.compute_fluxes_ext_central_kernel(d, d.evolve_max_timestep)
    assert dt == float(f["flux.flux_timestep"])
    assert np.array_equal(d.max_speed, f["flux.max_speed"])
    for q in ("stage", "xmomentum", "ymomentum"):
        assert np.array_equal(Q[q].explicit_update, f["flux.%s.explicit_update" % q]), q
    ref_bfs = float(f["flux.boundary_flux_sum"][0])
    assert abs(d.boundary_flux_sum[0] - ref_bfs) <= 1e-12 * max(1.0, abs(ref_bfs))
    for q in ("xmomentum", "ymomentum"):
        Q[q].semi_implicit_update[:] = 0.0
    gpu.compute_forcing_terms_manning_friction_flat()
    for q in ("xmomentum", "ymomentum"):
        assert normwise(Q[q].semi_implicit_update, f["forcing.%s.semi_implicit_update" % q]) <= POW_TOL, q
    d.timestep = float(f["update.timestep"])
    gpu.update_conserved_quantities_kernal(d)
    for q in ("stage", "xmomentum", "ymomentum"):
        assert normwise(Q[q].centroid_values, f["update.%s.centroid_values" % q]) <= POW_TOL, q
    gpu.close()
