"""Failure detection with host-side injection (no device fault).

A NaN written into one cell's stage through the public API stands for a
state that has diverged.  The device checks every conserved value it
updates; the first non-finite one stops the scenario's step loop and the
host call raises AGX_E_NUMERIC with the count of bad cell updates.  In a
pool, the other scenarios run on and give bitwise the results they give
alone.  (The reference has no such check: a NaN cell fails its CFL speed
test, shallow_water/sw_domain_openmp.c:680-690, and spreads.)
"""
import numpy as np
import pytest

import anuga_core_gb300 as agx
from anuga_core_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_the_state_stops_the_step_loop(precision):
    d = workloads.dam_break(m=20, flow_algorithm="DE1", precision=precision)
    for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
        pass
    w = d.quantities["stage"].centroid_values.copy()
    w[137] = np.nan
    d.set_quantity("stage", w, location="centroids")
    with pytest.raises(agx._lib.AgxError) as ei:
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
    assert ei.value.code == -5 and "non-finite" in str(ei.value), str(ei.value)
    st = d._scn.stats() if precision == "fp64" else None
    if st is not None:
        assert st.nonfinite_cells > 0 and st.reason == agx._lib.STOP_ERROR
        assert st.total_steps <= 2 + d.total_steps    # stopped at the first step after the injection


def test_nan_in_the_state_per_phase_update_raises():
    d = workloads.dam_break(m=12, flow_algorithm="DE0")
    w = d.quantities["stage"].centroid_values.copy()
    w[5] = np.inf
    d.set_quantity("stage", w, location="centroids")
    d.distribute_to_vertices_and_edges()
    d.update_boundary()
    d.compute_fluxes()
    d.compute_forcing_terms()
    d.timestep = 0.5 * d.flux_timestep
    with pytest.raises(agx._lib.AgxError) as ei:
        d.update_conserved_quantities()
    assert ei.value.code == -5 and "non-finite" in str(ei.value)


def test_nan_in_one_pool_scenario_leaves_the_others_unaffected():
    from anuga_core_gb300.batch import Batch
    make = lambda m, alg: workloads.dam_break(m=m, flow_algorithm=alg, precision="mixed")
    specs = [(10, "DE1"), (14, "DE1"), (9, "DE0")]
    B = Batch([make(*s) for s in specs], distribute=True)
    w = B.get_centroids(1)["stage_c"]
    w[3] = np.nan
    B.pool.set_field(B.sids[1], "stage_c", w)
    for sid in B.sids:
        B.pool.set_clock(sid, 0.0, 1e300, -1.0, 40)
    B.pool.advance()
    with pytest.raises(agx._lib.AgxError) as ei:
        B.stats(1)
    assert "non-finite" in str(ei.value)
    for i in (0, 2):
        st = B.stats(i)
        assert st.total_steps == 40 and st.nonfinite_cells == 0
        alone = Batch([make(*specs[i])], distribute=True)
        alone.advance_steps(40)
        a, b = B.get_centroids(i), alone.get_centroids(0)
        for f in a:
            assert np.array_equal(a[f], b[f]), (i, f)
        alone.close()
    B.close()
