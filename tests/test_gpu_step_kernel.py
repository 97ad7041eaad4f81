"""The one-kernel step of the mixed pool (a cooperative launch whose grid
barriers separate the stage-1 fluxes, the first update, the stage-2 fluxes,
the rates and the clocks) against the separate kernels of the step graph:
the same scenarios advanced both ways give bitwise the same states, times
and step counts."""
import numpy as np
import pytest

from anuga_core_gb300 import workloads
from anuga_core_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _batch(variant, grid_mode):
    doms = [workloads.batch_scenario(m, 42 * 1000 + i, "dam" if i % 2 == 0 else "inflow")
            for i, m in enumerate((12, 30, 7, 45, 20, 64))]
    doms.append(workloads.dam_break(m=16, flow_algorithm="DE0", precision="mixed"))   # one stage per step
    rain = workloads.dam_break(m=14, flow_algorithm="DE1", precision="mixed")
    from anuga_core_gb300 import Rate_operator
    Rate_operator(rain, rate=3.0e-4, indices=np.arange(0, len(rain), 3))
    doms.append(rain)
    B = Batch(doms, distribute=True)
    B.pool.set_variant(variant, grid_mode)
    return B


@pytest.mark.parametrize("variant", [0, 1])
def test_one_kernel_step_equals_the_step_graph(variant):
    out = []
    for grid_mode in (0, 2):
        B = _batch(variant, grid_mode)
        B.advance_steps(7)
        B.advance_to([st.time + 1.5 for st in (B.stats(i) for i in range(len(B.sids)))])
        out.append(([B.get_centroids(i) for i in range(len(B.sids))],
                    [(B.stats(i).time, B.stats(i).total_steps, B.stats(i).boundary_flux_integral)
                     for i in range(len(B.sids))],
                    B.pool.operator_influx(B.sids[-1], 0)))
        B.close()
    (a, sa, qa), (b, sb, qb) = out
    for i, (x, y) in enumerate(zip(a, b)):
        for f in x:
            assert np.array_equal(x[f], y[f]), (i, f)
    for (t1, n1, f1), (t2, n2, f2) in zip(sa, sb):
        assert t1 == t2 and n1 == n2
        assert abs(f1 - f2) <= 1e-12 * max(abs(f1), 1.0)
    assert qa > 0 and abs(qa - qb) <= 1e-12 * qa        # the influx sums run in another order
