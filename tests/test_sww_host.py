"""SWW file layout (no GPU): the writer's dimensions, variables and the
storable-height mask of a frame formed on the host."""
import numpy as np

from anuga_core_gb300 import workloads
from anuga_core_gb300.sww import SWW_file, read_sww


def test_sww_layout_and_host_frame(tmp_path):
    d = workloads.dam_break(m=6)
    d.set_datadir(str(tmp_path))
    d.set_name("layout")
    d.set_minimum_storable_height(0.5)
    w = SWW_file(d)
    w.store_connectivity()
    w.store_timestep()
    w.store_timestep()
    f = read_sww(str(tmp_path / "layout.sww"))
    P, N = d.mesh.number_of_nodes, len(d)
    assert f["x"].shape == (P,) and f["volumes"].shape == (N, 3)
    for q in ("stage", "xmomentum", "ymomentum"):
        assert f[q].shape == (2, P) and f[q].dtype.itemsize == 4 and f[q + "_c"].shape == (2, N)
    assert f["time"].shape == (2,)
    zc = d.quantities["elevation"].centroid_values
    h = d.quantities["stage"].centroid_values - zc
    masked = h < 0.5
    assert masked.any() and (~masked).any()
    assert np.array_equal(f["stage_c"][0][masked], zc[masked].astype(np.float32))
    v, c = w.host_frame()
    assert np.array_equal(f["stage"][1], v[0]) and np.array_equal(f["stage_c"][1], c[0])
