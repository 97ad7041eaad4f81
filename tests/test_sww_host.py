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
    # the mask is taken at the nodes (file/sww.py:380-400): where the node's
    # mean stage minus its mean bed is below minimum_storable_height, the
    # stage stored is the bed and the momenta are zero; centroid values are
    # stored as they are.  The DE algorithms average centroid values to nodes.
    assert d.get_using_centroid_averaging()
    zn = w._smooth(None, d.quantities["elevation"].centroid_values)
    wn = w._smooth(None, d.quantities["stage"].centroid_values)
    masked = wn - zn < 0.5
    assert masked.any() and (~masked).any()
    assert np.array_equal(f["stage"][0][masked], zn[masked].astype(np.float32))
    assert np.array_equal(f["stage"][0][~masked], wn[~masked].astype(np.float32))
    assert (f["xmomentum"][0][masked] == 0).all()
    assert np.array_equal(f["stage_c"][0], d.quantities["stage"].centroid_values.astype(np.float32))
    v, c = w.host_frame()
    assert np.array_equal(f["stage"][1], v[0]) and np.array_equal(f["stage_c"][1], c[0])


def test_node_means_follow_the_reference_summation_order():
    """Node means add each node's vertex values (or the centroid values of
    its triangles) one at a time in the order of the mesh's
    vertex_value_indices and divide by the count (quantity.c:823-915)."""
    d = workloads.dam_break(m=5)
    w = SWW_file(d)
    rng = np.random.default_rng(3)
    vv = rng.normal(size=(len(d), 3)) * 1e3
    got = w._smooth(vv)
    flat = vv.ravel()
    vvi = np.argsort(d.mesh.triangles.ravel())
    counts = np.bincount(d.mesh.triangles.ravel(), minlength=d.mesh.number_of_nodes)
    want = np.zeros(d.mesh.number_of_nodes)
    q = 0
    for p in range(d.mesh.number_of_nodes):
        total = 0.0
        for _ in range(counts[p]):
            total += flat[vvi[q]]
            q += 1
        want[p] = total / counts[p]
    assert np.array_equal(got, want)
    cv = rng.normal(size=len(d)) * 1e3
    got_c = w._smooth(None, cv)
    q = 0
    for p in range(d.mesh.number_of_nodes):
        total = 0.0
        for _ in range(counts[p]):
            total += cv[vvi[q] // 3]
            q += 1
        want[p] = total / counts[p]
    assert np.array_equal(got_c, want)
