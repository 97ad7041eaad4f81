"""sww output formed on the device against the file the reference writes.

tests/golden/sww_inflow_de1.npz holds the variables of the .sww file the
reference's SWW_file.store_timestep wrote (file/sww.py:260-435) for the
inflow case, partly dry, with minimum_storable_height 0.05 m.  The plain
FP64 form must write the same file bit for bit: node means of the vertex
values in the reference's order, the storable-height mask at the nodes
(stage set to the bed, momenta to zero), centroid values as they are, all in
single precision.  The mixed form forms the same frame on the device from
its own state: bitwise the frame the host forms from its quantities, and
within 1 mm of the reference's stage.
"""
import numpy as np
import pytest

from anuga_core_gb300.mesh import rectangular_cross
from anuga_core_gb300.sww import read_sww
from helpers import make_domain

pytestmark = pytest.mark.gpu

KINDS = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
         "top": ("reflective", None), "bottom": ("reflective", None)}
VARS = ("time", "x", "y", "volumes", "elevation", "elevation_c", "elevation_range", "friction_c",
        "stage", "xmomentum", "ymomentum", "stage_c", "xmomentum_c", "ymomentum_c",
        "stage_range", "xmomentum_range", "ymomentum_range")


def _domain(f, precision, tmp_path, name):
    m = int(f["mesh.m"])
    p = f["mesh.points"]
    L = float(p[:, 0].max())
    p2, e, b = rectangular_cross(m, m, L, L)
    state = dict(stage=f["init.stage"], xmom=f["init.xmom"], ymom=f["init.ymom"],
                 elevation=f["init.elevation_c"], friction=f["init.friction"])
    d = make_domain(p2, e, b, "DE1", state, KINDS, precision=precision)
    d.set_quantity("elevation", f["init.elevation_v"], location="vertices")
    assert np.array_equal(d.quantities["elevation"].centroid_values, f["init.elevation_c"])
    d.set_quantity("stage", f["init.stage"], location="centroids")
    d.set_store(True)
    d.set_datadir(str(tmp_path))
    d.set_name(name)
    d.set_minimum_storable_height(float(f["minimum_storable_height"]))
    return d


def test_plain_sww_file_equals_the_reference_file(golden, tmp_path):
    f = golden("sww_inflow_de1.npz")
    d = _domain(f, "fp64", tmp_path, "plain")
    frames = 0
    for _ in d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"])):
        frames += 1
        v, c = d.writer._device_frame()
        hv, hc = d.writer.host_frame()
        assert np.array_equal(v, hv) and np.array_equal(c, hc)
    got = read_sww(str(tmp_path / "plain.sww"))
    for k in VARS:
        ref = f["sww." + k]
        assert got[k].shape == ref.shape, k
        assert np.array_equal(got[k].astype(ref.dtype.newbyteorder("=")), ref), k
    masked = (f["sww.stage"] == f["sww.elevation"][None, :])
    assert masked.any() and (f["sww.xmomentum"][masked] == 0).all()
    assert frames == f["sww.time"].size


def test_mixed_sww_frames_from_the_device(golden, tmp_path):
    f = golden("sww_inflow_de1.npz")
    d = _domain(f, "mixed", tmp_path, "mixed")
    for i, _ in enumerate(d.evolve(yieldstep=float(f["yieldstep"]), finaltime=float(f["finaltime"]))):
        v, c = d.writer._device_frame()
        hv, hc = d.writer.host_frame()
        assert np.array_equal(v, hv) and np.array_equal(c, hc), i
    got = read_sww(str(tmp_path / "mixed.sww"))
    assert got["stage"].shape == f["sww.stage"].shape
    assert np.array_equal(got["time"], f["sww.time"])
    assert np.abs(got["stage"] - f["sww.stage"]).max() <= 1.0e-3
    assert np.abs(got["stage_c"] - f["sww.stage_c"]).max() <= 1.0e-3


def test_frames_are_written_while_the_next_yieldstep_runs(tmp_path):
    """The frame's copy and the file append run beside the next yieldstep;
    the file is complete when evolve returns, and the same as with
    synchronous writing."""
    from anuga_core_gb300 import workloads
    out = []
    for asynchronous in (True, False):
        d = workloads.dam_break(m=20, flow_algorithm="DE1")
        d.set_store(True)
        d.set_datadir(str(tmp_path))
        d.set_name("dam_%d" % asynchronous)
        d.set_minimum_storable_height(0.05)
        for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
            pass                                   # the writer object exists from the first yield
        d.writer.asynchronous = asynchronous
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        out.append(read_sww(str(tmp_path / ("dam_%d.sww" % asynchronous))))
    for k in ("stage", "xmomentum", "stage_c", "time"):
        assert np.array_equal(out[0][k], out[1][k]), k
    assert out[0]["stage"].shape[0] == 5
