"""agx_compute_fluxes_noalloc (include/agx_noalloc.h) against
agx_compute_fluxes on the same state, through the C ABI.

The no-allocation entry point reads caller-owned device arrays and keeps its
scratch in a fixed device array of the library.  Bars: explicit updates, max
speeds and the flux timestep bit-identical to agx_compute_fluxes on two calls
in a row; the boundary flux sum (added with atomics, order-dependent in the
last place) within 1e-12 relative.  Sizes above AGX_NOALLOC_MAX_CELLS are
rejected before any device work.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from anuga_core_gb300.mesh import Mesh, rectangular_cross
from helpers import make_domain, random_state

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "agx_noalloc.h")


def _max_cells():
    m = re.search(r"#define\s+AGX_NOALLOC_MAX_CELLS\s+(\d+)", open(HEADER).read())
    return int(m.group(1))


_PTRS = ["conn", "edge_slot", "edge_opp", "normals", "edgelengths", "radii", "inv_area",
         "stage_e", "xmom_e", "ymom_e", "elev_e", "height_e", "stage_b", "xmom_b", "ymom_b",
         "stage_c", "height_c", "elev_c", "stage_x", "xmom_x", "ymom_x", "max_speed"]


class FluxBuffers(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int64), ("B", ctypes.c_int64), ("E", ctypes.c_int64)] + \
               [(n, ctypes.c_void_p) for n in _PTRS]


def _bind(L):
    from anuga_core_gb300 import _lib
    f = L.agx_compute_fluxes_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.POINTER(_lib.Params), ctypes.POINTER(FluxBuffers), ctypes.c_int32, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, ctypes.c_int32]
    return f


def test_size_above_the_scratch_limit_is_rejected():
    """Rejected on the host, before any CUDA call, with a message naming the limit."""
    from anuga_core_gb300 import _lib
    try:
        L = _lib.load()
    except Exception as e:          # library not built in this environment
        pytest.skip("libagx.so not loadable: %s" % e)
    f = _bind(L)
    buf = FluxBuffers()
    buf.N = _max_cells() + 1
    buf.E = 3 * buf.N
    err = ctypes.create_string_buffer(512)
    p = _lib.Params()
    dt = ctypes.c_double(-1.0)
    rc = f(ctypes.byref(p), ctypes.byref(buf), 0, None, ctypes.byref(dt), None, err, 512)
    assert rc == -1                 # AGX_E_INVALID
    assert b"AGX_NOALLOC_MAX_CELLS" in err.value
    assert dt.value == -1.0


def _case(m, n, seed, alg):
    p, e, b = rectangular_cross(m, n, 3.0 * m, 3.0 * n)
    mesh = Mesh(p, e, b)
    st = random_state(mesh, seed)
    kinds = {"left": ("dirichlet", (float(np.max(st["stage"])) + 0.2, 0.1, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    d = make_domain(p, e, b, alg, st, kinds)
    d.distribute_to_vertices_and_edges()
    d.update_boundary()
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,seed,alg", [(40, 30, 11, "DE1"), (20, 25, 12, "DE0")])
def test_noalloc_fluxes_equal_compute_fluxes(m, n, seed, alg):
    import torch
    from anuga_core_gb300 import _lib
    d = _case(m, n, seed, alg)
    scn = d._scn
    T = d._tables
    N, B = scn.N, scn.B
    assert N <= _max_cells()
    dev = torch.device("cuda", 0)

    # the existing entry point, on the scenario's own arrays
    want = {}
    for substep in (0, 1):
        dt_ref = scn.compute_fluxes(substep)
        want[substep] = dict(dt=dt_ref, bfs=scn.stats().boundary_flux_sum[substep],
                             x=[scn.get(f).copy() for f in ("stage_x", "xmom_x", "ymom_x")])
        if substep == 0:
            want[0]["max_speed"] = scn.get("max_speed").copy()

    # caller-owned device arrays: the tables and the outputs
    tab = {k: torch.from_numpy(np.ascontiguousarray(T[k])).to(dev)
           for k in ("conn", "edge_slot", "edge_opp", "normals", "edgelengths", "radii", "inv_area")}
    out = {k: torch.full((N,), float("nan"), dtype=torch.float64, device=dev)
           for k in ("stage_x", "xmom_x", "ymom_x", "max_speed")}
    buf = FluxBuffers()
    buf.N, buf.B, buf.E = N, B, int(T["edge_slot"].shape[0])
    for k, t in tab.items():
        setattr(buf, k, t.data_ptr())
    for k, t in out.items():
        setattr(buf, k, t.data_ptr())
    for k in ("stage_e", "xmom_e", "ymom_e", "elev_e", "height_e", "stage_b", "xmom_b", "ymom_b",
              "stage_c", "height_c", "elev_c"):
        setattr(buf, k, scn.device_ptr(k)[0])
    torch.cuda.synchronize()

    f = _bind(_lib.load())
    params = d._params()
    stream = torch.cuda.current_stream().cuda_stream
    err = ctypes.create_string_buffer(512)
    for substep in (0, 1):
        for call in range(2):                       # two calls in a row
            dt = ctypes.c_double()
            bfs = ctypes.c_double()
            rc = f(ctypes.byref(params), ctypes.byref(buf), substep, ctypes.c_void_p(stream), ctypes.byref(dt),
                   ctypes.byref(bfs), err, 512)
            assert rc == 0, err.value
            w = want[substep]
            assert dt.value == w["dt"], (substep, call)
            for k, ref in zip(("stage_x", "xmom_x", "ymom_x"), w["x"]):
                assert np.array_equal(out[k].cpu().numpy(), ref), (k, substep, call)
            if substep == 0:
                assert np.array_equal(out["max_speed"].cpu().numpy(), w["max_speed"]), call
            assert abs(bfs.value - w["bfs"]) <= 1e-12 * max(abs(w["bfs"]), 1e-300), (bfs.value, w["bfs"])


@pytest.mark.gpu
def test_noalloc_rejects_bad_edge_lists_and_recovers():
    """An edge slot out of range, and an edge list that leaves slots
    unwritten, are reported as AGX_E_INVALID (every load stays inside the
    caller's arrays: the kernels check each index before using it); a valid
    call with the same buffers right after gives the parity results."""
    import torch
    from anuga_core_gb300 import _lib
    d = _case(20, 25, 12, "DE0")
    scn = d._scn
    T = d._tables
    N, B = scn.N, scn.B
    dt_ref = scn.compute_fluxes(0)
    x_ref = scn.get("stage_x").copy()
    dev = torch.device("cuda", 0)
    tab = {k: torch.from_numpy(np.ascontiguousarray(T[k])).to(dev)
           for k in ("conn", "edge_slot", "edge_opp", "normals", "edgelengths", "radii", "inv_area")}
    out = {k: torch.zeros((N,), dtype=torch.float64, device=dev) for k in ("stage_x", "xmom_x", "ymom_x", "max_speed")}
    E = int(T["edge_slot"].shape[0])

    def buffers(edge_slot, n_edges):
        buf = FluxBuffers()
        buf.N, buf.B, buf.E = N, B, n_edges
        for k, t in tab.items():
            setattr(buf, k, t.data_ptr())
        buf.edge_slot = edge_slot.data_ptr()
        for k, t in out.items():
            setattr(buf, k, t.data_ptr())
        for k in ("stage_e", "xmom_e", "ymom_e", "elev_e", "height_e", "stage_b", "xmom_b", "ymom_b",
                  "stage_c", "height_c", "elev_c"):
            setattr(buf, k, scn.device_ptr(k)[0])
        return buf

    bad = tab["edge_slot"].clone()
    bad[E // 2] = 3 * N                              # one slot index past the last slot
    torch.cuda.synchronize()
    f = _bind(_lib.load())
    params = d._params()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    err = ctypes.create_string_buffer(512)
    dt = ctypes.c_double()
    rc = f(ctypes.byref(params), ctypes.byref(buffers(bad, E)), 0, stream, ctypes.byref(dt), None, err, 512)
    assert rc == -1 and b"out of range" in err.value, (rc, err.value)
    rc = f(ctypes.byref(params), ctypes.byref(buffers(tab["edge_slot"], E - 1)), 0, stream, ctypes.byref(dt), None,
           err, 512)                                 # the last edge left out: its slots are not written
    assert rc == -1 and b"slot results" in err.value, (rc, err.value)
    for _ in range(2):
        rc = f(ctypes.byref(params), ctypes.byref(buffers(tab["edge_slot"], E)), 0, stream, ctypes.byref(dt), None,
               err, 512)
        assert rc == 0, err.value
        assert dt.value == dt_ref
        assert np.array_equal(out["stage_x"].cpu().numpy(), x_ref)
