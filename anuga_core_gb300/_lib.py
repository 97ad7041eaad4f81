"""ctypes binding of libagx.so (declarations in include/agx.h).

The library is the only compute path: if it is missing, or no CUDA device is
visible, importing the device layer raises instead of falling back to a CPU
implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)

AGX_PREC_FP64 = 0
AGX_PREC_MIXED = 1

FIELDS = ["stage_c", "xmom_c", "ymom_c", "elev_c", "friction_c", "height_c",
          "stage_e", "xmom_e", "ymom_e", "elev_e", "height_e",
          "stage_v", "xmom_v", "ymom_v", "elev_v", "height_v",
          "stage_b", "xmom_b", "ymom_b",
          "stage_x", "xmom_x", "ymom_x",
          "stage_s", "xmom_s", "ymom_s",
          "max_speed"]
FIELD = {n: i for i, n in enumerate(FIELDS)}

(BC_NONE, BC_REFLECTIVE, BC_TRANSMISSIVE, BC_TRANSMISSIVE_C, BC_DIRICHLET, BC_TIME_SERIES, BC_TRANSMISSIVE_N0,
 BC_TRANSMISSIVE_SET_STAGE, BC_TRANSMISSIVE_ZERO_MOM, BC_FLATHER, BC_CHARACTERISTIC, BC_INFLOW) = range(12)
STOP_YIELD, STOP_FINAL, STOP_MAXSTEPS, STOP_ERROR = 1, 2, 3, 4
PHASES = ("prep", "extrap", "bc", "flux", "accum", "update", "rate", "small")
PHASE_COUNT = len(PHASES)


class MeshDesc(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int64), ("n_boundary", ctypes.c_int64), ("n_edges", ctypes.c_int64),
                ("conn", _i32p), ("surr", _i32p), ("geo", _f64p), ("edge_slot", _i32p),
                ("edge_opp", _i32p), ("normals", _f64p), ("edgelengths", _f64p), ("radii", _f64p),
                ("areas", _f64p), ("inv_area", _f64p), ("boundary_slot", _i32p),
                ("vertex_coordinates", _f64p)]


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("g", "epsilon", "minimum_allowed_height", "beta_w", "beta_w_dry", "beta_uh",
                 "beta_uh_dry", "beta_vh", "beta_vh_dry", "CFL", "evolve_max_timestep",
                 "evolve_min_timestep")] + \
               [(n, ctypes.c_int32) for n in
                ("extrapolate_velocity_second_order", "low_froude", "timestepping_method",
                 "protect_zero_ymom", "use_sloped_mannings", "max_smallsteps", "precision", "reserved")]


class StepStats(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("last_timestep", ctypes.c_double),
                ("min_timestep", ctypes.c_double), ("max_timestep", ctypes.c_double),
                ("flux_timestep", ctypes.c_double), ("mass_added", ctypes.c_double),
                ("boundary_flux_sum", ctypes.c_double * 3), ("steps", ctypes.c_int64),
                ("total_steps", ctypes.c_int64), ("negative_cells", ctypes.c_int64),
                ("reason", ctypes.c_int32), ("order", ctypes.c_int32),
                ("boundary_flux_integral", ctypes.c_double), ("nonfinite_cells", ctypes.c_int64)]


class AgxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("agx error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load(path=None):
    """Load libagx.so (building it first if its sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if _build.needs_build():
        _build.build()
    if not os.path.exists(path):
        raise ImportError("libagx.so not built: run python -c 'import __graft_entry__ as g; g.build()'")
    L = ctypes.CDLL(path)
    H = ctypes.c_void_p
    P = ctypes.POINTER
    sig = {
        "agx_scenario_create": ([P(MeshDesc), P(Params), P(H)], ctypes.c_int32),
        "agx_scenario_destroy": ([H], ctypes.c_int32),
        "agx_scenario_footprint": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32], ctypes.c_int64),
        "agx_set_field": ([H, ctypes.c_int32, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_get_field": ([H, ctypes.c_int32, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_device_ptr": ([H, ctypes.c_int32, P(ctypes.c_void_p), P(ctypes.c_int64)], ctypes.c_int32),
        "agx_set_state": ([H, _f64p, _f64p, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_sww_bind": ([H, ctypes.c_int64, _i32p, _i32p], ctypes.c_int32),
        "agx_sww_frame": ([H, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_float),
                           ctypes.POINTER(ctypes.c_float)], ctypes.c_int32),
        "agx_sww_frame_async": ([H, ctypes.c_double, ctypes.c_int32], ctypes.c_int32),
        "agx_sww_frame_wait": ([H, P(ctypes.POINTER(ctypes.c_float)), P(ctypes.POINTER(ctypes.c_float))],
                               ctypes.c_int32),
        "agx_get_state": ([H, _f64p, _f64p, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_set_boundary": ([H, _i32p, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_set_boundary_series": ([H, _f64p, ctypes.c_int64], ctypes.c_int32),
        "agx_add_rate_operator": ([H, _i32p, ctypes.c_int64, ctypes.c_double, ctypes.c_double], ctypes.c_int32),
        "agx_clear_operators": ([H], ctypes.c_int32),
        "agx_apply_operator": ([H, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double], ctypes.c_int32),
        "agx_add_inlet_operator": ([H, _i32p, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                    ctypes.c_double, ctypes.c_double], ctypes.c_int32),
        "agx_operator_influx": ([H, ctypes.c_int32, _f64p], ctypes.c_int32),
        "agx_protect": ([H, _f64p], ctypes.c_int32),
        "agx_distribute": ([H, ctypes.c_int32], ctypes.c_int32),
        "agx_update_boundary": ([H, ctypes.c_double], ctypes.c_int32),
        "agx_compute_fluxes": ([H, ctypes.c_int32, _f64p], ctypes.c_int32),
        "agx_compute_forcing": ([H], ctypes.c_int32),
        "agx_update_conserved": ([H, ctypes.c_double, P(ctypes.c_int64)], ctypes.c_int32),
        "agx_backup": ([H], ctypes.c_int32),
        "agx_saxpy": ([H, ctypes.c_double, ctypes.c_double], ctypes.c_int32),
        "agx_divide_conserved": ([H, ctypes.c_double], ctypes.c_int32),
        "agx_set_riverwalls": ([H, _i32p, ctypes.c_int64, ctypes.c_int64, _f64p, _i32p, ctypes.c_int32,
                                ctypes.c_int32, _f64p], ctypes.c_int32),
        "agx_set_clock": ([H, ctypes.c_double, ctypes.c_double, ctypes.c_double], ctypes.c_int32),
        "agx_set_fixed_flux_timestep": ([H, ctypes.c_double], ctypes.c_int32),
        "agx_advance": ([H, ctypes.c_int64, P(StepStats)], ctypes.c_int32),
        "agx_get_stats": ([H, P(StepStats)], ctypes.c_int32),
        "agx_set_stream": ([H, ctypes.c_void_p], ctypes.c_int32),
        "agx_time_phases": ([H, ctypes.c_int32, _f64p, ctypes.c_int32], ctypes.c_int32),
        "agx_last_error": ([ctypes.c_char_p, ctypes.c_int32], ctypes.c_int32),
        "agx_version": ([], ctypes.c_int32),
        "agx_kernel_launches": ([], ctypes.c_int64),
        "agx_fp64_throughput": ([_f64p, _f64p, _f64p], ctypes.c_int32),
        "agx_soft64_throughput": ([_f64p], ctypes.c_int32),
        "agx_soft64_check": ([ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)],
                             ctypes.c_int32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _frame_arrays(fn, args, P, N):
    """Wait through `fn` for a frame in page-locked memory and copy it out."""
    fp = ctypes.POINTER(ctypes.c_float)
    v, c = fp(), fp()
    check(fn(*args, ctypes.byref(v), ctypes.byref(c)))
    vv = np.ctypeslib.as_array(v, shape=(3 * P,)).copy().reshape(3, P) if P else np.zeros((3, 0), np.float32)
    cc = np.ctypeslib.as_array(c, shape=(3 * N,)).copy().reshape(3, N)
    return vv, cc


def last_error():
    L = load()
    buf = ctypes.create_string_buffer(512)
    L.agx_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(code):
    if code != 0:
        raise AgxError(code, last_error())
    return code


def require_device():
    """Raise unless a CUDA device is visible to this process."""
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:  # pragma: no cover - torch is the device-memory plumbing
        ok = False
    if not ok:
        raise RuntimeError("anuga_core_gb300 needs a CUDA device (GB300); none is visible")


def ptr_f64(a):
    return a.ctypes.data_as(_f64p)


def ptr_i32(a):
    return a.ctypes.data_as(_i32p)


def mesh_desc(T):
    """MeshDesc over the numpy tables of tables.pack_tables (keeps references)."""
    d = MeshDesc()
    d.n_cells = T["conn"].shape[0]
    d.n_boundary = T["boundary_slot"].shape[0]
    d.n_edges = T["edge_slot"].shape[0]
    d.conn = ptr_i32(T["conn"])
    d.surr = ptr_i32(T["surr"])
    d.geo = ptr_f64(T["geo"])
    d.edge_slot = ptr_i32(T["edge_slot"])
    d.edge_opp = ptr_i32(T["edge_opp"])
    d.normals = ptr_f64(T["normals"])
    d.edgelengths = ptr_f64(T["edgelengths"])
    d.radii = ptr_f64(T["radii"])
    d.areas = ptr_f64(T["areas"])
    d.inv_area = ptr_f64(T["inv_area"])
    d.boundary_slot = ptr_i32(T["boundary_slot"])
    d.vertex_coordinates = ptr_f64(T["vertex_coordinates"])
    return d


class Scenario:
    """Owning wrapper of one agx scenario handle."""

    def __init__(self, tables, params):
        self.L = load()
        self.tables = tables
        self._desc = mesh_desc(tables)
        self.params = params
        h = ctypes.c_void_p()
        check(self.L.agx_scenario_create(ctypes.byref(self._desc), ctypes.byref(params), ctypes.byref(h)))
        self.h = h
        self.N = int(self._desc.n_cells)
        self.B = int(self._desc.n_boundary)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.agx_scenario_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field_len(self, name):
        if name.endswith("_e") or name.endswith("_v"):
            return 3 * self.N
        if name.endswith("_b"):
            return self.B
        return self.N

    def set(self, name, values):
        a = np.ascontiguousarray(np.asarray(values, np.float64).ravel())
        check(self.L.agx_set_field(self.h, FIELD[name], ptr_f64(a), a.size))

    def get(self, name, out=None):
        n = self.field_len(name)
        a = np.empty(n, np.float64) if out is None else out
        check(self.L.agx_get_field(self.h, FIELD[name], ptr_f64(a), n))
        return a

    def set_state(self, w, uh, vh):
        """stage, xmomentum, ymomentum centroid values in one call."""
        a = [np.ascontiguousarray(np.asarray(x, np.float64).ravel()) for x in (w, uh, vh)]
        check(self.L.agx_set_state(self.h, ptr_f64(a[0]), ptr_f64(a[1]), ptr_f64(a[2]), a[0].size))

    def get_state(self, w=None, uh=None, vh=None):
        out = [np.empty(self.N) if x is None else x for x in (w, uh, vh)]
        check(self.L.agx_get_state(self.h, ptr_f64(out[0]), ptr_f64(out[1]), ptr_f64(out[2]), self.N))
        return out

    def sww_bind(self, node_offsets, node_slots):
        off = np.ascontiguousarray(node_offsets, np.int32)
        sl = np.ascontiguousarray(node_slots, np.int32)
        check(self.L.agx_sww_bind(self.h, off.size - 1, ptr_i32(off), ptr_i32(sl)))
        self._sww_P = off.size - 1

    def sww_frame(self, min_storable_height, centroid_averaging=True):
        """(vertex [3, P], centroid [3, N]) float32 output frame."""
        fp = ctypes.POINTER(ctypes.c_float)
        v = np.empty((3, self._sww_P), np.float32)
        c = np.empty((3, self.N), np.float32)
        check(self.L.agx_sww_frame(self.h, float(min_storable_height), 1 if centroid_averaging else 0,
                                   v.ctypes.data_as(fp), c.ctypes.data_as(fp)))
        return v, c

    def sww_frame_async(self, min_storable_height, centroid_averaging=True):
        """Start forming a frame and copying it to page-locked memory; returns at once."""
        check(self.L.agx_sww_frame_async(self.h, float(min_storable_height), 1 if centroid_averaging else 0))

    def sww_frame_wait(self):
        """The frame started last, as copies of (vertex [3, P], centroid [3, N]) float32."""
        return _frame_arrays(self.L.agx_sww_frame_wait, (self.h,), self._sww_P, self.N)

    def device_ptr(self, name):
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        check(self.L.agx_device_ptr(self.h, FIELD[name], ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def set_boundary(self, kind, values):
        k = np.ascontiguousarray(kind, np.int32)
        v = np.ascontiguousarray(values, np.float64).reshape(-1)
        check(self.L.agx_set_boundary(self.h, ptr_i32(k), ptr_f64(v), k.size))

    def set_boundary_series(self, rows):
        r = np.ascontiguousarray(rows, np.float64).reshape(-1, 4)
        check(self.L.agx_set_boundary_series(self.h, ptr_f64(r), r.shape[0]))

    def add_rate(self, indices, rate, factor=1.0):
        if indices is None:
            check(self.L.agx_add_rate_operator(self.h, None, 0, float(rate), float(factor)))
        else:
            idx = np.ascontiguousarray(indices, np.int32)
            check(self.L.agx_add_rate_operator(self.h, ptr_i32(idx), idx.size, float(rate), float(factor)))

    def clear_operators(self):
        check(self.L.agx_clear_operators(self.h))

    def add_inlet(self, indices, Q, area, flags=0, velocity=(0.0, 0.0)):
        idx = np.ascontiguousarray(indices, np.int32)
        check(self.L.agx_add_inlet_operator(self.h, ptr_i32(idx), idx.size, float(Q), float(area), int(flags),
                                            float(velocity[0]), float(velocity[1])))

    def apply_operator(self, op, rate, factor, timestep):
        check(self.L.agx_apply_operator(self.h, int(op), float(rate), float(factor), float(timestep)))

    def operator_influx(self, op):
        v = ctypes.c_double()
        check(self.L.agx_operator_influx(self.h, op, ctypes.byref(v)))
        return v.value

    def protect(self):
        v = ctypes.c_double()
        check(self.L.agx_protect(self.h, ctypes.byref(v)))
        return v.value

    def distribute(self, with_protect=True):
        check(self.L.agx_distribute(self.h, 1 if with_protect else 0))

    def update_boundary(self, t):
        check(self.L.agx_update_boundary(self.h, float(t)))

    def compute_fluxes(self, substep):
        v = ctypes.c_double()
        check(self.L.agx_compute_fluxes(self.h, int(substep), ctypes.byref(v)))
        return v.value

    def compute_forcing(self):
        check(self.L.agx_compute_forcing(self.h))

    def update_conserved(self, dt):
        n = ctypes.c_int64()
        check(self.L.agx_update_conserved(self.h, float(dt), ctypes.byref(n)))
        return n.value

    def backup(self):
        check(self.L.agx_backup(self.h))

    def saxpy(self, a, b):
        check(self.L.agx_saxpy(self.h, float(a), float(b)))

    def divide(self, divisor):
        check(self.L.agx_divide_conserved(self.h, float(divisor)))

    def set_riverwalls(self, edge_counter, elevation, row_index, hydraulic):
        cnt = np.ascontiguousarray(edge_counter, np.int32)
        el = np.ascontiguousarray(elevation, np.float64)
        row = np.ascontiguousarray(row_index, np.int32)
        hyd = np.ascontiguousarray(hydraulic, np.float64)
        check(self.L.agx_set_riverwalls(self.h, ptr_i32(cnt), cnt.size, el.size, el.ctypes.data_as(_f64p),
                                        ptr_i32(row), hyd.shape[0], hyd.shape[1], hyd.ctypes.data_as(_f64p)))

    def set_clock(self, time, yield_time, final_time):
        check(self.L.agx_set_clock(self.h, float(time), float(yield_time), float(final_time)))

    def advance(self, max_steps=0):
        st = StepStats()
        check(self.L.agx_advance(self.h, int(max_steps), ctypes.byref(st)))
        return st

    def set_stream(self, stream_ptr):
        check(self.L.agx_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)))

    def time_phases(self, reps=2):
        ms = np.zeros(PHASE_COUNT)
        check(self.L.agx_time_phases(self.h, int(reps), ptr_f64(ms), PHASE_COUNT))
        return dict(zip(PHASES, ms.tolist()))

    def stats(self):
        st = StepStats()
        check(self.L.agx_get_stats(self.h, ctypes.byref(st)))
        return st

    def set_fixed_flux_timestep(self, flux_timestep):
        check(self.L.agx_set_fixed_flux_timestep(self.h, float(flux_timestep or 0.0)))


def kernel_launches():
    return int(load().agx_kernel_launches())


def fp64_throughput():
    """Measured FP64 DFMA / DDIV / DSQRT rates of the current device, G ops/s."""
    v = [np.zeros(1) for _ in range(3)]
    check(load().agx_fp64_throughput(*[ptr_f64(a) for a in v]))
    return {"dfma_gops": float(v[0][0]), "ddiv_gops": float(v[1][0]), "dsqrt_gops": float(v[2][0])}


def footprint(n_cells, n_boundary, n_edges, precision=AGX_PREC_FP64):
    return int(load().agx_scenario_footprint(n_cells, n_boundary, n_edges, precision))


def soft64_throughput():
    """G op/s of binary64 add, mul, div, sqrt on the FP64 pipe and on the
    integer pipes (exactly rounded), and half on each for div and mul."""
    v = np.zeros(10)
    check(load().agx_soft64_throughput(ptr_f64(v)))
    keys = ("fp64_add", "fp64_mul", "fp64_div", "fp64_sqrt", "int_add", "int_mul", "int_div", "int_sqrt",
            "half_div", "half_mul")
    return dict(zip(keys, v.tolist()))


def soft64_check(n, seed=1):
    """Mismatches of the device's integer-instruction add, sub, mul, div and
    sqrt against its FP64 pipe over n drawn cases each."""
    m = (ctypes.c_ulonglong * 5)()
    check(load().agx_soft64_check(int(n), int(seed), m))
    return dict(zip(("add", "sub", "mul", "div", "sqrt"), [int(x) for x in m]))
