"""Mixed-precision scenarios on a device pool (ctypes binding of agx_pool_*).

``Pool`` holds many scenarios in one device arena and advances every active
one per graph launch (the batched and serving forms).  ``MixedScenario`` is a
pool with one scenario, exposing the interface the Domain uses for the plain
FP64 scenario, so ``Domain.set_gpu_options(precision='mixed')`` switches the
step to the mixed-precision kernels.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .tables import pack_mixed

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)
_pool_lib = None


def lib():
    global _pool_lib
    if _pool_lib is None:
        L = _lib.load()
        H = ctypes.c_void_p
        P = ctypes.POINTER
        sig = {
            "agx_pool_create": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, P(H)], ctypes.c_int32),
            "agx_pool_destroy": ([H], ctypes.c_int32),
            "agx_pool_footprint": ([ctypes.c_int64, ctypes.c_int64, ctypes.c_int32], ctypes.c_int64),
            "agx_pool_bytes_per_cell": ([], ctypes.c_int64),
            "agx_pool_set_stream": ([H, ctypes.c_void_p], ctypes.c_int32),
            "agx_pool_set_state": ([H, ctypes.c_int32, _f64p, _f64p, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_get_state": ([H, ctypes.c_int32, _f64p, _f64p, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_add": ([H, ctypes.c_int64, ctypes.c_int64, _i32p, _f32p, _f64p, _f64p, _i32p, _i32p, _i32p,
                              _i32p, _i32p, ctypes.c_int64, _i32p, P(_lib.Params), P(ctypes.c_int32)],
                             ctypes.c_int32),
            "agx_pool_remove": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_set_field": ([H, ctypes.c_int32, ctypes.c_int32, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_get_field": ([H, ctypes.c_int32, ctypes.c_int32, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_set_boundary": ([H, ctypes.c_int32, _i32p, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_set_boundary_series": ([H, ctypes.c_int32, _f64p, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_add_rate": ([H, ctypes.c_int32, _i32p, ctypes.c_int64, ctypes.c_double, ctypes.c_double],
                                  ctypes.c_int32),
            "agx_pool_add_inlet": ([H, ctypes.c_int32, _i32p, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int32, ctypes.c_double, ctypes.c_double], ctypes.c_int32),
            "agx_pool_operators_from_host": ([H, ctypes.c_int32, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_apply_operator": ([H, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double], ctypes.c_int32),
            "agx_pool_set_riverwalls": ([H, ctypes.c_int32, _i32p, ctypes.c_int64, ctypes.c_int64, _f64p, _i32p,
                                         ctypes.c_int32, ctypes.c_int32, _f64p], ctypes.c_int32),
            "agx_pool_clear_operators": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_distribute": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_set_fixed_flux_timestep": ([H, ctypes.c_int32, ctypes.c_double], ctypes.c_int32),
            "agx_pool_sww_bind": ([H, ctypes.c_int32, ctypes.c_int64, _i32p, _i32p], ctypes.c_int32),
            "agx_pool_sww_frame_async": ([H, ctypes.c_int32, ctypes.c_double, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_sww_frame_wait": ([H, ctypes.c_int32, P(ctypes.POINTER(ctypes.c_float)),
                                         P(ctypes.POINTER(ctypes.c_float))], ctypes.c_int32),
            "agx_pool_set_clock": ([H, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int64], ctypes.c_int32),
            "agx_pool_deactivate": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_advance": ([H, P(ctypes.c_int32)], ctypes.c_int32),
            "agx_pool_step_begin": ([H], ctypes.c_int32),
            "agx_pool_step_stage": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_step_end": ([H, P(ctypes.c_int32)], ctypes.c_int32),
            "agx_pool_get_stats": ([H, ctypes.c_int32, P(_lib.StepStats)], ctypes.c_int32),
            "agx_pool_operator_influx": ([H, ctypes.c_int32, ctypes.c_int32, _f64p], ctypes.c_int32),
            "agx_pool_time_phases": ([H, ctypes.c_int32, _f64p, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_grid": ([H], ctypes.c_int32),
            "agx_pool_set_variant": ([H, ctypes.c_int32, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_set_l2_window": ([H, ctypes.c_int32], ctypes.c_int32),
            "agx_pool_snapshot": ([H], ctypes.c_int32),
            "agx_pool_launch_chunk": ([H, ctypes.c_int64], ctypes.c_int32),
            "agx_pool_wait": ([H, P(ctypes.c_int32)], ctypes.c_int32),
            "agx_pool_stats_all": ([H, ctypes.c_int32, _i32p, P(_lib.StepStats), _i32p], ctypes.c_int32),
            "agx_pool_capacity": ([H, P(ctypes.c_int64), P(ctypes.c_int64), P(ctypes.c_int64), P(ctypes.c_int32)],
                                  ctypes.c_int32),
            "agx_pool_restore": ([H], ctypes.c_int32),
            "agx_pool_last_error": ([ctypes.c_char_p, ctypes.c_int32], ctypes.c_int32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _pool_lib = L
    return _pool_lib


def _err():
    buf = ctypes.create_string_buffer(512)
    lib().agx_pool_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(code):
    if code != 0:
        raise _lib.AgxError(code, _err())
    return code


def footprint(cells, boundary, scenarios=1):
    return int(lib().agx_pool_footprint(int(cells), int(boundary), int(scenarios)))


def bytes_per_cell():
    return int(lib().agx_pool_bytes_per_cell())


class Pool:
    """Device pool of mixed-precision scenarios (capacities fixed at creation)."""

    def __init__(self, cap_cells, cap_boundary, cap_scenarios=1):
        self.L = lib()
        h = ctypes.c_void_p()
        check(self.L.agx_pool_create(int(cap_cells), int(cap_boundary), int(cap_scenarios), ctypes.byref(h)))
        self.h = h
        self.cap_cells = int(cap_cells)
        self.cap_boundary = int(cap_boundary)
        self.cap_scenarios = int(cap_scenarios)
        self._keep = {}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.agx_pool_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, ptr):
        check(self.L.agx_pool_set_stream(self.h, ctypes.c_void_p(ptr or 0)))

    def add(self, mesh, params, tables=None):
        T = tables if tables is not None else pack_mixed(mesh)
        N = T["conn"].shape[0]
        B = T["boundary_cell"].shape[0]
        sid = ctypes.c_int32()
        hc = T["halo_cells"] if T["halo_cells"].size else np.zeros(1, np.int32)
        check(self.L.agx_pool_add(self.h, N, B, T["conn"].ctypes.data_as(_i32p), T["geo"].ctypes.data_as(_f32p),
                                  T["area"].ctypes.data_as(_f64p), T["radius"].ctypes.data_as(_f64p),
                                  T["order"].ctypes.data_as(_i32p),
                                  T["boundary_cell"].ctypes.data_as(_i32p), T["lnk"].ctypes.data_as(_i32p),
                                  T["halo_off"].ctypes.data_as(_i32p), T["halo_cnt"].ctypes.data_as(_i32p),
                                  T["halo_cells"].size, hc.ctypes.data_as(_i32p), ctypes.byref(params),
                                  ctypes.byref(sid)))
        self._keep[sid.value] = (N, B)
        return sid.value

    def remove(self, sid):
        check(self.L.agx_pool_remove(self.h, int(sid)))
        self._keep.pop(sid, None)

    def set_field(self, sid, name, values):
        a = np.ascontiguousarray(np.asarray(values, np.float64).ravel())
        check(self.L.agx_pool_set_field(self.h, sid, _lib.FIELD[name], a.ctypes.data_as(_f64p), a.size))

    def set_state(self, sid, w, uh, vh):
        """stage, xmomentum, ymomentum centroid values of one scenario in one call."""
        a = [np.ascontiguousarray(np.asarray(x, np.float64).ravel()) for x in (w, uh, vh)]
        check(self.L.agx_pool_set_state(self.h, sid, *[x.ctypes.data_as(_f64p) for x in a], a[0].size))

    def get_state(self, sid, w=None, uh=None, vh=None):
        N, _ = self._keep[sid]
        out = [np.empty(N) if x is None else x for x in (w, uh, vh)]
        check(self.L.agx_pool_get_state(self.h, sid, *[x.ctypes.data_as(_f64p) for x in out], N))
        return out

    def get_field(self, sid, name, out=None):
        N, _ = self._keep[sid]
        n = 3 * N if (name.endswith("_e") or name.endswith("_v")) else N
        a = np.empty(n, np.float64) if out is None else out
        check(self.L.agx_pool_get_field(self.h, sid, _lib.FIELD[name], a.ctypes.data_as(_f64p), n))
        return a

    def set_boundary(self, sid, kind, values):
        k = np.ascontiguousarray(kind, np.int32)
        v = np.ascontiguousarray(values, np.float64).reshape(-1)
        check(self.L.agx_pool_set_boundary(self.h, sid, k.ctypes.data_as(_i32p), v.ctypes.data_as(_f64p), k.size))

    def set_boundary_series(self, sid, rows):
        r = np.ascontiguousarray(rows, np.float64).reshape(-1, 4)
        check(self.L.agx_pool_set_boundary_series(self.h, sid, r.ctypes.data_as(_f64p), r.shape[0]))

    def add_rate(self, sid, indices, rate, factor=1.0):
        if indices is None:
            check(self.L.agx_pool_add_rate(self.h, sid, None, 0, float(rate), float(factor)))
        else:
            idx = np.ascontiguousarray(indices, np.int32)
            check(self.L.agx_pool_add_rate(self.h, sid, idx.ctypes.data_as(_i32p), idx.size, float(rate),
                                           float(factor)))

    def add_inlet(self, sid, indices, Q, area, flags=0, velocity=(0.0, 0.0)):
        idx = np.ascontiguousarray(indices, np.int32)
        check(self.L.agx_pool_add_inlet(self.h, sid, idx.ctypes.data_as(_i32p), idx.size, float(Q), float(area),
                                        int(flags), float(velocity[0]), float(velocity[1])))

    def operators_from_host(self, sid, on=True):
        """Leave the scenario's operators out of the step loop; the caller
        applies them after each step with apply_operator."""
        check(self.L.agx_pool_operators_from_host(self.h, sid, 1 if on else 0))

    def apply_operator(self, sid, op, rate, factor, timestep):
        check(self.L.agx_pool_apply_operator(self.h, sid, int(op), float(rate), float(factor), float(timestep)))

    def set_riverwalls(self, sid, edge_counter, elevation, row_index, hydraulic):
        cnt = np.ascontiguousarray(edge_counter, np.int32)
        el = np.ascontiguousarray(elevation, np.float64)
        row = np.ascontiguousarray(row_index, np.int32)
        hyd = np.ascontiguousarray(hydraulic, np.float64).reshape(-1, 5)
        check(self.L.agx_pool_set_riverwalls(self.h, sid, cnt.ctypes.data_as(_i32p), cnt.size, el.size,
                                             el.ctypes.data_as(_f64p), row.ctypes.data_as(_i32p), hyd.shape[0],
                                             hyd.shape[1], hyd.ctypes.data_as(_f64p)))

    def clear_operators(self, sid):
        check(self.L.agx_pool_clear_operators(self.h, sid))

    def operator_influx(self, sid, op):
        v = ctypes.c_double()
        check(self.L.agx_pool_operator_influx(self.h, sid, op, ctypes.byref(v)))
        return v.value

    def sww_bind(self, sid, node_offsets, node_slots):
        off = np.ascontiguousarray(node_offsets, np.int32)
        sl = np.ascontiguousarray(node_slots, np.int32)
        check(self.L.agx_pool_sww_bind(self.h, int(sid), off.size - 1, off.ctypes.data_as(_i32p),
                                       sl.ctypes.data_as(_i32p)))

    def sww_frame_async(self, sid, min_storable_height, centroid_averaging=True):
        check(self.L.agx_pool_sww_frame_async(self.h, int(sid), float(min_storable_height),
                                              1 if centroid_averaging else 0))

    def sww_frame_wait(self, sid, P):
        N, _ = self._keep[sid]
        return _lib._frame_arrays(self.L.agx_pool_sww_frame_wait, (self.h, int(sid)), P, N)

    def set_fixed_flux_timestep(self, sid, flux_timestep):
        check(self.L.agx_pool_set_fixed_flux_timestep(self.h, int(sid), float(flux_timestep or 0.0)))

    def distribute(self, sid):
        check(self.L.agx_pool_distribute(self.h, sid))

    def set_clock(self, sid, time, yield_time, final_time, max_steps=0):
        check(self.L.agx_pool_set_clock(self.h, sid, float(time), float(yield_time), float(final_time),
                                        int(max_steps)))

    def deactivate(self, sid):
        check(self.L.agx_pool_deactivate(self.h, sid))

    def advance(self):
        n = ctypes.c_int32()
        check(self.L.agx_pool_advance(self.h, ctypes.byref(n)))
        return n.value

    def step_begin(self):
        """First stage of one step of every active scenario (see step_end)."""
        check(self.L.agx_pool_step_begin(self.h))

    def step_stage(self, stage):
        """Stage 2 or 3 of the split step on its own (after step_begin)."""
        check(self.L.agx_pool_step_stage(self.h, int(stage)))

    def step_end(self):
        """The remaining stages, step-loop operators and clocks; returns the
        number of scenarios whose clock stopped."""
        n = ctypes.c_int32()
        check(self.L.agx_pool_step_end(self.h, ctypes.byref(n)))
        return n.value

    def stats(self, sid):
        st = _lib.StepStats()
        check(self.L.agx_pool_get_stats(self.h, sid, ctypes.byref(st)))
        return st

    def time_phases(self, reps=2):
        ms = np.zeros(_lib.PHASE_COUNT)
        check(self.L.agx_pool_time_phases(self.h, int(reps), ms.ctypes.data_as(_f64p), _lib.PHASE_COUNT))
        return dict(zip(_lib.PHASES, ms.tolist()))

    @property
    def grid(self):
        return int(self.L.agx_pool_grid(self.h))

    def set_variant(self, variant, grid_mode):
        check(self.L.agx_pool_set_variant(self.h, int(variant), int(grid_mode)))
        self.variant = (int(variant), int(grid_mode))

    def set_l2_window(self, on):
        check(self.L.agx_pool_set_l2_window(self.h, 1 if on else 0))
        self.l2_window = bool(on)

    def snapshot(self):
        check(self.L.agx_pool_snapshot(self.h))

    def restore(self):
        check(self.L.agx_pool_restore(self.h))

    def scenarios(self):
        return sorted(self._keep)

    def launch_chunk(self, max_steps):
        check(self.L.agx_pool_launch_chunk(self.h, int(max_steps)))

    def wait(self):
        n = ctypes.c_int32()
        check(self.L.agx_pool_wait(self.h, ctypes.byref(n)))
        return n.value

    def stats_all(self, sids):
        n = len(sids)
        arr = (_lib.StepStats * max(n, 1))()
        ids = np.ascontiguousarray(sids, np.int32)
        run = np.zeros(max(n, 1), np.int32)
        check(self.L.agx_pool_stats_all(self.h, n, ids.ctypes.data_as(_i32p), arr, run.ctypes.data_as(_i32p)))
        return [arr[i] for i in range(n)], run[:n].astype(bool)

    def capacity(self):
        fc, fb, fh = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        fs = ctypes.c_int32()
        check(self.L.agx_pool_capacity(self.h, ctypes.byref(fc), ctypes.byref(fb), ctypes.byref(fh), ctypes.byref(fs)))
        return dict(cells=fc.value, boundary=fb.value, halo=fh.value, scenarios=fs.value)


class MixedScenario:
    """One mixed-precision scenario (a pool of one) with the Scenario interface."""

    CENTROID_IN = ("stage_c", "xmom_c", "ymom_c", "elev_c", "friction_c")

    def __init__(self, mesh, plain_tables, params):
        self.mesh = mesh
        self.N = len(mesh)
        self.B = int(mesh.boundary_length)
        self.params = params
        self.tables = pack_mixed(mesh)
        self.pool = Pool(self.N, max(self.B, 1), 1)
        self.sid = self.pool.add(mesh, params, self.tables)
        self._elev_set = False

    def close(self):
        self.pool.close()

    def field_len(self, name):
        return 3 * self.N if (name.endswith("_e") or name.endswith("_v")) else (self.B if name.endswith("_b") else self.N)

    def set(self, name, values):
        if name in self.CENTROID_IN:
            self.pool.set_field(self.sid, name, values)

    def set_state(self, w, uh, vh):
        self.pool.set_state(self.sid, w, uh, vh)

    def get_state(self, w=None, uh=None, vh=None):
        return self.pool.get_state(self.sid, w, uh, vh)

    def get(self, name, out=None):
        n = self.field_len(name)
        out = np.empty(n) if out is None else out
        if name.endswith("_b") or name.endswith("_s") or name == "elev_v":
            if name == "elev_v":
                v = self.pool.get_field(self.sid, "elev_e")
                e = v.reshape(-1, 3)
                out.reshape(-1, 3)[:] = np.stack([e[:, 1] + e[:, 2] - e[:, 0], e[:, 0] + e[:, 2] - e[:, 1],
                                                  e[:, 0] + e[:, 1] - e[:, 2]], 1)
                return out
            out[:] = 0.0       # not kept by the mixed form
            return out
        return self.pool.get_field(self.sid, name, out=out)

    def device_ptr(self, name):
        raise NotImplementedError("device views are provided for the FP64 scenario")

    def set_boundary(self, kind, values):
        self.pool.set_boundary(self.sid, kind, values)

    def set_boundary_series(self, rows):
        self.pool.set_boundary_series(self.sid, rows)

    def add_rate(self, indices, rate, factor=1.0):
        self.pool.add_rate(self.sid, indices, rate, factor)

    def add_inlet(self, indices, Q, area, flags=0, velocity=(0.0, 0.0)):
        self.pool.add_inlet(self.sid, indices, Q, area, flags, velocity)

    def operators_from_host(self, on=True):
        self.pool.operators_from_host(self.sid, on)

    def set_riverwalls(self, edge_counter, elevation, row_index, hydraulic):
        self.pool.set_riverwalls(self.sid, edge_counter, elevation, row_index, hydraulic)

    def apply_operator(self, op, rate, factor, timestep):
        self.pool.apply_operator(self.sid, op, rate, factor, timestep)

    def clear_operators(self):
        self.pool.clear_operators(self.sid)

    def operator_influx(self, op):
        return self.pool.operator_influx(self.sid, op)

    def distribute(self, with_protect=True):
        self.pool.distribute(self.sid)

    def protect(self):
        self.pool.distribute(self.sid)
        return 0.0

    def update_boundary(self, t):
        pass   # boundary values are evaluated inside the flux kernel

    def _no_phase(self, *a):
        raise NotImplementedError("per-phase calls are provided by the FP64 scenario; the mixed form "
                                  "runs whole steps (evolve / advance_steps)")

    compute_fluxes = compute_forcing = update_conserved = backup = saxpy = _no_phase

    def set_clock(self, time, yield_time, final_time):
        self._clock = (time, yield_time, final_time)

    def advance(self, max_steps=0):
        t, y, f = getattr(self, "_clock", (0.0, 1e300, -1.0))
        self.pool.set_clock(self.sid, t, y, f, max_steps)
        self.pool.advance()
        return self.pool.stats(self.sid)

    def step_begin(self):
        """One step (set_clock first) up to the end of its first stage;
        returns the step's timestep."""
        t, y, f = getattr(self, "_clock", (0.0, 1e300, -1.0))
        self.pool.set_clock(self.sid, t, y, f, 1)
        self.pool.step_begin()
        return self.pool.stats(self.sid).last_timestep

    def step_stage(self, stage):
        self.pool.step_stage(stage)

    def step_end(self):
        self.pool.step_end()
        return self.pool.stats(self.sid)

    def stats(self):
        return self.pool.stats(self.sid)

    def set_fixed_flux_timestep(self, flux_timestep):
        self.pool.set_fixed_flux_timestep(self.sid, flux_timestep)

    def sww_bind(self, node_offsets, node_slots):
        self.pool.sww_bind(self.sid, node_offsets, node_slots)
        self._sww_P = len(node_offsets) - 1

    def sww_frame_async(self, min_storable_height, centroid_averaging=True):
        self.pool.sww_frame_async(self.sid, min_storable_height, centroid_averaging)

    def sww_frame_wait(self):
        return self.pool.sww_frame_wait(self.sid, self._sww_P)

    def sww_frame(self, min_storable_height, centroid_averaging=True):
        self.sww_frame_async(min_storable_height, centroid_averaging)
        return self.sww_frame_wait()

    def set_stream(self, ptr):
        self.pool.set_stream(ptr)

    def time_phases(self, reps=2):
        return self.pool.time_phases(reps)
