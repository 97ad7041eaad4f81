"""Drop-in shallow-water Domain whose DE timestep runs on the GPU.

Keeps the user-facing API of the reference's ``anuga.Domain``
(shallow_water/shallow_water_domain.py:144 and
abstract_2d_finite_volumes/generic_domain.py): construction from points,
triangles and a boundary dictionary, ``set_flow_algorithm``,
``set_quantity``/``get_quantity``, ``set_boundary``, fractional-step
operators, ``evolve(yieldstep, finaltime|duration)`` as a generator, sww
output and the per-phase methods (``distribute_to_vertices_and_edges``,
``update_boundary``, ``compute_fluxes``, ``compute_forcing_terms``,
``update_timestep``, ``update_conserved_quantities``, ...).

What changes is where the work happens: quantity storage, boundary
evaluation and the step loop live on the device (libagx), and a whole
yieldstep runs as one graph launch with a device-side loop.  The host arrays
behind ``Quantity`` objects are mirrors refreshed on access.
"""
from __future__ import annotations

import os
import pickle
import time
import warnings

import numpy as np

from . import _lib
from .mesh import Mesh, rectangular_cross
from .quantity import Quantity, DEVICE_FIELDS
from .operators import boundary_flux_integral_operator
from .tables import pack_tables

EPSILON = 1.0e-12        # anuga/config.py:12
G = 9.8                  # anuga/config.py:45
MAX_TIMESTEP = 1.0e3     # anuga/config.py:154
MIN_TIMESTEP = 1.0e-6    # anuga/config.py min_timestep
MAX_SMALLSTEPS = 50      # anuga/config.py max_smallsteps

# shallow_water_domain.py:583-707
# shallow_water/shallow_water_domain.py:583-877 (_set_DE*_defaults)
FLOW_ALGORITHMS = {
    "DE0": dict(CFL=0.9, timestepping_method="euler", minimum_allowed_height=1.0e-12,
                beta_w=0.5, beta_w_dry=0.0, beta_uh=0.5, beta_uh_dry=0.0, beta_vh=0.5, beta_vh_dry=0.0),
    "DE1": dict(CFL=1.0, timestepping_method="rk2", minimum_allowed_height=1.0e-5,
                beta_w=1.0, beta_w_dry=0.0, beta_uh=1.0, beta_uh_dry=0.0, beta_vh=1.0, beta_vh_dry=0.0),
    "DE2": dict(CFL=1.0, timestepping_method="rk3", minimum_allowed_height=1.0e-5,
                beta_w=1.0, beta_w_dry=0.0, beta_uh=1.0, beta_uh_dry=0.0, beta_vh=1.0, beta_vh_dry=0.0),
    "DE0_7": dict(CFL=0.9, timestepping_method="euler", minimum_allowed_height=1.0e-12,
                  beta_w=0.7, beta_w_dry=0.1, beta_uh=0.7, beta_uh_dry=0.1, beta_vh=0.7, beta_vh_dry=0.1),
    "DE1_7": dict(CFL=1.0, timestepping_method="rk2", minimum_allowed_height=1.0e-12,
                  beta_w=0.75, beta_w_dry=0.1, beta_uh=0.75, beta_uh_dry=0.1, beta_vh=0.75, beta_vh_dry=0.1),
}
_TIMESTEPPING = {"euler": 1, "rk2": 2, "rk3": 3}

_STATE_FIELDS = ("stage_c", "xmom_c", "ymom_c")     # pulled eagerly at every yield
_SYNCED, _DEV_NEWER, _HOST_NEWER = 0, 1, 2


def manning_friction_implicit(domain):
    """Marker for the default forcing term (shallow_water/friction.py:23).  It
    is evaluated on the device inside the update kernel."""
    return None


class Domain:
    def __init__(self, coordinates=None, vertices=None, boundary=None, tagged_elements=None,
                 geo_reference=None, use_inscribed_circle=False, mesh=None, starttime=0.0,
                 verbose=False, **kwargs):
        if mesh is None:
            if coordinates is None or vertices is None:
                raise ValueError("Domain needs coordinates and vertices (or a mesh)")
            mesh = Mesh(coordinates, vertices, boundary, use_inscribed_circle=use_inscribed_circle)
        self.mesh = mesh
        self.verbose = verbose
        self.tagged_elements = tagged_elements or {}
        self.number_of_triangles = self.number_of_elements = len(mesh)
        self.conserved_quantities = ["stage", "xmomentum", "ymomentum"]
        self.evolved_quantities = ["stage", "xmomentum", "ymomentum"]
        self.other_quantities = ["elevation", "friction", "height", "xvelocity", "yvelocity", "x", "y"]
        self.quantities = {}
        for name in self.conserved_quantities + self.other_quantities:
            self.quantities[name] = Quantity(self, name)
        self._farr = {}
        for qn, fields in DEVICE_FIELDS.items():
            Q = self.quantities[qn]
            for slot, f in zip(("centroid_values", "edge_values", "vertex_values", "boundary_values",
                                "explicit_update", "semi_implicit_update"), fields):
                if f is not None:
                    self._farr[f] = Q._arr[slot]
        self._farr["max_speed"] = np.zeros(len(mesh))
        self._fstate = {f: _SYNCED for f in self._farr}
        self._scn = None
        self._scn_key = None
        self.fractional_step_operators = []
        self.forcing_terms = [manning_friction_implicit]
        self.boundary_map = None
        self.boundary_objects = None
        self.starttime = float(starttime)
        self.relative_time = 0.0
        self.evolve_starttime = 0.0
        self.timestep = 0.0
        self.flux_timestep = 0.0
        self.evolved_called = False
        self.yieldstep_counter = 0
        self.number_of_steps = 0
        self.total_steps = 0
        self.number_of_first_order_steps = 0
        self.recorded_min_timestep = MAX_TIMESTEP
        self.recorded_max_timestep = MIN_TIMESTEP
        self.g = G
        self.epsilon = EPSILON
        self.evolve_max_timestep = MAX_TIMESTEP
        self.evolve_min_timestep = MIN_TIMESTEP
        self.max_smallsteps = MAX_SMALLSTEPS
        self.low_froude = 0
        self.extrapolate_velocity_second_order = True
        self.use_sloped_mannings = False
        self.centroid_transmissive_bc = False
        self.protect_zero_ymom = False
        self.precision = "fp64"
        self.multiprocessor_mode = 2
        self.store = True
        self.name = "domain"
        self.datadir = "."
        self.writer = None
        self.minimum_storable_height = 1.0e-3
        self.set_flow_algorithm("DE0")
        # riverwalls (structures/riverwall.py; shallow_water_domain.py:366-379)
        self.edge_flux_type = np.zeros(3 * len(mesh), np.int64)
        self.edge_river_wall_counter = np.zeros(3 * len(mesh), np.int64)
        self.number_of_riverwall_edges = 0
        from .riverwall import RiverWall
        self.riverwallData = RiverWall(self)
        self.create_riverwalls = self.riverwallData.create_riverwalls
        self.quantities["x"].set_values(self.mesh.vertex_coordinates[:, 0].reshape(-1, 3))
        self.quantities["y"].set_values(self.mesh.vertex_coordinates[:, 1].reshape(-1, 3))
        self._mass_added_seen = 0.0
        # boundary fluxes of the last step's stages, and their time integral
        # (shallow_water_domain.py:380-387: the operator comes first among
        # the fractional steps)
        self.boundary_flux_sum = np.zeros(3)
        self.boundary_flux_integral = boundary_flux_integral_operator(self)
        self.volume_history = []
        self.fixed_flux_timestep = None
        # anuga/config.py:151 (generic_domain.py:331-332)
        self.protect_against_isolated_degenerate_timesteps = False

    # ------------------------------------------------------------------
    # mesh accessors
    def __len__(self):
        return self.number_of_triangles

    @property
    def boundary(self):
        return self.mesh.boundary

    @property
    def boundary_length(self):
        return self.mesh.boundary_length

    @property
    def areas(self):
        return self.mesh.areas

    @property
    def normals(self):
        return self.mesh.normals

    @property
    def neighbours(self):
        return self.mesh.neighbours

    @property
    def centroid_coordinates(self):
        return self.mesh.centroid_coordinates

    @property
    def vertex_coordinates(self):
        return self.mesh.vertex_coordinates

    @property
    def edge_coordinates(self):
        return self.mesh.edge_midpoint_coordinates

    @property
    def tag_boundary_cells(self):
        return self.mesh.tag_boundary_cells

    @property
    def boundary_cells(self):
        return self.mesh.boundary_cells

    @property
    def boundary_edges(self):
        return self.mesh.boundary_edges

    def get_centroid_coordinates(self, absolute=False):
        return self.mesh.centroid_coordinates

    def get_vertex_coordinates(self, absolute=False):
        return self.mesh.vertex_coordinates

    def get_edge_midpoint_coordinates(self, absolute=False):
        return self.mesh.edge_midpoint_coordinates

    def get_boundary_tags(self):
        return self.mesh.get_boundary_tags()

    def get_area(self):
        return self.mesh.get_area()

    # ------------------------------------------------------------------
    # configuration
    def set_flow_algorithm(self, flow_algorithm="DE0"):
        flow_algorithm = str(flow_algorithm).upper().replace(".", "_")
        if flow_algorithm not in FLOW_ALGORITHMS:
            raise ValueError("Unknown flow_algorithm. \nPossible choices are:\n" + ", ".join(FLOW_ALGORITHMS) + ".")
        d = FLOW_ALGORITHMS[flow_algorithm]
        self.flow_algorithm = flow_algorithm
        self.CFL = d["CFL"]
        self.timestepping_method = d["timestepping_method"]
        self.minimum_allowed_height = d["minimum_allowed_height"]
        for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
            setattr(self, k, d[k])
        self.default_order = 2
        self._order_ = 2
        # the DE algorithms store node values as means of centroid values
        # (shallow_water_domain.py:596, 659, 722)
        self.using_centroid_averaging = True
        self._invalidate_device()

    def set_using_centroid_averaging(self, flag=True):
        """Node values (sww output) as means of the adjacent centroid values
        (True) or of the vertex values (False); generic_domain.py:765-782."""
        self.using_centroid_averaging = bool(flag)

    def get_using_centroid_averaging(self):
        return self.using_centroid_averaging

    def get_flow_algorithm(self):
        return self.flow_algorithm

    def set_CFL(self, cfl):
        self.CFL = float(cfl)
        self._invalidate_device()

    def set_timestepping_method(self, m):
        m = {1: "euler", 2: "rk2", 3: "rk3"}.get(m, m)
        if m not in _TIMESTEPPING:
            raise ValueError("%s is an incorrect timestepping type" % (m,))
        self.timestepping_method = m
        self._invalidate_device()

    def get_timestepping_method(self):
        return self.timestepping_method

    def set_minimum_allowed_height(self, h):
        self.minimum_allowed_height = float(h)
        self._invalidate_device()

    def set_betas(self, beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry):
        self.beta_w, self.beta_w_dry = beta_w, beta_w_dry
        self.beta_uh, self.beta_uh_dry = beta_uh, beta_uh_dry
        self.beta_vh, self.beta_vh_dry = beta_vh, beta_vh_dry
        self._invalidate_device()

    def set_low_froude(self, low_froude=0):
        self.low_froude = int(low_froude)
        self._invalidate_device()

    def set_use_sloped_mannings(self, flag=True):
        self.use_sloped_mannings = bool(flag)
        self._invalidate_device()

    def set_centroid_transmissive_bc(self, flag):
        self.centroid_transmissive_bc = bool(flag)
        self._bind_boundaries()

    def set_multiprocessor_mode(self, mode=2):
        """Accepted for compatibility; the DE step always runs on the GPU."""
        self.multiprocessor_mode = int(mode)

    def set_gpu_options(self, precision=None):
        if precision is not None:
            if precision not in ("fp64", "mixed"):
                raise ValueError("precision must be 'fp64' or 'mixed'")
            self.precision = precision
            self._invalidate_device()

    def set_fixed_flux_timestep(self, flux_timestep=None):
        """Disable variable timestepping with a fixed flux timestep, or
        re-enable it with None (generic_domain.py:2332-2346)."""
        if flux_timestep is not None and not flux_timestep > 0.0:
            raise Exception("flux_timestep needs to be greater than 0.0")
        self.fixed_flux_timestep = None if flux_timestep is None else float(flux_timestep)
        if self._scn is not None:
            self._scn.set_fixed_flux_timestep(self.fixed_flux_timestep)

    def set_evolve_max_timestep(self, t):
        self.evolve_max_timestep = float(t)
        self._invalidate_device()

    def set_store(self, flag=True):
        self.store = bool(flag)

    def set_name(self, name):
        self.name = str(name)

    def get_name(self):
        return self.name

    def set_datadir(self, d):
        self.datadir = str(d)

    def set_minimum_storable_height(self, h):
        self.minimum_storable_height = float(h)

    def set_starttime(self, t):
        self.starttime = float(t)

    def get_time(self):
        return self.starttime + self.relative_time

    def get_relative_time(self):
        return self.relative_time

    def set_relative_time(self, t):
        self.relative_time = float(t)

    def get_timestep(self):
        return self.timestep

    def get_evolve_starttime(self):
        return self.evolve_starttime

    # ------------------------------------------------------------------
    # quantities
    def get_quantity(self, name):
        return self.quantities[name]

    def set_quantity(self, name, *args, **kwargs):
        if "expression" in kwargs:
            raise NotImplementedError("expression= is not provided; pass an array or function")
        self.quantities[name].set_values(*args, **kwargs)

    def _quantity_changed(self, name):
        pass

    def get_conserved_quantities(self, vol_id, vertex=None, edge=None):
        out = []
        for n in self.conserved_quantities:
            Q = self.quantities[n]
            if edge is not None:
                out.append(Q.edge_values[vol_id, edge])
            elif vertex is not None:
                out.append(Q.vertex_values[vol_id, vertex])
            else:
                out.append(Q.centroid_values[vol_id])
        return np.array(out)

    # ------------------------------------------------------------------
    # host mirror <-> device synchronisation
    def _host_view(self, field, arr):
        if self._scn is not None and self._fstate.get(field) == _DEV_NEWER:
            self._scn.get(field, out=arr.reshape(-1))
        if field in self._fstate:
            # the caller may edit the array in place: send it back before the
            # next device operation
            self._fstate[field] = _HOST_NEWER if self._scn is not None else _SYNCED

    def _host_modified(self, field):
        if field in self._fstate and self._scn is not None:
            self._fstate[field] = _HOST_NEWER

    def _refresh_velocity(self, Q, slot):
        src = {"xvelocity": "xmomentum", "yvelocity": "ymomentum"}[Q.name]
        if slot == "centroid_values":
            h = self.quantities["height"].centroid_values
            m = self.quantities[src].centroid_values
        elif slot == "edge_values":
            h = self.quantities["height"].edge_values
            m = self.quantities[src].edge_values
        else:
            return
        with np.errstate(divide="ignore", invalid="ignore"):
            Q._arr[slot][...] = np.where(h > self.minimum_allowed_height, m / h, 0.0)

    def _push_dirty(self):
        for f, st in self._fstate.items():
            if st == _HOST_NEWER:
                self._scn.set(f, self._farr[f])
                self._fstate[f] = _SYNCED

    def _mark_device_newer(self, fields=None):
        for f in (self._fstate if fields is None else fields):
            self._fstate[f] = _DEV_NEWER

    def _pull(self, fields):
        for f in fields:
            if self._fstate[f] == _DEV_NEWER:
                self._scn.get(f, out=self._farr[f].reshape(-1))
                self._fstate[f] = _SYNCED

    def _params(self):
        p = _lib.Params()
        p.g = self.g
        p.epsilon = self.epsilon
        p.minimum_allowed_height = self.minimum_allowed_height
        for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
            setattr(p, k, getattr(self, k))
        p.CFL = self.CFL
        p.evolve_max_timestep = self.evolve_max_timestep
        p.evolve_min_timestep = self.evolve_min_timestep
        p.extrapolate_velocity_second_order = 1 if self.extrapolate_velocity_second_order else 0
        p.low_froude = self.low_froude
        p.timestepping_method = _TIMESTEPPING[self.timestepping_method]
        p.protect_zero_ymom = 1 if self.protect_zero_ymom else 0
        p.use_sloped_mannings = 1 if self.use_sloped_mannings else 0
        p.max_smallsteps = self.max_smallsteps
        p.precision = _lib.AGX_PREC_FP64 if self.precision == "fp64" else _lib.AGX_PREC_MIXED
        return p

    def _invalidate_device(self):
        if self._scn is not None:
            self.flush_sww()
            # keep the device state: pull everything the host may not have yet
            self._pull([f for f in self._fstate])
            self.boundary_flux_integral.fold_device()
            self._scn.close()
            self._scn = None
            for f in self._fstate:
                self._fstate[f] = _SYNCED

    def _riverwalls_changed(self):
        self._invalidate_device()

    def _ensure_device(self):
        if self._scn is not None:
            return self._scn
        _lib.require_device()
        per_side = None
        if self.low_froude:
            per_side = np.ones((len(self), 3), bool)
        rw = self.riverwallData
        if rw.active:
            # the weir correction uses each side's own heads: no shared edge flux
            marks = (self.edge_flux_type == 1).reshape(-1, 3)
            per_side = marks if per_side is None else (per_side | marks)
        if self.precision == "mixed":
            from .mixed import MixedScenario
            self._scn = MixedScenario(self.mesh, None, self._params())
            if rw.active:
                self._scn.set_riverwalls(self.edge_river_wall_counter, rw.riverwall_elevation,
                                         rw.hydraulic_properties_rowIndex, rw.hydraulic_properties)
        else:
            key = (self.low_froude, tuple(rw.riverwall_edges) if rw.active else ())
            if not hasattr(self, "_tables") or self._tables_key != key:
                self._tables = pack_tables(self.mesh, per_side_edges=per_side)
                self._tables_key = key
            self._scn = _lib.Scenario(self._tables, self._params())
            if rw.active:
                self._scn.set_riverwalls(self.edge_river_wall_counter, rw.riverwall_elevation,
                                         rw.hydraulic_properties_rowIndex, rw.hydraulic_properties)
        up = self._upload_fields()
        for f in self._fstate:
            if f in up:
                self._scn.set(f, self._farr[f])
            self._fstate[f] = _SYNCED
        self._bind_boundaries()
        self._bind_operators()
        if self.fixed_flux_timestep is not None:
            self._scn.set_fixed_flux_timestep(self.fixed_flux_timestep)
        return self._scn

    def _upload_fields(self):
        if self.precision == "mixed":
            return {"stage_c", "xmom_c", "ymom_c", "elev_c", "friction_c"}
        return {"stage_c", "xmom_c", "ymom_c", "elev_c", "friction_c", "elev_v",
                "stage_e", "xmom_e", "ymom_e", "elev_e", "height_e",
                "stage_b", "xmom_b", "ymom_b", "stage_s", "xmom_s", "ymom_s"}

    def device_tensor(self, name, location="centroids"):
        """Zero-copy torch view of a device field (the handle outlives it)."""
        import torch
        scn = self._ensure_device()
        self._push_dirty()
        loc = {"centroids": "_c", "edges": "_e", "vertices": "_v", "boundary": "_b"}[location]
        field = DEVICE_FIELDS[name][("_c", "_e", "_v", "_b").index(loc)]
        ptr, n = scn.device_ptr(field)
        self._fstate[field] = _DEV_NEWER   # the caller may write through the view

        class _CAI:
            __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3}
        return torch.as_tensor(_CAI(), device="cuda")

    # ------------------------------------------------------------------
    # boundaries and operators
    def set_boundary(self, boundary_map):
        if self.boundary_map is None:
            self.boundary_map = {}
        for tag, B in boundary_map.items():
            if tag not in self.mesh.tag_boundary_cells:
                raise ValueError("Tag %s provided does not exist in the domain. Boundary tags are %s"
                                 % (tag, self.get_boundary_tags()))
            self.boundary_map[tag] = B
        self.boundary_objects = [(k, self.boundary_map.get(self.mesh.boundary[k])) for k in sorted(self.mesh.boundary)]
        self._bind_boundaries()

    def _boundary_arrays(self, t):
        Bn = self.mesh.boundary_length
        kind = np.zeros(Bn, np.int32)
        vals = np.zeros((Bn, 3))
        series = None
        for tag, ids in self.mesh.tag_boundary_cells.items():
            B = self.boundary_map.get(tag) if self.boundary_map else None
            if B is None:
                continue
            k = getattr(B, "effective_kind", B.kind)
            kind[ids] = k
            if getattr(B, "series", None) is not None:
                if series is not None and not np.array_equal(series, B.series):
                    raise NotImplementedError("one time series per domain is supported")
                series = B.series
            elif hasattr(B, "edge_values"):
                m = self.mesh
                s = 3 * np.asarray(m.boundary_cells)[ids] + np.asarray(m.boundary_edges)[ids]
                nrm = np.asarray(m.normals).reshape(-1, 2)
                mid = np.asarray(m.edge_midpoint_coordinates)
                vals[ids] = B.edge_values(t, nrm[s, 0], nrm[s, 1], mid[s, 0], mid[s, 1], tag)
            elif k in (_lib.BC_DIRICHLET, _lib.BC_TRANSMISSIVE_N0, _lib.BC_TRANSMISSIVE_SET_STAGE, _lib.BC_FLATHER,
                       _lib.BC_CHARACTERISTIC):
                vals[ids] = B.values(t)
        return kind, vals, series

    def _bind_boundaries(self, t=None):
        if self._scn is None or self.boundary_map is None:
            return
        kind, vals, series = self._boundary_arrays(self.get_time() if t is None else t)
        self._scn.set_boundary(kind, vals)
        if series is not None:
            self._scn.set_boundary_series(series)

    def _operators_changed(self):
        if self._scn is not None:
            self._bind_operators()

    def _bind_operators(self):
        """Register every Rate_operator on the device (indices uploaded once).
        Constant ones run inside the device step loop; the others are applied
        from the host step by step (agx_apply_operator) with the rate the
        host evaluates."""
        self._scn.clear_operators()
        self._dev_ops = []
        t = self.get_time()
        for op in self.fractional_step_operators:
            if hasattr(op, "rate"):
                self._scn.add_rate(op.indices, op.get_rate(t), op.get_factor(t))
            elif hasattr(op, "update_Q"):
                self._scn.add_inlet(op.indices, op.update_Q(t), op.area, op.flags,
                                    op.velocity if op.velocity is not None else (0.0, 0.0))
            else:
                continue
            op._dev_index = len(self._dev_ops)
            self._dev_ops.append(op)

    def set_conserved_state(self, stage, xmomentum, ymomentum):
        """Centroid stage, xmomentum and ymomentum in one call and one
        device transfer (page-locked arrays are read by the device directly)."""
        scn = self._ensure_device()
        self._push_dirty()
        scn.set_state(stage, xmomentum, ymomentum)
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c"])

    def get_conserved_state(self, stage=None, xmomentum=None, ymomentum=None):
        """Centroid stage, xmomentum and ymomentum from the device in one
        call, into the given arrays (page-locked ones are written by the
        device directly) or new ones; returns the three arrays."""
        scn = self._ensure_device()
        self._push_dirty()
        return scn.get_state(stage, xmomentum, ymomentum)

    def _apply_rate_now(self, op, rate, factor, dt):
        """One application of a registered Rate_operator on the device."""
        scn = self._ensure_device()
        self._push_dirty()
        scn.apply_operator(op._dev_index, rate, factor, dt)
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c"])

    def _device_loop_ok(self):
        if self.boundary_map is None:
            return True
        for B in self.boundary_map.values():
            if B is not None and not getattr(B, "device_loop", True):
                return False
        for op in self.fractional_step_operators:
            if not getattr(op, "device_loop", False):
                return False
        if any(f is not manning_friction_implicit for f in self.forcing_terms):
            return False
        if self.protect_against_isolated_degenerate_timesteps:
            return False          # evaluated by the host between the phases of each step
        return True

    # ------------------------------------------------------------------
    # per-phase interface (the reference's plugin surface)
    def protect_against_infinitesimal_and_negative_heights(self):
        scn = self._ensure_device()
        self._push_dirty()
        m = scn.protect()
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c"])
        return m

    def distribute_to_vertices_and_edges(self):
        scn = self._ensure_device()
        self._push_dirty()
        scn.distribute(True)
        self._mark_device_newer()

    def update_boundary(self):
        scn = self._ensure_device()
        self._push_dirty()
        if not self._device_loop_ok():
            self._bind_boundaries(self.get_time())
        scn.update_boundary(self.relative_time)
        self._mark_device_newer(["stage_b", "xmom_b", "ymom_b"])

    def compute_fluxes(self):
        scn = self._ensure_device()
        self._push_dirty()
        substep = getattr(self, "_substep", 0)
        self.flux_timestep = scn.compute_fluxes(substep)
        self._mark_device_newer(["stage_x", "xmom_x", "ymom_x", "max_speed"])

    def compute_forcing_terms(self):
        scn = self._ensure_device()
        for f in self.forcing_terms:
            if f is manning_friction_implicit:
                self._push_dirty()
                scn.compute_forcing()
                self._mark_device_newer(["xmom_s", "ymom_s"])
            else:
                f(self)

    def apply_protection_against_isolated_degenerate_timesteps(self):
        """generic_domain.py:2520-2560: when the speed histogram (10 bins from
        the minimum to the maximum speed) has cells in its top bin and none in
        bins 4-8, the momenta of the cells above the top bin's edge are set
        to zero.  Evaluated on the host from the device's max speeds."""
        if self.protect_against_isolated_degenerate_timesteps is False:
            return
        speed = self.max_speed
        if np.max(speed) < 10.0:
            return
        mx, mn = max(speed), min(speed)
        bins = np.array([mn]) if mx == mn else np.arange(mn, mx, (mx - mn) / 10)
        n = np.concatenate([np.searchsorted(np.sort(speed), bins), [len(speed)]], axis=0)
        hist = n[1:] - n[:-1]
        if len(hist) > 1 and hist[-1] > 0 and hist[4] == hist[5] == hist[6] == hist[7] == hist[8] == 0:
            idx = np.nonzero(speed > bins[-1])[0]
            for q in ("xmomentum", "ymomentum"):
                c = self.quantities[q].centroid_values
                c[idx] = 0.0
                self._host_modified(DEVICE_FIELDS[q][0])
            speed[idx] = 0.0          # the host's view only: the next flux call recomputes them

    def update_timestep(self, yieldstep, finaltime):
        """generic_domain.py:2349-2415."""
        self.apply_protection_against_isolated_degenerate_timesteps()
        if self.fixed_flux_timestep is not None:
            self.flux_timestep = self.fixed_flux_timestep
        timestep = min(self.CFL * self.flux_timestep, self.evolve_max_timestep)
        self.recorded_max_timestep = max(timestep, self.recorded_max_timestep)
        self.recorded_min_timestep = min(timestep, self.recorded_min_timestep)
        if timestep < self.evolve_min_timestep:
            self.smallsteps = getattr(self, "smallsteps", 0) + 1
            if self.smallsteps > self.max_smallsteps:
                self.smallsteps = 0
                if self._order_ == 1:
                    raise RuntimeError("WARNING: Too small timestep %.16f reached even after %d steps "
                                       "of 1 order scheme" % (timestep, self.max_smallsteps))
                self._order_ = 1
        else:
            self.smallsteps = 0
            if self._order_ == 1 and self.default_order == 2:
                self._order_ = 2
        rf = getattr(self, "relative_finaltime", None)
        if rf is not None and self.relative_time + timestep > rf:
            timestep = rf - self.relative_time
        if self.relative_time + timestep > self.relative_yieldtime:
            timestep = self.relative_yieldtime - self.relative_time
        self.timestep = timestep

    def update_conserved_quantities(self):
        scn = self._ensure_device()
        self._push_dirty()
        n = scn.update_conserved(self.timestep)
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c", "stage_s", "xmom_s", "ymom_s"])
        if n > 0:
            warnings.warn("Negative cells being set to zero depth, possible loss of conservation.")
        return n

    def backup_conserved_quantities(self):
        scn = self._ensure_device()
        self._push_dirty()
        scn.backup()

    def saxpy_conserved_quantities(self, a, b):
        scn = self._ensure_device()
        self._push_dirty()
        scn.saxpy(a, b)
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c"])

    def apply_fractional_steps(self):
        for op in self.fractional_step_operators:
            op()

    def evolve_one_euler_step(self, yieldstep, finaltime):
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 0
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()

    def evolve_one_rk2_step(self, yieldstep, finaltime):
        self.backup_conserved_quantities()
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 0
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()
        self.set_relative_time(self.get_relative_time() + self.timestep)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 1
        self.compute_fluxes()
        self._substep = 0
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy_conserved_quantities(0.5, 0.5)

    def evolve_one_rk3_step(self, yieldstep, finaltime):
        """generic_domain.py:2053-2172: Q1 = E(dt) Q0; Q2 = 0.25 E(dt) Q1 + 0.75 Q0
        (at t + dt/2); Q = (2 E(dt) Q2 + Q0) / 3."""
        initial_time = self.get_relative_time()
        self.backup_conserved_quantities()
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 0
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()
        self.set_relative_time(self.relative_time + self.timestep)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 1
        self.compute_fluxes()
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy_conserved_quantities(0.25, 0.75)
        self.set_relative_time(initial_time + self.timestep * 0.5)
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self._substep = 2
        self.compute_fluxes()
        self._substep = 0
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy_conserved_quantities(2.0, 1.0)
        scn = self._ensure_device()
        scn.divide(3.0)
        self._mark_device_newer(["stage_c", "xmom_c", "ymom_c"])
        self.set_relative_time(initial_time + self.timestep)

    # ------------------------------------------------------------------
    # time stepping
    def _device_steps(self, max_steps=0):
        scn = self._scn
        self._push_dirty()
        rf = self.relative_finaltime if getattr(self, "relative_finaltime", None) is not None else -1.0
        scn.set_clock(self.relative_time, self.relative_yieldtime, rf)
        st = scn.advance(max_steps)
        return self._take_stats(st)

    def _take_stats(self, st):
        self._mark_device_newer()
        self.relative_time = st.time
        self.timestep = st.last_timestep
        self.flux_timestep = st.flux_timestep
        self.number_of_steps += st.steps
        self.total_steps += st.steps
        self.recorded_min_timestep = min(self.recorded_min_timestep, st.min_timestep)
        self.recorded_max_timestep = max(self.recorded_max_timestep, st.max_timestep)
        self.boundary_flux_sum = np.array(st.boundary_flux_sum[:])
        self._order_ = st.order
        self._last_stats = st
        return st.reason

    def _host_step_mixed(self):
        """One step of the mixed form when a boundary or an operator is a
        Python function of time: boundary values evaluated at the step's start
        time for the first stage, at t + dt for the second and (rk3) at
        t + dt/2 for the third (as generic_domain.py:1974-2172), then every
        operator applied in registration order with the step's timestep, at
        the time the reference's operators see (the step's start for Euler,
        its end otherwise)."""
        if any(f is not manning_friction_implicit for f in self.forcing_terms):
            raise NotImplementedError("the mixed form applies Manning friction only; other forcing terms run "
                                      "on precision='fp64'")
        scn = self._scn
        t0 = self.relative_time
        self._push_dirty()
        host_bc = any(B is not None and not getattr(B, "device_loop", True) for B in self.boundary_map.values())
        if host_bc:
            self._bind_boundaries(self.get_time())
        rf = self.relative_finaltime if getattr(self, "relative_finaltime", None) is not None else -1.0
        scn.set_clock(t0, self.relative_yieldtime, rf)
        dt = scn.step_begin()
        if host_bc and self.timestepping_method != "euler":
            self._bind_boundaries(self.starttime + t0 + dt)
            if self.timestepping_method == "rk3":
                scn.step_stage(2)
                self._bind_boundaries(self.starttime + t0 + dt * 0.5)
        reason = self._take_stats(scn.step_end())
        t1 = self.relative_time
        if self.timestepping_method == "euler":
            self.relative_time = t0
        for op in self.fractional_step_operators:
            if op is not self.boundary_flux_integral:     # integrated by the device clock
                op()
        self.relative_time = t1
        return 0 if reason == _lib.STOP_MAXSTEPS else reason

    def _host_step(self, yieldstep, finaltime):
        if self.precision == "mixed":
            return self._host_step_mixed()
        t0 = self.relative_time
        if self.timestepping_method == "euler":
            self.evolve_one_euler_step(yieldstep, finaltime)
        elif self.timestepping_method == "rk3":
            self.evolve_one_rk3_step(yieldstep, finaltime)
        else:
            self.evolve_one_rk2_step(yieldstep, finaltime)
        # operators: device ones through the library in one shot
        for op in self.fractional_step_operators:
            op()
        self.relative_time = t0 + self.timestep
        self.number_of_steps += 1
        self.total_steps += 1
        rf = getattr(self, "relative_finaltime", None)
        if rf is not None and self.relative_time >= rf - EPSILON:
            if self.relative_time > rf:
                raise RuntimeError("WARNING (domain.py): time overshot finaltime. ")
            self.relative_time = rf
            return _lib.STOP_FINAL
        if self.relative_time >= self.relative_yieldtime:
            return _lib.STOP_YIELD
        return 0

    def evolve(self, yieldstep=None, outputstep=None, finaltime=None, duration=None,
               skip_initial_step=False):
        """Generator as in shallow_water_domain.py:2300-2407 / generic_domain.py:1715-1912."""
        if finaltime is not None:
            finaltime = float(finaltime)
        if outputstep is None:
            outputstep = yieldstep
        if yieldstep is None:
            self.output_frequency = 1
        else:
            of = outputstep / yieldstep
            if not float(of).is_integer():
                raise ValueError("outputstep (%s) should be an integer multiple of yieldstep (%s)"
                                 % (outputstep, yieldstep))
            self.output_frequency = int(of)
        if not (0 <= self.beta_w <= 2.0):
            raise ValueError("Attribute self.beta_w must be in the interval [0, 2]")
        self._ensure_device()
        self.distribute_to_vertices_and_edges()
        if self.store and (self.relative_time == 0.0 or not self.evolved_called):
            self._initialise_storage()
        try:
            for t in self._evolve_base(yieldstep, finaltime, duration, skip_initial_step):
                if self.store and self.yieldstep_counter % self.output_frequency == 0:
                    self.store_timestep()
                if getattr(self, "checkpoint", False):
                    self._maybe_checkpoint()
                yield t
                self.yieldstep_counter += 1
        finally:
            self.flush_sww()

    # ------------------------------------------------------------------
    # checkpoint / resume (shallow_water_domain.py:1123-1157, :2376-2397;
    # shallow_water/checkpoint.py)
    def set_checkpointing(self, checkpoint=True, checkpoint_dir="CHECKPOINTS", checkpoint_step=10,
                          checkpoint_time=None):
        """Pickle the domain every ``checkpoint_step`` yieldsteps, or every
        ``checkpoint_time`` wall-clock seconds if that is given, into
        ``checkpoint_dir/<name>_<time>.pickle``; ``load_checkpoint_file``
        restores it."""
        if not checkpoint:
            self.checkpoint = False
            return
        os.makedirs(checkpoint_dir, exist_ok=True)
        self.checkpoint_dir = checkpoint_dir
        if checkpoint_time is not None:
            self.walltime_prev = time.time()
            self.checkpoint_time = checkpoint_time
            self.checkpoint_step = 0
        else:
            self.checkpoint_step = checkpoint_step
        self.checkpoint = True

    def _maybe_checkpoint(self):
        if self.checkpoint_step == 0:
            save = time.time() - self.walltime_prev > self.checkpoint_time
        else:
            save = self.yieldstep_counter % self.checkpoint_step == 0
        if save:
            name = os.path.join(self.checkpoint_dir, self.get_name()) + "_" + str(self.get_time()) + ".pickle"
            with open(name, "wb") as fh:
                pickle.dump(self, fh)
            self.walltime_prev = time.time()

    def __getstate__(self):
        """The host state with every device field pulled; the device handle is
        left out and made again (with the fields uploaded) on first use."""
        if self._scn is not None:
            self._pull([f for f in self._fstate])
        state = self.__dict__.copy()
        state["_scn"] = None
        state["_scn_key"] = None
        state["_fstate"] = {f: _SYNCED for f in self._fstate}
        return state

    def __setstate__(self, state):
        self.__dict__.update(state)

    def _evolve_base(self, yieldstep, finaltime, duration, skip_initial_step):
        if self.boundary_map is None:
            raise RuntimeError("Boundary tags must be bound to boundary objects before evolving system, "
                               "e.g. using the method set_boundary. This system has the boundary tags %s"
                               % self.get_boundary_tags())
        if self.evolved_called:
            skip_initial_step = True
        self.evolved_called = True
        if skip_initial_step:
            self.evolve_starttime = self.relative_time
        if self.relative_time != self.evolve_starttime:
            self.relative_time = self.evolve_starttime
        yieldstep = self.evolve_max_timestep if yieldstep is None else float(yieldstep)
        self.yieldstep = yieldstep
        self._order_ = self.default_order
        if finaltime is not None and duration is not None:
            raise ValueError("Only one of finaltime and duration may be specified")
        self.relative_finaltime = getattr(self, "relative_finaltime", None)
        if finaltime is not None:
            self.finaltime = float(finaltime)
            self.relative_finaltime = self.finaltime - self.starttime
        if duration is not None:
            self.finaltime = float(duration) + self.get_time()
            self.relative_finaltime = float(duration) + self.relative_time
        if self.relative_finaltime is not None and self.relative_finaltime < self.relative_time:
            warnings.warn("finaltime %g is less than current time %g! finaltime set to current time"
                          % (self.relative_finaltime + self.starttime, self.get_time()))
            self.relative_finaltime = self.relative_time
            return
        self.relative_yieldtime = self.relative_time + yieldstep
        self.recorded_min_timestep = self.evolve_max_timestep
        self.recorded_max_timestep = self.evolve_min_timestep
        self.number_of_steps = 0
        self.number_of_first_order_steps = 0
        if not skip_initial_step:
            self.distribute_to_vertices_and_edges()
            self.update_boundary()
            self._pull(_STATE_FIELDS)
            yield self.get_time()
        device_loop = self._device_loop_ok()
        if self.precision == "mixed":
            self._scn.operators_from_host(not device_loop)
        while True:
            if device_loop:
                reason = self._device_steps()
            else:
                reason = self._host_step(yieldstep, self.relative_finaltime)
                while reason == 0:
                    reason = self._host_step(yieldstep, self.relative_finaltime)
            if reason == _lib.STOP_FINAL:
                self.relative_time = self.relative_finaltime
                self.distribute_to_vertices_and_edges()
                self.update_boundary()
                self._pull(_STATE_FIELDS)
                yield self.get_time()
                break
            if reason == _lib.STOP_YIELD:
                self.distribute_to_vertices_and_edges()
                self.update_boundary()
                self._pull(_STATE_FIELDS)
                yield self.get_time()
                self.relative_yieldtime += yieldstep
                self.recorded_min_timestep = self.evolve_max_timestep
                self.recorded_max_timestep = self.evolve_min_timestep
                self.number_of_steps = 0
                self.number_of_first_order_steps = 0
                continue
            raise RuntimeError("device step loop stopped unexpectedly (reason %d)" % reason)

    def advance_steps(self, n):
        """Advance exactly n timesteps on the device with no yield or final
        time (the fixed-step form used for throughput measurement)."""
        self._ensure_device()
        if not self._device_loop_ok():
            raise RuntimeError("advance_steps needs device-evaluable boundaries and operators")
        self.relative_yieldtime = float("inf")
        self.relative_finaltime = None
        reason = self._device_steps(max_steps=int(n))
        if reason not in (_lib.STOP_MAXSTEPS,):
            raise RuntimeError("advance_steps stopped early (reason %d)" % reason)
        return self._last_stats

    # ------------------------------------------------------------------
    # statistics and output
    @property
    def max_speed(self):
        self._pull(["max_speed"])
        return self._farr["max_speed"]

    def get_water_volume(self):
        """Volume of water, sum of area x depth over the cells (and
        appended to volume_history, shallow_water_domain.py:1630-1675)."""
        Q = self.quantities
        h = np.maximum(Q["stage"].centroid_values - Q["elevation"].centroid_values, 0.0)
        volume = float(np.sum(self.mesh.areas * h))
        self.volume_history.append(volume)
        return volume

    def get_boundary_flux_integral(self):
        """Time integral of the flux through the boundaries since the start
        (shallow_water_domain.py:1677-1700): positive for water that entered."""
        return self.boundary_flux_integral.get_integral()

    def get_fractional_step_volume_integral(self):
        """Volume the fractional-step operators (rates, inlets) have added
        (shallow_water_domain.py:1715-1745)."""
        total = 0.0
        for op in self.fractional_step_operators:
            if hasattr(op, "get_Q"):
                total += op.get_Q()
            elif hasattr(op, "get_total_applied_volume"):
                total += op.get_total_applied_volume()
        return total

    def report_water_volume_statistics(self, verbose=True, returnStats=False):
        """Volume, boundary flux integral, fractional-step volume and their
        balance against the first recorded volume (shallow_water_domain.py:2749-2781)."""
        if not self.volume_history:
            raise RuntimeError("call get_water_volume() at the start of the run first: the balance is "
                               "taken against the first recorded volume")
        vol = self.get_water_volume()
        flux = self.get_boundary_flux_integral()
        frac = self.get_fractional_step_volume_integral()
        if verbose:
            print(" ")
            print("    Volume V is:", vol)
            print("    Boundary Flux integral BF: ", flux)
            print("    (rate + inlet) Fractional Step volume integral FS: ", frac)
            print("    V - BF - FS - InitialVolume :", vol - flux - frac - self.volume_history[0])
            print(" ")
        if returnStats:
            return [vol, flux, frac]

    def timestepping_statistics(self):
        return ("Time = %.4f, delta t in [%.8f, %.8f], steps=%d"
                % (self.get_time(), self.recorded_min_timestep, self.recorded_max_timestep,
                   self.number_of_steps))

    def print_timestepping_statistics(self):
        print(self.timestepping_statistics())

    def _initialise_storage(self):
        from .sww import SWW_file
        self.writer = SWW_file(self)
        self.writer.store_connectivity()

    def store_timestep(self):
        if self.writer is not None:
            self.writer.store_timestep()

    def flush_sww(self):
        """Wait until the sww frames started so far are in the file (the
        frames are copied and written while the next yieldstep runs)."""
        if self.writer is not None:
            self.writer.flush()


def rectangular_cross_domain(*args, **kwargs):
    """anuga.rectangular_cross_domain (anuga/extras.py:13-46)."""
    verbose = kwargs.pop("verbose", False)
    points, vertices, boundary = rectangular_cross(*args, **kwargs)
    return Domain(points, vertices, boundary, verbose=verbose)
