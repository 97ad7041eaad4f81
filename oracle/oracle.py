"""Python driver for the CPU oracle (test infrastructure only).

Wraps ``liborc.so`` (oracle/de_oracle.c) with ctypes and runs the reference's
time-stepping loop around it.  Used by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of bench.py as the parity checker; never by the product.

The loop mirrors the reference:

* ``_evolve_base``            abstract_2d_finite_volumes/generic_domain.py:1715-1912
* ``evolve_one_euler_step``   generic_domain.py:1914-1972
* ``evolve_one_rk2_step``     generic_domain.py:1974-2051
* ``evolve_one_rk3_step``     generic_domain.py:2053-2172
* ``update_timestep``         generic_domain.py:2349-2415
* ``update_conserved_quantities`` shallow_water/shallow_water_domain.py:2089-2163
* ``Rate_operator.__call__``  operators/rate_operators.py:149-258 (constant rates)
* ``Inlet_operator.__call__`` structures/inlet_operator.py:75-165 with
  structures/inlet.py:107-226 (constant discharge)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")

EPSILON = 1.0e-12   # anuga/config.py epsilon


def build(force=False):
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
            os.path.join(HERE, "de_oracle.c")):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)


class _OrcDomain(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int64), ("B", ctypes.c_int64),
        ("g", ctypes.c_double), ("epsilon", ctypes.c_double),
        ("minimum_allowed_height", ctypes.c_double), ("H0", ctypes.c_double),
        ("beta_w", ctypes.c_double), ("beta_w_dry", ctypes.c_double),
        ("beta_uh", ctypes.c_double), ("beta_uh_dry", ctypes.c_double),
        ("beta_vh", ctypes.c_double), ("beta_vh_dry", ctypes.c_double),
        ("extrapolate_velocity_second_order", ctypes.c_int64),
        ("low_froude", ctypes.c_int64),
        ("ncol_riverwall_hydraulic_properties", ctypes.c_int64),
        ("neighbours", _ip), ("neighbour_edges", _ip), ("surrogate_neighbours", _ip),
        ("number_of_boundaries", _ip), ("tri_full_flag", _ip),
        ("normals", _dp), ("edgelengths", _dp), ("radii", _dp), ("areas", _dp),
        ("edge_coordinates", _dp), ("centroid_coordinates", _dp),
        ("edge_flux_type", _ip), ("edge_river_wall_counter", _ip), ("riverwall_rowIndex", _ip),
        ("riverwall_elevation", _dp), ("riverwall_hydraulic_properties", _dp),
        ("stage_c", _dp), ("xmom_c", _dp), ("ymom_c", _dp), ("bed_c", _dp), ("height_c", _dp),
        ("stage_e", _dp), ("xmom_e", _dp), ("ymom_e", _dp), ("bed_e", _dp), ("height_e", _dp),
        ("stage_v", _dp), ("xmom_v", _dp), ("ymom_v", _dp), ("bed_v", _dp), ("height_v", _dp),
        ("stage_b", _dp), ("xmom_b", _dp), ("ymom_b", _dp),
        ("stage_x", _dp), ("xmom_x", _dp), ("ymom_x", _dp),
        ("stage_s", _dp), ("xmom_s", _dp), ("ymom_s", _dp),
        ("max_speed", _dp), ("x_work", _dp), ("y_work", _dp),
        ("boundary_flux_sum", _dp),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_protect.restype = ctypes.c_double
        L.orc_protect.argtypes = [ctypes.POINTER(_OrcDomain), ctypes.c_int]
        L.orc_extrapolate.restype = ctypes.c_int
        L.orc_extrapolate.argtypes = [ctypes.POINTER(_OrcDomain)]
        L.orc_compute_fluxes.restype = ctypes.c_double
        L.orc_compute_fluxes.argtypes = [ctypes.POINTER(_OrcDomain), ctypes.c_int64, ctypes.c_double]
        L.orc_manning_flat.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int64] + [_dp] * 7
        L.orc_manning_sloped.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int64] + [_dp] * 8
        L.orc_update.restype = ctypes.c_int
        L.orc_update.argtypes = [ctypes.c_int64, ctypes.c_double, _dp, _dp, _dp]
        L.orc_fix_negative.restype = ctypes.c_int64
        L.orc_fix_negative.argtypes = [ctypes.POINTER(_OrcDomain)]
        L.orc_backup.argtypes = [ctypes.c_int64, _dp, _dp]
        L.orc_saxpy.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_double, _dp, _dp]
        L.orc_bc_reflective.argtypes = [ctypes.POINTER(_OrcDomain), _ip, ctypes.c_int64, _ip, _ip]
        L.orc_bc_transmissive.argtypes = [ctypes.POINTER(_OrcDomain), _ip, ctypes.c_int64, _ip, _ip, ctypes.c_int]
        L.orc_bc_dirichlet.argtypes = [ctypes.POINTER(_OrcDomain), _ip, ctypes.c_int64] + [ctypes.c_double] * 3
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_set_parallel_extrapolation.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n):
    lib().orc_set_threads(int(n))


def set_parallel_extrapolation(on):
    """Timing mode: parallel extrapolation loop like the reference's OpenMP
    build (order-dependent at chunk boundaries); parity runs leave it off."""
    lib().orc_set_parallel_extrapolation(1 if on else 0)


def _p(a):
    if a is None:
        return None
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    return a.ctypes.data_as(_ip)


# Algorithm defaults, shallow_water/shallow_water_domain.py:583-877
FLOW_DEFAULTS = {
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


class OracleDomain:
    """A DE-family domain (DE0, DE1, DE2, DE0_7, DE1_7) advanced by the CPU oracle.

    ``mesh`` is any object with the reference's mesh attributes (the
    product's ``anuga_core_gb300.mesh.Mesh`` or a reference ``Domain``).
    ``boundaries`` is a list of ``(ids, kind, values)`` with kind in
    ``reflective``, ``transmissive``, ``transmissive_centroid``,
    ``dirichlet``.  ``rates`` is a list of ``(indices or None, rate, factor)``.
    """

    def __init__(self, mesh, flow_algorithm="DE0", protect_zero_ymom=False,
                 use_sloped_mannings=False, low_froude=0, g=9.8):
        N = len(mesh)
        self.N = N
        self.B = B = int(mesh.boundary_length)
        d = FLOW_DEFAULTS[flow_algorithm]
        self.flow_algorithm = flow_algorithm
        self.CFL = d["CFL"]
        self.timestepping_method = d["timestepping_method"]
        self.timestep_fluxcalls = {"euler": 1, "rk2": 2, "rk3": 3}[self.timestepping_method]
        self.evolve_max_timestep = 1.0e3    # anuga/config.py max_timestep
        self.evolve_min_timestep = 1.0e-6   # anuga/config.py min_timestep
        self.max_smallsteps = 50
        self.protect_zero_ymom = protect_zero_ymom
        self.use_sloped_mannings = use_sloped_mannings
        c = lambda a, t=np.float64: np.ascontiguousarray(a, dtype=t)
        self.neighbours = c(mesh.neighbours, np.int64).ravel()
        self.neighbour_edges = c(mesh.neighbour_edges, np.int64).ravel()
        self.surrogate_neighbours = c(mesh.surrogate_neighbours, np.int64).ravel()
        self.number_of_boundaries = c(mesh.number_of_boundaries, np.int64)
        self.tri_full_flag = np.ones(N, np.int64)
        self.normals = c(mesh.normals).ravel()
        self.edgelengths = c(mesh.edgelengths).ravel()
        self.radii = c(mesh.radii)
        self.areas = c(mesh.areas)
        self.edge_coordinates = c(mesh.edge_midpoint_coordinates).ravel()
        self.centroid_coordinates = c(mesh.centroid_coordinates).ravel()
        self.vertex_coordinates = c(mesh.vertex_coordinates).ravel()
        self.boundary_cells = c(mesh.boundary_cells, np.int64)
        self.boundary_edges = c(mesh.boundary_edges, np.int64)
        z = lambda n: np.zeros(n, np.float64)
        for q in ("stage", "xmom", "ymom", "bed", "height"):
            setattr(self, q + "_c", z(N))
            setattr(self, q + "_e", z(3 * N))
            setattr(self, q + "_v", z(3 * N))
        for q in ("stage", "xmom", "ymom"):
            setattr(self, q + "_b", z(B))
            setattr(self, q + "_x", z(N))
            setattr(self, q + "_s", z(N))
            setattr(self, q + "_0", z(N))
        self.friction_c = z(N)
        self.max_speed = z(N)
        self.x_work = z(N)
        self.y_work = z(N)
        self.boundary_flux_sum = z(3)
        self.D = D = _OrcDomain()
        D.N, D.B = N, B
        D.g, D.epsilon = g, EPSILON
        D.minimum_allowed_height = d["minimum_allowed_height"]
        D.H0 = 1.0e-5
        for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
            setattr(D, k, d[k])
        D.extrapolate_velocity_second_order = 1
        D.low_froude = low_froude
        for name in ("neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
                     "tri_full_flag", "normals", "edgelengths", "radii", "areas", "edge_coordinates",
                     "centroid_coordinates", "stage_c", "xmom_c", "ymom_c", "bed_c", "height_c",
                     "stage_e", "xmom_e", "ymom_e", "bed_e", "height_e", "stage_v", "xmom_v",
                     "ymom_v", "bed_v", "height_v", "stage_b", "xmom_b", "ymom_b", "stage_x",
                     "xmom_x", "ymom_x", "stage_s", "xmom_s", "ymom_s", "max_speed", "x_work",
                     "y_work", "boundary_flux_sum"):
            setattr(D, name, _p(getattr(self, name)))
        self.Dp = ctypes.pointer(D)
        self.boundaries = []
        self.rates = []
        self.inlets = []
        self.ops = []              # operators in registration order
        self.relative_time = 0.0
        self.starttime = 0.0
        self.timestep = 0.0
        self.flux_timestep = 0.0
        self.smallsteps = 0
        self._order_ = 2
        self.default_order = 2
        self.number_of_steps = 0
        self.total_steps = 0
        self.evolved_called = False
        self.timesteps = []
        self.negative_cells = 0

    @property
    def minimum_allowed_height(self):
        return self.D.minimum_allowed_height

    # --- state -------------------------------------------------------------
    def set_centroid_state(self, stage, xmom, ymom, elevation, friction):
        self.stage_c[:] = stage
        self.xmom_c[:] = xmom
        self.ymom_c[:] = ymom
        self.bed_c[:] = elevation
        self.friction_c[:] = friction

    def set_bed_vertex_values(self, zv):
        self.bed_v[:] = np.asarray(zv, np.float64).ravel()

    def set_riverwalls(self, edge_flux_type, edge_river_wall_counter, riverwall_elevation,
                       hydraulic_properties_rowIndex, hydraulic_properties):
        """Riverwall tables in the reference's layout (structures/riverwall.py)."""
        c = lambda a, t=np.float64: np.ascontiguousarray(a, dtype=t).ravel()
        self.rw = dict(flux_type=c(edge_flux_type, np.int64), counter=c(edge_river_wall_counter, np.int64),
                       row=c(hydraulic_properties_rowIndex, np.int64), elevation=c(riverwall_elevation),
                       hyd=c(hydraulic_properties))
        D = self.D
        D.edge_flux_type = self.rw["flux_type"].ctypes.data_as(_ip)
        D.edge_river_wall_counter = self.rw["counter"].ctypes.data_as(_ip)
        D.riverwall_rowIndex = self.rw["row"].ctypes.data_as(_ip)
        D.riverwall_elevation = _p(self.rw["elevation"])
        D.riverwall_hydraulic_properties = _p(self.rw["hyd"])
        D.ncol_riverwall_hydraulic_properties = np.asarray(hydraulic_properties).shape[-1]

    def set_boundaries(self, boundaries):
        self.boundaries = [(np.ascontiguousarray(ids, np.int64), kind, vals)
                           for ids, kind, vals in boundaries]

    def add_rate(self, indices, rate, factor=1.0):
        idx = None if indices is None else np.asarray(indices, np.int64)
        self.rates.append([idx, float(rate), float(factor), 0.0])
        self.ops.append(("rate", self.rates[-1]))

    def add_inlet(self, indices, Q, velocity=None, zero_velocity=False):
        """Inlet_operator (structures/inlet_operator.py:17-165): discharge Q
        (constant, m^3/s) into the cells `indices`."""
        idx = np.asarray(indices, np.int64)
        rec = dict(idx=idx, Q=float(Q), velocity=velocity, zero_velocity=bool(zero_velocity),
                   area=float(np.sum(self.areas[idx])), applied=0.0)
        self.inlets.append(rec)
        self.ops.append(("inlet", rec))

    # inlet_operator.py:75-165 with inlet.py:107-226 (set_stages_evenly,
    # set_depths, get_velocities; velocity_protection = 1e-6, config.py:18)
    def _apply_inlet(self, r):
        idx = r["idx"]
        areas = self.areas[idx]
        stages = self.stage_c[idx]
        elev = self.bed_c[idx]
        depths = stages - elev
        current_volume = np.sum(depths * areas)
        total_area = r["area"]
        Q = 0.5 * (r["Q"] + r["Q"])
        volume = Q * self.timestep
        u = self.xmom_c[idx] * depths / (depths * depths + 1.0e-6)
        v = self.ymom_c[idx] * depths / (depths * depths + 1.0e-6)
        if volume >= 0.0:
            order = stages.argsort()
            summed_areas = np.cumsum(areas[order])
            summed_volume = np.zeros_like(areas)
            summed_volume[1:] = np.cumsum(summed_areas[:-1] * np.diff(stages[order]))
            index = np.nonzero(summed_volume <= volume)[0][-1]
            depth = (volume - summed_volume[index]) / summed_areas[index]
            new = stages.copy()
            new[order[0:index + 1]] = stages[order[index]] + depth
            self.stage_c[idx] = new
        elif current_volume + volume >= 0.0:
            depth = (current_volume + volume) / total_area
            self.stage_c[idx] = elev + depth
        else:
            self.stage_c[idx] = elev
            self.xmom_c[idx] = 0.0
            self.ymom_c[idx] = 0.0
            r["applied"] += -current_volume
            return
        d_new = self.stage_c[idx] - elev
        if r["velocity"] is not None:
            self.xmom_c[idx] = d_new * r["velocity"][0]
            self.ymom_c[idx] = d_new * r["velocity"][1]
        else:
            self.xmom_c[idx] = d_new * u
            self.ymom_c[idx] = d_new * v
        if r["zero_velocity"]:
            self.xmom_c[idx] = 0.0
            self.ymom_c[idx] = 0.0
        r["applied"] += volume

    # --- phases ------------------------------------------------------------
    def protect(self):
        return lib().orc_protect(self.Dp, 1 if self.protect_zero_ymom else 0)

    def extrapolate(self):
        lib().orc_extrapolate(self.Dp)

    def distribute_to_vertices_and_edges(self):
        m = self.protect()
        self.extrapolate()
        return m

    def update_boundary(self):
        L = lib()
        for ids, kind, vals in self.boundaries:
            if kind == "reflective":
                L.orc_bc_reflective(self.Dp, _p(ids), ids.size, _p(self.boundary_cells), _p(self.boundary_edges))
            elif kind in ("transmissive", "transmissive_centroid"):
                L.orc_bc_transmissive(self.Dp, _p(ids), ids.size, _p(self.boundary_cells),
                                      _p(self.boundary_edges), 1 if kind == "transmissive_centroid" else 0)
            elif kind == "dirichlet":
                w, uh, vh = (float(v) for v in vals)
                L.orc_bc_dirichlet(self.Dp, _p(ids), ids.size, w, uh, vh)
            else:
                self._bc_numpy(ids, kind, vals)

    def _stage_of(self, f):
        # a function of time giving the stage (or a vector whose first entry is)
        v = f(self.starttime + self.relative_time) if callable(f) else f
        try:
            return float(v)
        except TypeError:
            return float(v[0])

    def _bc_numpy(self, ids, kind, vals):
        """The stage/momentum boundaries of shallow_water/boundaries.py,
        restated on the boundary slots ``ids``."""
        k = self.boundary_cells[ids]
        e = self.boundary_edges[ids]
        s = 3 * k + e
        n1 = self.normals[2 * s]
        n2 = self.normals[2 * s + 1]
        if kind == "transmissive_set_stage":      # boundaries.py:295-383
            self.stage_b[ids] = self._stage_of(vals)
            self.xmom_b[ids] = self.xmom_e[s]
            self.ymom_b[ids] = self.ymom_e[s]
        elif kind == "transmissive_zero_momentum":  # boundaries.py:520-552
            self.stage_b[ids] = self.stage_e[s]
            self.xmom_b[ids] = 0.0
            self.ymom_b[ids] = 0.0
        elif kind == "time_stage_zero_momentum":  # boundaries.py:553-638 (stage f(t), momenta 0)
            self.stage_b[ids] = self._stage_of(vals)
            self.xmom_b[ids] = 0.0
            self.ymom_b[ids] = 0.0
        elif kind == "dirichlet_discharge":       # boundaries.py:850-901
            stage0, wh0 = vals
            self.stage_b[ids] = stage0
            self.xmom_b[ids] = -wh0 * n1
            self.ymom_b[ids] = -wh0 * n2
        elif kind == "flather":                   # boundaries.py:1242-1330
            stage_outside = self._stage_of(vals)
            w_in, q1, q2 = self.stage_e[s], self.xmom_e[s], self.ymom_e[s]
            z_edge = self.bed_e[s]
            bed = self.bed_c[k]
            depth_inside = np.maximum(w_in - bed, 0.0)
            stage_out = 0.0 * w_in + stage_outside
            q0_dry = np.where(bed <= stage_out, stage_out, z_edge)
            with np.errstate(divide="ignore", invalid="ignore"):
                sg = (self.D.g / depth_inside) ** 0.5
                ndotq = n1 * q1 + n2 * q2
                w1 = 0.0 - sg * stage_out
                w2 = np.where(ndotq > 0.0, (n2 * q1 - n1 * q2) / depth_inside, 0.0 * ndotq)
                w3 = ndotq / depth_inside + sg * w_in
                q0_wet = (w3 - w1) / (2.0 * sg)
                qperp = (w3 + w1) / 2.0 * depth_inside
                qpar = w2 * depth_inside
                q1_wet = qperp * n1 + qpar * n2
                q2_wet = qperp * n2 - qpar * n1
            dry = np.logical_or(depth_inside == 0.0, stage_out > bed)
            self.stage_b[ids] = np.where(dry, q0_dry, q0_wet)
            self.xmom_b[ids] = np.where(dry, 0.0 * q1, q1_wet)
            self.ymom_b[ids] = np.where(dry, 0.0 * q2, q2_wet)
        elif kind == "inflow":                    # boundaries.py:902-992 (slope 0: depth 1)
            rate = float(vals)
            length = 0.0
            for j in range(len(ids)):
                length += self.edgelengths[s[j]]
            mu = rate / length
            self.stage_b[ids] = self.bed_e[s] + 1.0
            self.xmom_b[ids] = mu * (-n1)
            self.ymom_b[ids] = mu * (-n2)
        elif kind == "time_space":                # generic_boundary_conditions.py:419-517
            t = self.starttime + self.relative_time
            x = self.edge_coordinates[2 * s]
            y = self.edge_coordinates[2 * s + 1]
            for j in range(len(ids)):
                q = np.asarray(vals(t, x[j], y[j]), float).ravel()
                self.stage_b[ids[j]], self.xmom_b[ids[j]], self.ymom_b[ids[j]] = q[0], q[1], q[2]
        elif kind == "characteristic":            # boundaries.py:757-848
            w_outside = self._stage_of(vals)
            w_in, q1, q2 = self.stage_e[s], self.xmom_e[s], self.ymom_e[s]
            ze = self.bed_e[s]
            w_out = 0.0 * w_in + w_outside
            sqrt_g = self.D.g ** 0.5
            h_in = np.maximum(w_in - ze, 0)
            uh_in = n1 * q1 + n2 * q2
            vh_in = n2 * q1 - n1 * q2
            with np.errstate(divide="ignore", invalid="ignore"):
                u_in = np.where(h_in > 0.0, uh_in / h_in, 0.0)
            h_out = np.maximum(w_out - ze, 0)
            sh_in = h_in ** 0.5
            sh_out = h_out ** 0.5
            h_m = (0.5 * (sh_in + sh_out) + u_in / 4.0 / sqrt_g) ** 2
            u_m = 0.5 * u_in + sqrt_g * (sh_in - sh_out)
            uh_m = h_m * u_m
            vh_m = np.where(uh_in > 0.0, vh_in, 0.0)
            w_m = h_m + ze
            dry = np.logical_or(h_in == 0.0, h_out == 0.0)
            self.stage_b[ids] = np.where(dry, w_out, w_m)
            self.xmom_b[ids] = np.where(dry, 0.0, uh_m * n1 + vh_m * n2)
            self.ymom_b[ids] = np.where(dry, 0.0, uh_m * n2 - vh_m * n1)
        else:
            raise ValueError("unknown boundary kind %r" % kind)

    def compute_fluxes(self, substep):
        self.flux_timestep = lib().orc_compute_fluxes(self.Dp, substep, self.evolve_max_timestep)
        return self.flux_timestep

    def compute_forcing_terms(self):
        L = lib()
        if self.use_sloped_mannings:
            L.orc_manning_sloped(self.D.g, self.D.minimum_allowed_height, self.N, _p(self.vertex_coordinates),
                                 _p(self.stage_c), _p(self.bed_v), _p(self.xmom_c), _p(self.ymom_c),
                                 _p(self.friction_c), _p(self.xmom_s), _p(self.ymom_s))
        else:
            L.orc_manning_flat(self.D.g, self.D.minimum_allowed_height, self.N, _p(self.stage_c),
                               _p(self.bed_c), _p(self.xmom_c), _p(self.ymom_c), _p(self.friction_c),
                               _p(self.xmom_s), _p(self.ymom_s))

    def update_conserved_quantities(self):
        L = lib()
        for q in ("stage", "xmom", "ymom"):
            err = L.orc_update(self.N, self.timestep, _p(getattr(self, q + "_c")),
                               _p(getattr(self, q + "_x")), _p(getattr(self, q + "_s")))
            if err != 0:
                raise RuntimeError("update: non-positive semi-implicit denominator")
        self.negative_cells += L.orc_fix_negative(self.Dp)

    def backup(self):
        for q in ("stage", "xmom", "ymom"):
            lib().orc_backup(self.N, _p(getattr(self, q + "_c")), _p(getattr(self, q + "_0")))

    def saxpy(self, a, b):
        for q in ("stage", "xmom", "ymom"):
            lib().orc_saxpy(self.N, a, b, _p(getattr(self, q + "_c")), _p(getattr(self, q + "_0")))

    def update_timestep(self, yieldstep, finaltime):
        timestep = min(self.CFL * self.flux_timestep, self.evolve_max_timestep)
        if timestep < self.evolve_min_timestep:
            self.smallsteps += 1
            if self.smallsteps > self.max_smallsteps:
                self.smallsteps = 0
                if self._order_ == 1:
                    raise RuntimeError("Too small timestep %.16f reached" % timestep)
                self._order_ = 1
        else:
            self.smallsteps = 0
            if self._order_ == 1 and self.default_order == 2:
                self._order_ = 2
        if self.relative_finaltime is not None and self.relative_time + timestep > self.relative_finaltime:
            timestep = self.relative_finaltime - self.relative_time
        if self.relative_time + timestep > self.relative_yieldtime:
            timestep = self.relative_yieldtime - self.relative_time
        self.timestep = timestep

    def apply_fractional_steps(self):
        for kind, r in self.ops:
            if kind == "inlet":
                self._apply_inlet(r)
                continue
            idx, rate, factor = r[0], r[1], r[2]
            if rate >= 0.0:
                local = factor * self.timestep * rate
                if idx is None:
                    self.stage_c[:] = self.stage_c[:] + local
                else:
                    self.stage_c[idx] = self.stage_c[idx] + local
            else:
                sel = slice(None) if idx is None else idx
                heights = self.stage_c[sel] - self.bed_c[sel]
                local = np.maximum(factor * self.timestep * rate, -heights)
                fac = np.where(local < 0.0, (local + heights) / (heights + 1.0e-10), 1.0)
                self.stage_c[sel] = self.stage_c[sel] + local
                self.xmom_c[sel] = self.xmom_c[sel] * fac
                self.ymom_c[sel] = self.ymom_c[sel] * fac

    def euler_step(self, yieldstep, finaltime):
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(0)
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()

    def rk2_step(self, yieldstep, finaltime):
        self.backup()
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(0)
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()
        self.relative_time = self.relative_time + self.timestep
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(1)
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy(0.5, 0.5)

    def rk3_step(self, yieldstep, finaltime):
        t0 = self.relative_time
        self.backup()
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(0)
        self.compute_forcing_terms()
        self.update_timestep(yieldstep, finaltime)
        self.update_conserved_quantities()
        self.relative_time = self.relative_time + self.timestep
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(1)
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy(0.25, 0.75)
        self.relative_time = t0 + self.timestep * 0.5
        self.distribute_to_vertices_and_edges()
        self.update_boundary()
        self.compute_fluxes(2)
        self.compute_forcing_terms()
        self.update_conserved_quantities()
        self.saxpy(2.0, 1.0)
        for q in ("stage", "xmom", "ymom"):
            c = getattr(self, q + "_c")
            c[:] = c / 3.0
        self.relative_time = t0 + self.timestep

    def evolve(self, yieldstep=None, finaltime=None, max_steps=None):
        """Generator with the reference's yield semantics; ``max_steps``
        stops after that many steps (the step-count form of the benchmark)."""
        if yieldstep is None:
            yieldstep = self.evolve_max_timestep
        yieldstep = float(yieldstep)
        skip_initial = self.evolved_called
        self.evolved_called = True
        self.relative_finaltime = None if finaltime is None else float(finaltime) - self.starttime
        self.relative_yieldtime = self.relative_time + yieldstep
        self.number_of_steps = 0
        if not skip_initial:
            self.distribute_to_vertices_and_edges()
            self.update_boundary()
            yield self.relative_time
        while True:
            t0 = self.relative_time
            if self.timestepping_method == "euler":
                self.euler_step(yieldstep, finaltime)
            elif self.timestepping_method == "rk3":
                self.rk3_step(yieldstep, finaltime)
            else:
                self.rk2_step(yieldstep, finaltime)
            self.apply_fractional_steps()
            self.relative_time = t0 + self.timestep
            self.timesteps.append(self.timestep)
            self.number_of_steps += 1
            self.total_steps += 1
            if max_steps is not None and self.total_steps >= max_steps:
                self.distribute_to_vertices_and_edges()
                self.update_boundary()
                yield self.relative_time
                return
            if self.relative_finaltime is not None and self.relative_time >= self.relative_finaltime - EPSILON:
                if self.relative_time > self.relative_finaltime:
                    raise RuntimeError("time overshot finaltime")
                self.relative_time = self.relative_finaltime
                self.distribute_to_vertices_and_edges()
                self.update_boundary()
                yield self.relative_time
                return
            if self.relative_time >= self.relative_yieldtime:
                self.distribute_to_vertices_and_edges()
                self.update_boundary()
                yield self.relative_time
                self.relative_yieldtime += yieldstep
                self.number_of_steps = 0
                self.max_speed[:] = 0.0
