"""Fractional-step operators applied after each flow step.

``Rate_operator`` follows operators/rate_operators.py:149-258: after every
full timestep, ``stage_c[idx] += factor * dt * rate`` (with the momentum
scaling branch for negative rates).  ``boundary_flux_integral_operator``
follows operators/boundary_flux_integral_operator.py:20-62: the time
integral of the boundary flux sums, which the Domain creates first.  ``Inlet_operator`` follows
structures/inlet_operator.py:17-165: a discharge Q into an inlet region,
filling its lowest cells to a level surface.  Both run on the device: with
constant values inside the device step loop; given as functions of time, the
host evaluates them once per step and the device applies them.
"""
from __future__ import annotations

import numpy as np

from .geometry import inside_polygon


class Operator:
    def __getstate__(self):
        # a pickled operator (checkpoint) keeps the volume applied so far: the
        # device counters start again from zero when the domain is restored
        state = self.__dict__.copy()
        total = None
        if hasattr(self, "get_Q"):
            total = self.get_Q()
        elif hasattr(self, "get_total_applied_volume"):
            total = self.get_total_applied_volume()
        if total is not None:
            state["_influx_offset"] = float(total)
            if "cumulative_influx" in state:
                state["cumulative_influx"] = 0.0
        return state

    device_loop = True

    def __init__(self, domain):
        self.domain = domain
        domain.fractional_step_operators.append(self)

    def __call__(self):  # host-driven path
        raise NotImplementedError

    def log_timestepping_statistics(self):
        pass


class boundary_flux_integral_operator(Operator):
    """Integral over time of the flux through the domain's boundaries
    (operators/boundary_flux_integral_operator.py:20-62; created by the
    Domain's constructor as shallow_water_domain.py:386-387 does).

    After every step the integral grows by the step's boundary flux sums
    weighted by its stages: dt b0 (euler), dt (b0 + b1) / 2 (rk2),
    dt (b0 + b1 + 4 b2) / 6 (rk3).  Steps whose clock runs on the device
    (the device step loop; every step of the mixed form) are integrated there;
    steps the host drives phase by phase are integrated here, as the
    reference does."""

    device_loop = True

    def __init__(self, domain, description=None, label=None, logging=False, verbose=False):
        super().__init__(domain)
        self.label = label or "boundary_flux_integral"
        self._host = 0.0            # steps integrated on the host, and device totals folded in

    def _device_part(self):
        scn = self.domain._scn
        if scn is None:
            return 0.0
        return float(scn.stats().boundary_flux_integral)

    def fold_device(self):
        """Move the device total into the host part (before the device
        scenario is destroyed)."""
        self._host += self._device_part()

    def get_integral(self):
        return self._host + self._device_part()

    @property
    def boundary_flux_integral(self):
        return np.array([self.get_integral()])

    def __call__(self):
        """A step driven by the host, phase by phase (plain form)."""
        d = self.domain
        dt = d.timestep
        b = np.array(d._scn.stats().boundary_flux_sum[:]) if d._scn is not None else d.boundary_flux_sum
        m = d.timestepping_method
        if m == "euler":
            self._host = self._host + dt * b[0]
        elif m == "rk2":
            self._host = self._host + 0.5 * dt * (b[0] + b[1])
        elif m == "rk3":
            self._host = self._host + 1.0 / 6.0 * dt * (b[0] + b[1] + 4.0 * b[2])
        else:
            raise Exception("Cannot compute boundary flux integral with this timestepping method")
        d.boundary_flux_sum = np.zeros(3)

    def __getstate__(self):
        state = self.__dict__.copy()
        state["_host"] = self.get_integral()     # the restored domain's device clock starts at zero
        return state

    def parallel_safe(self):
        return True

    def statistics(self):
        return self.label + ": Boundary_flux_integral operator"

    def timestepping_statistics(self):
        return "    " + self.label + ": Integrating the boundary flux"


class Rate_operator(Operator):
    def __init__(self, domain, rate=0.0, factor=1.0, region=None, indices=None, polygon=None,
                 center=None, radius=None, default_rate=0.0, label=None, monitor=False, verbose=False):
        super().__init__(domain)
        if polygon is not None:
            indices = inside_polygon(domain.get_centroid_coordinates(), polygon)
        elif center is not None and radius is not None:
            c = domain.get_centroid_coordinates()
            indices = np.nonzero((c[:, 0] - center[0]) ** 2 + (c[:, 1] - center[1]) ** 2 <= radius ** 2)[0]
        elif region is not None:
            indices = region
        self.indices = None if indices is None else np.asarray(indices, np.int64)
        self.rate = rate
        self.factor = factor
        self.cumulative_influx = 0.0
        self.device_loop = not callable(rate) and not callable(factor)
        self.label = label
        domain._operators_changed()

    def get_rate(self, t=None):
        return float(self.rate(t)) if callable(self.rate) else float(self.rate)

    def get_factor(self, t=None):
        return float(self.factor(t)) if callable(self.factor) else float(self.factor)

    def __call__(self):
        """Host-driven step (a boundary or operator of the domain is a Python
        function of time): the host evaluates rate(t) and factor(t), the
        device applies them (rate_operators.py:149-258)."""
        d = self.domain
        t = d.get_time()
        dt = d.get_timestep()
        d._apply_rate_now(self, self.get_rate(t), self.get_factor(t), dt)

    def get_Q(self):
        """Cumulative influx (m^3) applied by this operator on the device."""
        d = self.domain
        if d._scn is not None and getattr(self, "_dev_index", None) is not None:
            return d._scn.operator_influx(self._dev_index) + getattr(self, "_influx_offset", 0.0)
        return self.cumulative_influx + getattr(self, "_influx_offset", 0.0)


def line_intersect(mesh, line):
    """Triangles a line segment intersects, by the test of
    geometry/polygon.c:446-525 (__triangle_line_intersect): the segment
    crosses an edge (segment and edge parameters both in [0, 1]), or lies
    inside the triangle (edge crossings beyond both of its ends)."""
    V = np.asarray(mesh.vertex_coordinates, float).reshape(-1, 3, 2)
    p0x, p0y = float(line[0][0]), float(line[0][1])
    p1x, p1y = float(line[1][0]), float(line[1][1])
    ppx, ppy = -(p1y - p0y), p1x - p0x
    ux, uy = p1x - p0x, p1y - p0y
    hit = np.zeros(len(V), bool)
    A = np.zeros(len(V), np.int64)
    B = np.zeros(len(V), np.int64)
    for j in range(1, 4):
        t0 = V[:, j - 1]
        t1 = V[:, j % 3]
        tpx, tpy = -(t1[:, 1] - t0[:, 1]), t1[:, 0] - t0[:, 0]
        vx, vy = t0[:, 0] - p0x, t0[:, 1] - p0y
        wx, wy = t1[:, 0] - t0[:, 0], t1[:, 1] - t0[:, 1]
        u_tp = ux * tpx + uy * tpy
        ok = u_tp != 0.0
        with np.errstate(divide="ignore", invalid="ignore"):
            a = (vx * tpx + vy * tpy) / u_tp
            b = -(vx * ppx + vy * ppy) / (wx * ppx + wy * ppy)
        inb = (b >= 0.0) & (b <= 1.0)
        hit |= ok & (a >= 0.0) & (a <= 1.0) & inb
        A += (ok & (a > 1.0) & inb).astype(np.int64)
        B += (ok & (a < 0.0) & inb).astype(np.int64)
    hit |= (A >= 1) & (B >= 1)
    return np.nonzero(hit)[0]


def region_indices(domain, region):
    """Cells of an inlet region as the reference's Region with
    expand_polygon=True (abstract_2d_finite_volumes/region.py:244-285): a
    line of two points gives the triangles it intersects; a polygon gives the
    triangles whose centroid is inside plus those its edges intersect."""
    r = np.asarray(region, float)
    if r.shape == (2, 2):
        return line_intersect(domain.mesh, r)
    idx = inside_polygon(domain.get_centroid_coordinates(), r)
    n = len(r)
    for j in range(n):
        idx = np.union1d(line_intersect(domain.mesh, [r[j], r[(j + 1) % n]]), idx)
    return np.asarray(idx, np.int64)


class Inlet_operator(Operator):
    """Discharge Q (m^3/s; a constant or a function of time) into an inlet
    region (structures/inlet_operator.py:17-165).

    region: cell indices, a polygon or a line of two points (selected as the
    reference's Region with expand_polygon=True), or an object with
    ``indices``.
    velocity: optional [u, v] for the momenta of the inlet cells;
    zero_velocity: set their momenta to zero.  At most 2048 cells."""

    def __init__(self, domain, region=None, Q=0.0, velocity=None, zero_velocity=False, default=0.0,
                 description=None, label=None, logging=False, verbose=False, center=None, radius=None):
        super().__init__(domain)
        mesh = domain.mesh
        if center is not None and radius is not None:
            c = domain.get_centroid_coordinates()
            idx = np.nonzero((c[:, 0] - center[0]) ** 2 + (c[:, 1] - center[1]) ** 2 <= radius ** 2)[0]
        elif hasattr(region, "indices"):
            idx = np.asarray(region.indices, np.int64)
        else:
            r = np.asarray(region)
            if r.ndim == 1 and np.issubdtype(r.dtype, np.integer):
                idx = r.astype(np.int64)
            elif r.ndim == 2 and r.shape[1] == 2 and r.shape[0] >= 2:
                idx = region_indices(domain, r)
            else:
                raise ValueError("region must be cell indices, a line of two points or a polygon")
        if idx.size == 0:
            raise ValueError("No triangles have been identified in region")
        self.indices = np.unique(idx)
        self.area = float(np.sum(mesh.areas[self.indices]))
        if velocity is not None and len(velocity) != 2:
            raise ValueError("velocity must be [u, v]")
        self.Q = Q
        self.velocity = velocity
        self.zero_velocity = bool(zero_velocity)
        self.default = default
        self.label = label
        self.device_loop = not callable(Q)
        domain._operators_changed()

    @property
    def flags(self):
        return (1 if self.velocity is not None else 0) | (2 if self.zero_velocity else 0)

    def update_Q(self, t):
        if callable(self.Q):
            try:
                return float(self.Q(t))
            except Exception:
                return float(self.default(t) if callable(self.default) else self.default)
        return float(self.Q)

    def __call__(self):
        """Host-driven step: Q(t) and Q(t + dt) from the host, applied on the device."""
        d = self.domain
        t = d.get_time()
        dt = d.get_timestep()
        d._apply_rate_now(self, self.update_Q(t), self.update_Q(t + dt), dt)

    def get_total_applied_volume(self):
        d = self.domain
        if d._scn is not None and getattr(self, "_dev_index", None) is not None:
            return d._scn.operator_influx(self._dev_index) + getattr(self, "_influx_offset", 0.0)
        return getattr(self, "_influx_offset", 0.0)
