"""Boundary condition objects (host descriptors of device boundary kinds).

Same constructors as the reference:

* ``Reflective_boundary(domain)``      shallow_water/boundaries.py:44-292
* ``Transmissive_boundary(domain)``    abstract_2d_finite_volumes/generic_boundary_conditions.py:139-195
* ``Dirichlet_boundary([w, uh, vh])``  generic_boundary_conditions.py:198-264
* ``Time_boundary(domain, function)``  generic_boundary_conditions.py:297-416
* ``Transmissive_n_momentum_zero_t_momentum_set_stage_boundary(domain, function)``
  shallow_water/boundaries.py:384-519

Each evaluates on the device.  Time-dependent boundaries given as a Python
function are sampled at the device time of every stage by the host-driven
step path; ``Time_boundary`` with a ``series=(times, values)`` table runs
inside the device step loop.
"""
from __future__ import annotations

import numpy as np

from . import _lib


class Boundary:
    kind = _lib.BC_NONE
    device_loop = True     # evaluable inside the graph-captured step loop

    def values(self, t):
        return (0.0, 0.0, 0.0)


class Reflective_boundary(Boundary):
    kind = _lib.BC_REFLECTIVE

    def __init__(self, domain=None):
        if domain is None:
            raise ValueError("Domain must be specified for reflective boundary")
        self.domain = domain

    def __repr__(self):
        return "Reflective_boundary"


class Transmissive_boundary(Boundary):
    kind = _lib.BC_TRANSMISSIVE

    def __init__(self, domain=None):
        if domain is None:
            raise ValueError("Domain must be specified for transmissive boundary")
        self.domain = domain

    @property
    def effective_kind(self):
        return _lib.BC_TRANSMISSIVE_C if getattr(self.domain, "centroid_transmissive_bc", False) \
            else _lib.BC_TRANSMISSIVE

    def __repr__(self):
        return "Transmissive_boundary"


class Dirichlet_boundary(Boundary):
    kind = _lib.BC_DIRICHLET

    def __init__(self, dirichlet_values=None):
        if dirichlet_values is None:
            raise ValueError("Must specify one value for each quantity")
        v = np.array(dirichlet_values, float).ravel()
        if v.size < 3:
            raise ValueError("Dirichlet_boundary needs (stage, xmomentum, ymomentum)")
        self.dirichlet_values = v

    def values(self, t):
        return tuple(self.dirichlet_values[:3])

    def __repr__(self):
        return "Dirichlet boundary (%s)" % self.dirichlet_values


class Time_boundary(Boundary):
    """Dirichlet values from a function of time f(t) -> (w, uh, vh), or from a
    table ``series=(times, values[n,3])`` interpolated linearly on the device."""
    kind = _lib.BC_TIME_SERIES

    def __init__(self, domain=None, function=None, series=None, default_boundary=None, verbose=False):
        if function is None and series is None:
            raise ValueError("Time_boundary needs a function or a series")
        self.domain = domain
        self.function = function
        self.series = None
        if series is not None:
            t, v = series
            t = np.asarray(t, float)
            v = np.asarray(v, float).reshape(len(t), -1)[:, :3]
            self.series = np.column_stack([t, v])
        self.device_loop = self.series is not None
        if function is not None and series is None:
            self.kind = _lib.BC_DIRICHLET

    def values(self, t):
        if self.function is not None:
            r = np.asarray(self.function(t), float).ravel()
            return tuple(r[:3])
        s = self.series
        return tuple(np.interp(t, s[:, 0], s[:, c]) for c in (1, 2, 3))


class Transmissive_n_momentum_zero_t_momentum_set_stage_boundary(Boundary):
    """Stage from f(t) (or a constant), normal momentum transmitted from the
    interior edge, tangential momentum zero."""
    kind = _lib.BC_TRANSMISSIVE_N0

    def __init__(self, domain=None, function=None, stage=None):
        self.domain = domain
        self.function = function
        self.stage = stage
        self.device_loop = function is None

    def values(self, t):
        w = float(self.function(t)) if self.function is not None else float(self.stage or 0.0)
        return (w, 0.0, 0.0)
