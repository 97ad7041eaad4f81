"""Boundary condition objects (host descriptors of device boundary kinds).

Same constructors as the reference:

* ``Reflective_boundary(domain)``      shallow_water/boundaries.py:44-292
* ``Transmissive_boundary(domain)``    abstract_2d_finite_volumes/generic_boundary_conditions.py:139-195
* ``Dirichlet_boundary([w, uh, vh])``  generic_boundary_conditions.py:198-264
* ``Time_boundary(domain, function)``  generic_boundary_conditions.py:297-416
* ``Transmissive_n_momentum_zero_t_momentum_set_stage_boundary(domain, function)``
  shallow_water/boundaries.py:384-519
* ``Transmissive_momentum_set_stage_boundary(domain, function)``  boundaries.py:295-383
* ``Transmissive_stage_zero_momentum_boundary(domain)``          boundaries.py:520-552
* ``Time_stage_zero_momentum_boundary(domain, function)``        boundaries.py:553-638
* ``Dirichlet_discharge_boundary(domain, stage0, wh0)``           boundaries.py:850-901
* ``Flather_external_stage_zero_velocity_boundary(domain, function)`` boundaries.py:1096-1330
* ``Characteristic_stage_boundary(domain, function, default_stage)``   boundaries.py:639-848
* ``Time_space_boundary(domain, function(t, x, y))``  generic_boundary_conditions.py:419-517
* ``Inflow_boundary(domain, rate)``                  shallow_water/boundaries.py:902-992
* ``Compute_fluxes_boundary()``                      generic_boundary_conditions.py:266-296

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


def _stage_value(v):
    # a stage function may return a number or a vector whose first entry is the stage
    try:
        return float(v)
    except TypeError:
        return float(np.asarray(v, float).ravel()[0])


class Transmissive_momentum_set_stage_boundary(Boundary):
    """Stage from f(t) (or a constant), both momenta transmitted from the
    interior edge."""
    kind = _lib.BC_TRANSMISSIVE_SET_STAGE

    def __init__(self, domain=None, function=None):
        if domain is None:
            raise Exception("Domain must be specified for this type boundary")
        if function is None:
            raise Exception("Function must be specified for this type boundary")
        self.domain = domain
        self.function = function
        self.device_loop = not callable(function)

    def values(self, t):
        w = _stage_value(self.function(t) if callable(self.function) else self.function)
        return (w, 0.0, 0.0)

    def __repr__(self):
        return "Transmissive_momentum_set_stage_boundary(%s)" % self.domain


class Transmissive_stage_zero_momentum_boundary(Boundary):
    """Stage transmitted from the interior edge, momenta zero."""
    kind = _lib.BC_TRANSMISSIVE_ZERO_MOM

    def __init__(self, domain=None):
        if domain is None:
            raise Exception("Domain must be specified for Transmissive_stage_zero_momentum boundary")
        self.domain = domain

    def __repr__(self):
        return "Transmissive_stage_zero_momentum_boundary(%s)" % self.domain


class Time_stage_zero_momentum_boundary(Boundary):
    """Stage from f(t), momenta zero (a Dirichlet value the host evaluates at
    every stage's time).  The reference's class stores the function as
    ``self.f`` but reads ``self.function`` when evaluated; this one applies
    the documented behaviour."""
    kind = _lib.BC_DIRICHLET
    device_loop = False

    def __init__(self, domain=None, function=None, default_boundary=None, verbose=False):
        if domain is None:
            raise Exception("You must specify a domain to Time_stage_zero_momemtum_boundary")
        if function is None:
            raise Exception("You must specify a function to Time_stage_zero_momemtum_boundary")
        try:
            q = float(function(0.0))
        except Exception as e:
            raise Exception("Function for time stage boundary could not be executed:\n%s" % e)
        self.domain = domain
        self.function = function
        self.default_boundary = default_boundary

    def values(self, t):
        return (_stage_value(self.function(t)), 0.0, 0.0)

    def __repr__(self):
        return "Time_stage_zero_momemtum_boundary"


class Dirichlet_discharge_boundary(Boundary):
    """Stage stage0 and momentum wh0 along the inward normal of each edge."""
    kind = _lib.BC_DIRICHLET

    def __init__(self, domain=None, stage0=None, wh0=None):
        if domain is None:
            raise Exception("Domain must be specified for this type of boundary")
        if stage0 is None:
            raise Exception("Stage must be specified for this type of boundary")
        self.domain = domain
        self.stage0 = stage0
        self.wh0 = 0.0 if wh0 is None else wh0

    def edge_values(self, t, n1, n2, x, y, tag=None):
        """Values of edges with outward normals (n1, n2): [stage0, -wh0 n1, -wh0 n2]."""
        return np.column_stack([np.full(n1.shape, float(self.stage0)), -self.wh0 * n1, -self.wh0 * n2])

    def __repr__(self):
        return "Dirichlet_Discharge_boundary(%s)" % self.domain


class Flather_external_stage_zero_velocity_boundary(Boundary):
    """Outside stage from f(t) and zero outside velocity combined with the
    inside state along the characteristics (a weakly reflecting boundary)."""
    kind = _lib.BC_FLATHER

    def __init__(self, domain=None, function=None):
        if domain is None:
            raise Exception("Domain must be specified for this type boundary")
        if function is None:
            raise Exception("Function must be specified for this type boundary")
        self.domain = domain
        self.function = function
        self.device_loop = not callable(function)

    def values(self, t):
        w = _stage_value(self.function(t) if callable(self.function) else self.function)
        return (w, 0.0, 0.0)

    def __repr__(self):
        return "Flather_external_stage_zero_velocity_boundary(%s)" % self.domain


class Characteristic_stage_boundary(Boundary):
    """Stage from f(t); momentum of a simple incoming wave from the Riemann
    invariant of the inside state."""
    kind = _lib.BC_CHARACTERISTIC

    def __init__(self, domain=None, function=None, default_stage=0.0):
        if domain is None:
            raise Exception("Domain must be specified for Characteristic_stage_boundary")
        if function is None:
            raise Exception("Function must be specified for Characteristic_stage_boundary")
        self.domain = domain
        self.function = function
        self.default_stage = default_stage
        self.device_loop = not callable(function)

    def values(self, t):
        w = _stage_value(self.function(t) if callable(self.function) else self.function)
        return (w, 0.0, 0.0)

    def __repr__(self):
        return "Characteristic_stage_boundary(%s)" % self.domain


class Time_space_boundary(Boundary):
    """Dirichlet values f(t, x, y) -> (w, uh, vh) at each edge's midpoint,
    evaluated by the host at every stage's time."""
    kind = _lib.BC_DIRICHLET
    device_loop = False

    def __init__(self, domain=None, function=None, default_boundary=None, verbose=False):
        if function is None:
            raise Exception("You must specify a function to Time_space_boundary")
        try:
            q = np.array(function(0.0, 0.0, 0.0), float)
        except Exception as e:
            raise Exception("Function for time_space_boundary could not be executed:\n%s" % e)
        if q.size != 3:
            raise Exception("Return value from time_space_boundary function must be a list of 3 values")
        self.domain = domain
        self.function = function
        self.default_boundary = default_boundary

    def edge_values(self, t, n1, n2, x, y, tag=None):
        out = np.empty((len(x), 3))
        for i in range(len(x)):
            out[i] = np.asarray(self.function(t, x[i], y[i]), float).ravel()[:3]
        return out

    def __repr__(self):
        return "Time space boundary"


class Inflow_boundary(Boundary):
    """A discharge ``rate`` (m^3/s) spread over the tag's edges: momentum
    rate / (total edge length) along each inward normal, stage 1 m above the
    edge's bed (the reference's Manning depth with a zero slope)."""
    kind = _lib.BC_INFLOW

    def __init__(self, domain=None, rate=0.0):
        if domain is None:
            raise Exception("Domain must be specified for Inflow boundary")
        self.domain = domain
        self.rate = rate
        self.tag = None
        self.length = None

    def _tag_length(self, tag):
        # the tag of the first edge evaluated fixes the length (the reference's cache)
        if self.tag is None:
            self.tag = tag
            m = self.domain.mesh
            length = 0.0
            lengths = np.asarray(m.edgelengths).reshape(-1, 3)
            for (v, e), t in m.boundary.items():
                if t == self.tag:
                    length += lengths[v, e]
            self.length = length
            self.average_momentum = self.rate / length
        return self.average_momentum

    def edge_values(self, t, n1, n2, x, y, tag=None):
        mu = self._tag_length(tag)
        return np.column_stack([np.full(n1.shape, 1.0), mu * (-n1), mu * (-n2)])

    def __repr__(self):
        return "Inflow_boundary(%s)" % self.domain


class Compute_fluxes_boundary(Boundary):
    """Leaves the boundary values as they are (the flux computation decides)."""
    kind = _lib.BC_NONE

    def __init__(self):
        self.domain = None

    def __repr__(self):
        return "Compute_fluxes_boundary(%s)" % self.domain
