"""Fractional-step operators applied after each flow step.

``Rate_operator`` follows operators/rate_operators.py:149-258: after every
full timestep, ``stage_c[idx] += factor * dt * rate`` (with the momentum
scaling branch for negative rates).  Constant rates run on the device inside
the step loop; a rate given as a function of time is evaluated on the host
once per step by the host-driven step path.
"""
from __future__ import annotations

import numpy as np

from .geometry import inside_polygon


class Operator:
    device_loop = True

    def __init__(self, domain):
        self.domain = domain
        domain.fractional_step_operators.append(self)

    def __call__(self):  # host-driven path
        raise NotImplementedError

    def log_timestepping_statistics(self):
        pass


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
        """Host-driven application (used when the rate is a function of time)."""
        d = self.domain
        t = d.get_time()
        dt = d.get_timestep()
        d._apply_rate_now(self.indices, self.get_rate(t), self.get_factor(t), dt)

    def get_Q(self):
        return self.cumulative_influx
