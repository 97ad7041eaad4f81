"""Batched scenarios: many independent meshes advanced together.

All scenarios of a ``Batch`` live in one device pool; every step of every
active scenario is taken by the same persistent kernels, and the step loop
runs as one CUDA graph launch with a device-side while loop (each scenario
keeps its own timestep, clock, boundaries and operators).  Scenarios of very
different sizes share the GPU without per-scenario launches.
"""
from __future__ import annotations

import numpy as np

from . import mixed
from .tables import hilbert_order, morton_order, pack_mixed


ORDERS = ("per-mesh", "hilbert", "morton")


def _tables(mesh, order):
    """Mixed tables of a mesh in one of ORDERS: the space-filling curve with
    the smaller halo cost for this mesh, or one curve for every mesh."""
    if order == "per-mesh":
        return pack_mixed(mesh)
    C = mesh.centroid_coordinates
    return pack_mixed(mesh, order=hilbert_order(C) if order == "hilbert" else morton_order(C))


class Batch:
    def __init__(self, domains, extra_cells=0, extra_scenarios=0, tables=None, distribute=False, order="per-mesh"):
        """distribute=True starts each scenario like evolve() does (protect
        and extrapolate first); False advances the state as it was set, like
        Domain.advance_steps.  order: the cell ordering of the meshes (one of
        ORDERS; tune_order picks it by timing)."""
        self.distribute = distribute
        self.domains = list(domains)
        self.extra = (int(extra_cells), int(extra_scenarios))
        self.order = order
        self.pool = self._pool(tables)

    def _pool(self, tables=None):
        cells = sum(len(d) for d in self.domains) + self.extra[0]
        bnd = sum(d.mesh.boundary_length for d in self.domains) + int(self.extra[0] // 8 + 64)
        ns = len(self.domains) + self.extra[1]
        self.pool = mixed.Pool(cells, max(bnd, 1), max(ns, 1))
        if getattr(self, "_stream", None):
            self.pool.set_stream(self._stream)
        self.sids = []
        for i, d in enumerate(self.domains):
            T = tables[i] if tables is not None else _tables(d.mesh, self.order)
            self.sids.append(self._add(d, T))
        return self.pool

    def tune_order(self, steps=3, reps=2):
        """Pick the cell ordering by timing: the pool is built with each of
        ORDERS from the domains' states, its kernel form tuned, and a few
        steps timed; the fastest pool is kept (in its initial state).
        Returns ({order: seconds per step}, chosen order)."""
        from .autotune import tune_pool
        res, forms = {}, {}
        for order in ORDERS:
            if order != self.order:
                self.pool.close()
                self.order = order
                self._pool()
            times, name = tune_pool(self.pool, steps=steps, reps=reps)
            res[order] = times[name]
            forms[order] = (times, name)
        best = min(res, key=res.get)
        if best != self.order:
            self.pool.close()
            self.order = best
            self._pool()
            forms[best] = tune_pool(self.pool, steps=steps, reps=reps)
        self.kernel_form = forms[best]          # ({form: seconds per step}, chosen form) of the kept pool
        return res, best

    def _add(self, d, T=None):
        T = T if T is not None else pack_mixed(d.mesh)
        sid = self.pool.add(d.mesh, d._params(), T)
        Q = d.quantities
        for f, q in (("elev_c", "elevation"), ("stage_c", "stage"), ("xmom_c", "xmomentum"),
                     ("ymom_c", "ymomentum"), ("friction_c", "friction")):
            self.pool.set_field(sid, f, Q[q]._arr["centroid_values"])
        if d.boundary_map is not None:
            kind, vals, series = d._boundary_arrays(d.get_time())
            self.pool.set_boundary(sid, kind, vals)
            if series is not None:
                self.pool.set_boundary_series(sid, series)
        for op in d.fractional_step_operators:
            if getattr(op, "device_loop", False) and hasattr(op, "rate"):
                self.pool.add_rate(sid, op.indices, op.get_rate(), op.get_factor())
        if self.distribute:
            self.pool.distribute(sid)
        return sid

    def add(self, d):
        self.domains.append(d)
        self.sids.append(self._add(d))
        return len(self.domains) - 1

    def remove(self, i):
        self.pool.remove(self.sids[i])
        self.sids[i] = None

    def set_stream(self, ptr):
        self._stream = ptr
        self.pool.set_stream(ptr)

    def advance_steps(self, n, which=None):
        """Advance the chosen scenarios (all by default) by exactly n steps."""
        idx = range(len(self.sids)) if which is None else which
        for i in idx:
            sid = self.sids[i]
            if sid is None:
                continue
            st = self.pool.stats(sid)
            self.pool.set_clock(sid, st.time, 1e300, -1.0, n)
        self.pool.advance()
        return [self.pool.stats(self.sids[i]) for i in idx if self.sids[i] is not None]

    def advance_to(self, times, max_steps=0):
        """Advance scenario i to times[i] (its next yield or final time)."""
        for i, t in enumerate(times):
            sid = self.sids[i]
            if sid is None or t is None:
                continue
            st = self.pool.stats(sid)
            self.pool.set_clock(sid, st.time, 1e300, float(t), max_steps)
        self.pool.advance()

    def get_centroids(self, i, fields=("stage_c", "xmom_c", "ymom_c")):
        sid = self.sids[i]
        return {f: self.pool.get_field(sid, f) for f in fields}

    def stats(self, i):
        return self.pool.stats(self.sids[i])

    def cells(self):
        return sum(len(d) for d, s in zip(self.domains, self.sids) if s is not None)

    def close(self):
        self.pool.close()
