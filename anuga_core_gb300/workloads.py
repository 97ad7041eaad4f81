"""Synthetic benchmark scenarios (seeded; no external data).

* ``dam_break``      : rectangular cross m x m over 100 m x 100 m, bed -x/20,
                       stage = bed + 1.0 m for x < 50 and bed + 0.1 m otherwise,
                       Manning 0.03, reflective walls, DE0 (40,000 triangles at m=100).
* ``inflow_bumps``   : rectangular cross m x m over 10 km x 10 km, bed = linear
                       slope + 64 Gaussian bumps (seeded centres, amplitudes
                       U(-5,5) m, widths U(100,800) m), slope chosen so that
                       about 30% of the cells are dry at stage 0; Dirichlet
                       stage 2 m west, transmissive east, reflective north and
                       south, Manning U(0.02,0.06) per cell, DE1 (4.0M
                       triangles at m=1000).
Each builder returns a configured Domain (store disabled).
"""
from __future__ import annotations

import numpy as np

from .domain import Domain
from .mesh import rectangular_cross
from .boundaries import Reflective_boundary, Transmissive_boundary, Dirichlet_boundary


def dam_break(m=100, flow_algorithm="DE0", precision="fp64"):
    p, e, b = rectangular_cross(m, m, 100.0, 100.0)
    d = Domain(p, e, b)
    d.set_flow_algorithm(flow_algorithm)
    d.set_gpu_options(precision=precision)
    d.set_store(False)
    d.set_quantity("elevation", lambda x, y: -x / 20)
    d.set_quantity("stage", lambda x, y: -x / 20 + np.where(x < 50, 1.0, 0.1))
    d.set_quantity("friction", 0.03)
    Br = Reflective_boundary(d)
    d.set_boundary({"left": Br, "right": Br, "top": Br, "bottom": Br})
    return d


def _bumps(n_bumps, L, rng):
    cx = rng.uniform(0, L, n_bumps)
    cy = rng.uniform(0, L, n_bumps)
    A = rng.uniform(-5, 5, n_bumps)
    s = rng.uniform(100.0 * L / 1.0e4, 800.0 * L / 1.0e4, n_bumps)
    return cx, cy, A, s


def _bump_field(x, y, bumps, chunk=1 << 20):
    cx, cy, A, s = bumps
    out = np.zeros_like(x)
    for a in range(0, x.size, chunk):
        xs = x[a:a + chunk]
        ys = y[a:a + chunk]
        acc = np.zeros_like(xs)
        for i in range(cx.size):
            acc += A[i] * np.exp(-((xs - cx[i]) ** 2 + (ys - cy[i]) ** 2) / (2.0 * s[i] ** 2))
        out[a:a + chunk] = acc
    return out


def inflow_bumps(m=1000, L=1.0e4, seed=1234, dry_fraction=0.30, flow_algorithm="DE1", precision="fp64"):
    rng = np.random.default_rng(seed)
    bumps = _bumps(64, L, rng)
    p, e, b = rectangular_cross(m, m, L, L)
    d = Domain(p, e, b)
    d.set_flow_algorithm(flow_algorithm)
    d.set_gpu_options(precision=precision)
    d.set_store(False)
    node_bumps = _bump_field(p[:, 0], p[:, 1], bumps)
    # slope s so that ~dry_fraction of the centroids lie above stage 0
    tri = d.mesh.triangles
    cb = (node_bumps[tri[:, 0]] + node_bumps[tri[:, 1]] + node_bumps[tri[:, 2]]) / 3.0
    cxx = d.mesh.centroid_coordinates[:, 0]
    lo, hi = -1e-2, 1e-2
    for _ in range(60):
        s = 0.5 * (lo + hi)
        frac = np.mean(s * cxx + cb > 0.0)
        if frac < dry_fraction:
            lo = s
        else:
            hi = s
    slope = 0.5 * (lo + hi)
    zn = slope * p[:, 0] + node_bumps
    d.set_quantity("elevation", zn[tri].reshape(-1, 3))
    d.set_quantity("stage", 0.0)
    d.set_quantity("friction", rng.uniform(0.02, 0.06, len(d)), location="centroids")
    d.set_boundary({"left": Dirichlet_boundary([2.0, 0.0, 0.0]), "right": Transmissive_boundary(d),
                    "top": Reflective_boundary(d), "bottom": Reflective_boundary(d)})
    d.workload_info = dict(slope=slope, seed=seed, dry_fraction=float(np.mean(slope * cxx + cb > 0.0)))
    return d


def batch_sizes(count=256, seed=42, lo=20, hi=400, target=20.0e6, tol=0.05, max_draws=1000):
    """Mesh sides m_i = round(exp(U(log lo, log hi))), redrawn with the same
    generator until sum(4 m_i^2) is within tol of target.  Returns (sides, draw)."""
    rng = np.random.default_rng(seed)
    for draw in range(max_draws):
        m = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(int)
        if abs(4 * np.sum(m * m) - target) <= tol * target:
            return m, draw
    raise RuntimeError("no draw within tolerance")


def batch_scenario(m, seed, kind, precision="mixed"):
    """One scenario of the batched workload: rectangular cross m x m over
    10m x 10m metres, slope + 8 Gaussian bumps, dam break (stage = bed + 1 m
    for x < L/2) or Dirichlet inflow (stage 1.5 m west), Manning U(0.02, 0.05), DE1."""
    rng = np.random.default_rng(seed)
    L = 10.0 * m
    p, e, b = rectangular_cross(m, m, L, L)
    d = Domain(p, e, b)
    d.set_flow_algorithm("DE1")
    d.set_gpu_options(precision=precision)
    d.set_store(False)
    cx = rng.uniform(0, L, 8)
    cy = rng.uniform(0, L, 8)
    A = rng.uniform(-2, 2, 8)
    s = rng.uniform(0.05 * L, 0.2 * L, 8)
    slope = rng.uniform(0.001, 0.005)
    zn = -slope * p[:, 0] + _bump_field(p[:, 0], p[:, 1], (cx, cy, A, s))
    tri = d.mesh.triangles
    d.set_quantity("elevation", zn[tri].reshape(-1, 3))
    zc = d.quantities["elevation"].centroid_values
    xc = d.mesh.centroid_coordinates[:, 0]
    if kind == "dam":
        d.set_quantity("stage", zc + np.where(xc < 0.5 * L, 1.0, 0.0), location="centroids")
        Br = Reflective_boundary(d)
        d.set_boundary({"left": Br, "right": Br, "top": Br, "bottom": Br})
    else:
        d.set_quantity("stage", zc, location="centroids")       # dry; filled from the west
        d.set_boundary({"left": Dirichlet_boundary([1.5, 0.0, 0.0]), "right": Transmissive_boundary(d),
                        "top": Reflective_boundary(d), "bottom": Reflective_boundary(d)})
    d.set_quantity("friction", rng.uniform(0.02, 0.05, len(d)), location="centroids")
    return d


def batch_workload(count=256, seed=42, precision="mixed", target=20.0e6):
    sides, draw = batch_sizes(count, seed, target=target)
    doms = [batch_scenario(int(m), seed * 1000 + i, "dam" if i % 2 == 0 else "inflow", precision)
            for i, m in enumerate(sides)]
    return doms, dict(sides=sides.tolist(), draw=draw, cells=int(4 * np.sum(sides * sides)))
