"""Shared builders for the parity tests: the same mesh and initial state are
given to the GPU Domain and to the CPU oracle."""
import numpy as np

import anuga_core_gb300 as agx
from anuga_core_gb300.mesh import Mesh, rectangular_cross

KINDS = {"reflective": agx.Reflective_boundary, "transmissive": agx.Transmissive_boundary}


def make_domain(points, elements, boundary, alg, state, kinds, precision="fp64", rates=()):
    d = agx.Domain(points, elements, boundary)
    d.set_flow_algorithm(alg)
    d.set_store(False)
    d.set_gpu_options(precision=precision)
    d.set_quantity("elevation", state["elevation"], location="centroids")
    d.set_quantity("stage", state["stage"], location="centroids")
    d.set_quantity("xmomentum", state["xmom"], location="centroids")
    d.set_quantity("ymomentum", state["ymom"], location="centroids")
    d.set_quantity("friction", state["friction"], location="centroids")
    bmap = {}
    for tag, (kind, vals) in kinds.items():
        if kind == "dirichlet":
            bmap[tag] = agx.Dirichlet_boundary(list(vals))
        else:
            bmap[tag] = KINDS[kind](d)
    d.set_boundary(bmap)
    for idx, rate in rates:
        agx.Rate_operator(d, rate=rate, indices=idx)
    return d


def make_oracle(oracle, mesh, alg, state, kinds, rates=()):
    od = oracle.OracleDomain(mesh, alg)
    od.set_centroid_state(state["stage"], state["xmom"], state["ymom"], state["elevation"], state["friction"])
    od.set_boundaries([(mesh.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in mesh.tag_boundary_cells])
    for idx, rate in rates:
        od.add_rate(idx, rate)
    return od


def random_state(mesh, seed, dry_fraction=0.3, slope=0.01):
    rng = np.random.default_rng(seed)
    C = mesh.centroid_coordinates
    x, y = C[:, 0], C[:, 1]
    L = max(x.max() - x.min(), 1e-9)
    z = slope * (x - x.min()) + 0.3 * np.sin(3 * y / L) + 0.1 * rng.standard_normal(len(x))
    level = np.quantile(z, dry_fraction)
    w = np.maximum(z, level) + rng.uniform(0, 0.05, len(x)) * (z < level)
    w = np.where(rng.uniform(size=len(x)) < 0.02, z - 0.01, w)   # a few cells below the bed
    h = np.maximum(w - z, 0)
    return dict(elevation=z, stage=w, xmom=rng.normal(0, 0.3, len(x)) * h, ymom=rng.normal(0, 0.3, len(x)) * h,
                friction=rng.uniform(0.01, 0.05, len(x)))


def normwise(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    s = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / s)
