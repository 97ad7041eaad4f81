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
* ``rain_polygon``   : unstructured mesh of a seeded 20-vertex random polygon
                       (Delaunay of a jittered lattice: triangles of at most
                       50 m^2, at most 12.5 m^2 inside a seeded refined
                       region), bed = 6-octave value noise in [-10, 30] m,
                       stage 0, rain 50 mm/h over a 1 km^2 square, Dirichlet
                       stage 3 m on a 500 m inflow segment, reflective walls,
                       DE1 (about 1.2M triangles at the default size).
Each builder returns a configured Domain (store disabled).
"""
from __future__ import annotations

import numpy as np

from .domain import Domain
from .geometry import inside_polygon
from .mesh import Mesh, rectangular_cross
from .operators import Rate_operator
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


# ---------------------------------------------------------------------------
# Unstructured workload: rain and inflow on a random polygon


def random_polygon(n_vertices, rng, r_lo=0.55, r_hi=1.0):
    """Star-shaped (hence simple) polygon: angle-sorted random directions with
    random radii, counter-clockwise, around the origin."""
    ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, n_vertices))
    r = rng.uniform(r_lo, r_hi, n_vertices)
    return np.stack([r * np.cos(ang), r * np.sin(ang)], 1)


def polygon_area(poly):
    x, y = poly[:, 0], poly[:, 1]
    return 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))


def value_noise(x, y, octaves=6, seed=7, base=4, lo=-10.0, hi=30.0):
    """Sum of `octaves` octaves of value noise (random values on a 2^k lattice
    over the points' bounding box, smoothstep-interpolated, amplitude halved
    per octave), rescaled to [lo, hi]."""
    rng = np.random.default_rng(seed)
    u = (x - x.min()) / max(x.max() - x.min(), 1e-12)
    v = (y - y.min()) / max(y.max() - y.min(), 1e-12)
    total = np.zeros_like(u)
    amp = 1.0
    for o in range(octaves):
        n = base << o
        G = rng.uniform(-1.0, 1.0, (n + 1, n + 1))
        fx, fy = u * n, v * n
        ix = np.minimum(fx.astype(np.int64), n - 1)
        iy = np.minimum(fy.astype(np.int64), n - 1)
        tx, ty = fx - ix, fy - iy
        sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
        a = G[ix, iy] * (1 - sx) + G[ix + 1, iy] * sx
        b = G[ix, iy + 1] * (1 - sx) + G[ix + 1, iy + 1] * sx
        total += amp * (a * (1 - sy) + b * sy)
        amp *= 0.5
    t = (total - total.min()) / max(total.max() - total.min(), 1e-12)
    return lo + (hi - lo) * t


def _lattice(x0, x1, y0, y1, h, rng, jitter):
    nx = int(np.floor((x1 - x0) / h)) + 1
    ny = int(np.floor((y1 - y0) / h)) + 1
    gx, gy = np.meshgrid(x0 + h * np.arange(nx), y0 + h * np.arange(ny), indexing="ij")
    pts = np.stack([gx.ravel(), gy.ravel()], 1)
    return pts + rng.uniform(-jitter, jitter, pts.shape) * h


def polygon_mesh(target_cells=1.2e6, seed=7, max_area=50.0, refine=4.0, n_vertices=20, jitter=0.1,
                 inflow_length=500.0):
    """Unstructured triangle mesh of a seeded random polygon with a refined
    interior region.

    Jittered square lattices (spacing sqrt(2 max_area) / 1.12, so that the
    jittered halves of a lattice square stay below max_area, and sqrt(refine)
    times finer inside the refined polygon) are triangulated by Delaunay; triangles
    whose centroid lies in the outer polygon are kept and oriented
    counter-clockwise.  Triangles above their area limit get their centroid
    inserted as a new point and the set is triangulated again (conforming by
    construction).  The polygon is scaled so that the mesh has about
    `target_cells` triangles.  Boundary edges within inflow_length / 2 of the
    polygon's first vertex are tagged 'inflow', the others 'wall'.
    Returns (mesh, info)."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    outer = random_polygon(n_vertices, rng)
    c_in = outer.mean(0) * 0.0 + rng.uniform(-0.2, 0.2, 2)
    inner = random_polygon(8, rng, 0.6, 1.0) * 0.22 + c_in
    h = np.sqrt(2.0 * max_area) / 1.12
    hf = h / np.sqrt(refine)
    a_out, a_in = polygon_area(outer), polygon_area(inner)
    # cells ~ 2 (A_out - A_in) / h^2 + 2 A_in / hf^2
    scale = np.sqrt(target_cells * h * h / (2.0 * (a_out + (refine - 1.0) * a_in)))
    outer *= scale
    inner *= scale
    x0, y0 = outer.min(0) - 2 * h
    x1, y1 = outer.max(0) + 2 * h
    coarse = _lattice(x0, x1, y0, y1, h, rng, jitter)
    coarse = np.delete(coarse, inside_polygon(coarse, inner), axis=0)
    ix0, iy0 = inner.min(0)
    ix1, iy1 = inner.max(0)
    fine = _lattice(ix0, ix1, iy0, iy1, hf, rng, jitter)
    fine = fine[inside_polygon(fine, inner)]
    pts = np.concatenate([coarse, fine])
    limit_fine = max_area / refine
    for _ in range(6):
        tri = Delaunay(pts).simplices.astype(np.int64)
        a = pts[tri]
        cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
        cen = a.mean(1)
        keep = np.zeros(len(tri), bool)
        keep[inside_polygon(cen, outer)] = True
        keep &= np.abs(cr) > 1e-9 * h * h
        tri, cr, cen = tri[keep], cr[keep], cen[keep]
        area = 0.5 * np.abs(cr)
        lim = np.full(len(tri), max_area)
        lim[inside_polygon(cen, inner)] = limit_fine
        big = area > lim
        if not big.any():
            break
        pts = np.concatenate([pts, cen[big]])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    used = np.unique(tri)
    remap = -np.ones(len(pts), np.int64)
    remap[used] = np.arange(len(used))
    pts = pts[used]
    tri = remap[tri]
    M0 = Mesh(pts, tri)
    E = M0.edge_midpoint_coordinates.reshape(-1, 3, 2)
    v0 = outer[0]
    bnd = {}
    for (vol, e) in M0.boundary:
        q = E[vol, e]
        bnd[(vol, e)] = "inflow" if np.hypot(q[0] - v0[0], q[1] - v0[1]) <= 0.5 * inflow_length else "wall"
    mesh = Mesh(pts, tri, bnd)
    info = dict(seed=seed, cells=len(mesh), polygon=outer.tolist(), refined=inner.tolist(),
                area_km2=float(np.sum(mesh.areas)) / 1e6, max_area=float(mesh.areas.max()))
    return mesh, info


_POLYGON_MESHES = {}


def rain_polygon(target_cells=1.2e6, seed=7, precision="mixed", flow_algorithm="DE1", rain_mm_per_hour=50.0,
                 inflow_stage=3.0, patch_km2=1.0):
    """The unstructured rain-and-inflow scenario (see the module docstring).
    The mesh of a (target_cells, seed) pair is built once per process."""
    from .boundaries import Dirichlet_boundary as _D, Reflective_boundary as _R
    key = (float(target_cells), int(seed))
    if key not in _POLYGON_MESHES:
        _POLYGON_MESHES[key] = polygon_mesh(target_cells, seed)
    mesh, info = _POLYGON_MESHES[key]
    info = dict(info)
    d = Domain(mesh.nodes, mesh.triangles, mesh.boundary)
    d.set_flow_algorithm(flow_algorithm)
    d.set_gpu_options(precision=precision)
    d.set_store(False)
    zn = value_noise(mesh.nodes[:, 0], mesh.nodes[:, 1], seed=seed)
    d.set_quantity("elevation", zn[mesh.triangles].reshape(-1, 3))
    d.set_quantity("stage", 0.0)
    d.set_quantity("friction", 0.03)
    d.set_boundary({"inflow": _D([inflow_stage, 0.0, 0.0]), "wall": _R(d)})
    # rain over a 1 km^2 square centred on the cell nearest the polygon's centroid
    C = mesh.centroid_coordinates
    c = C[np.argmin(np.hypot(C[:, 0] - C[:, 0].mean(), C[:, 1] - C[:, 1].mean()))]
    half = 500.0 * np.sqrt(patch_km2)
    square = [[c[0] - half, c[1] - half], [c[0] + half, c[1] - half], [c[0] + half, c[1] + half],
              [c[0] - half, c[1] + half]]
    rate = rain_mm_per_hour / 1000.0 / 3600.0
    op = Rate_operator(d, rate=rate, polygon=square)
    info.update(rain_cells=int(op.indices.size), rain_rate=rate, inflow_edges=len(mesh.tag_boundary_cells["inflow"])
                if "inflow" in mesh.tag_boundary_cells else 0)
    d.workload_info = info
    return d
