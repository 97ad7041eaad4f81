"""Device table construction for a mesh (host side, numpy).

Packs a :class:`~anuga_core_gb300.mesh.Mesh` into the flat arrays the CUDA
library consumes:

* ``conn``  int32 [N,4]: neighbours (boundary edges as -(m+1)) and a meta word
  (neighbour-edge ids, full flag, per-side flags, ordering bits, number of
  boundaries; bit layout in ``csrc/de_plain.cuh``).
* ``surr``  int32 [N,4]: surrogate neighbours, number of boundaries.
* ``geo``   float64 [N,11]: extrapolation geometry computed with the same
  operations as ``shallow_water/sw_domain_openmp.c:1445-1484, 1684-1696``.
* edge lists for the edge-once flux: ``edge_slot`` (slot 3k+i that evaluates
  the flux) and ``edge_opp`` (slot 3n+m that receives the negated flux, or -1).
"""
from __future__ import annotations

import numpy as np

GEO_STRIDE = 11


def pack_tables(mesh, tri_full_flag=None, per_side_edges=None, order=None):
    """Return a dict of numpy arrays for ``agx_scenario_create``.

    per_side_edges: optional bool [N,3] forcing per-side evaluation of slots
    (used for low-Froude scaling and riverwalls, where the edge flux is not
    antisymmetric).  order: original index of each cell (for the ordering
    bits); defaults to the identity.
    """
    N = len(mesh)
    nb = np.asarray(mesh.neighbours, np.int64)
    ne = np.asarray(mesh.neighbour_edges, np.int64)
    sn = np.asarray(mesh.surrogate_neighbours, np.int64)
    nbnd = np.asarray(mesh.number_of_boundaries, np.int64)
    if N >= (1 << 29):
        raise ValueError("mesh too large for 32-bit slot indices")
    full = np.ones(N, np.int64) if tri_full_flag is None else np.asarray(tri_full_flag, np.int64)
    normals = np.asarray(mesh.normals, np.float64)
    lengths = np.asarray(mesh.edgelengths, np.float64)
    cells = np.arange(N, dtype=np.int64)
    orig = cells if order is None else np.asarray(order, np.int64)

    # --- which interior slots can share one flux evaluation ---------------
    per_side = np.zeros((N, 3), bool) if per_side_edges is None else np.asarray(per_side_edges, bool).copy()
    interior = nb >= 0
    nbc = np.where(interior, nb, 0)
    nec = np.where(interior, ne, 0)
    # the two sides must be exact mirror images: normals negated, equal lengths
    nx_o = normals[nbc, 2 * nec]
    ny_o = normals[nbc, 2 * nec + 1]
    l_o = lengths[nbc, nec]
    mirror = np.ones((N, 3), bool)
    for i in range(3):
        mirror[:, i] = (normals[:, 2 * i] == -nx_o[:, i]) & (normals[:, 2 * i + 1] == -ny_o[:, i]) & \
                       (lengths[:, i] == l_o[:, i])
    # neighbour's back-pointer must point at us
    back = np.zeros((N, 3), bool)
    back[interior] = nb[nbc[interior], nec[interior]] == np.repeat(cells[:, None], 3, 1)[interior]
    per_side |= interior & ~(mirror & back)
    # a pair is per-side if either side asks for it
    ps_o = np.zeros((N, 3), bool)
    ps_o[interior] = per_side[nbc[interior], nec[interior]]
    per_side |= interior & ps_o

    meta = np.zeros(N, np.int64)
    for i in range(3):
        meta |= (np.where(interior[:, i], ne[:, i], 0) & 3) << (2 * i)
        meta |= per_side[:, i].astype(np.int64) << (9 + i)
        before = (sn[:, i] != cells) & (orig[sn[:, i]] < orig)
        meta |= before.astype(np.int64) << (12 + i)
    meta |= (full & 1) << 8
    meta |= (nbnd & 3) << 16
    conn = np.empty((N, 4), np.int32)
    conn[:, :3] = nb
    conn[:, 3] = meta
    surr = np.empty((N, 4), np.int32)
    surr[:, :3] = sn
    surr[:, 3] = nbnd

    # --- edge-once lists ---------------------------------------------------
    slot = 3 * cells[:, None] + np.arange(3)[None, :]
    opp_slot = 3 * nbc + nec
    owner = (~interior) | per_side | (interior & (cells[:, None] < nbc))
    edge_slot = slot[owner].astype(np.int32)
    opp = np.where(interior & ~per_side, opp_slot, -1)
    edge_opp = opp[owner].astype(np.int32)

    # --- extrapolation geometry --------------------------------------------
    C = np.asarray(mesh.centroid_coordinates, np.float64)
    Em = np.asarray(mesh.edge_midpoint_coordinates, np.float64).reshape(N, 3, 2)
    x = C[:, 0]
    y = C[:, 1]
    geo = np.zeros((N, GEO_STRIDE), np.float64)
    for i in range(3):
        geo[:, i] = Em[:, i, 0] - x
        geo[:, 3 + i] = Em[:, i, 1] - y
    x0, y0 = C[sn[:, 0], 0], C[sn[:, 0], 1]
    x1, y1 = C[sn[:, 1], 0], C[sn[:, 1], 1]
    x2, y2 = C[sn[:, 2], 0], C[sn[:, 2], 1]
    dx1 = x1 - x0
    dx2 = x2 - x0
    dy1 = y1 - y0
    dy2 = y2 - y0
    area2 = dy2 * dx1 - dy1 * dx2
    typical = nbnd <= 1
    with np.errstate(divide="ignore", invalid="ignore"):
        inv_area2 = 1.0 / area2
    geo[typical, 6] = dx1[typical]
    geo[typical, 7] = dx2[typical]
    geo[typical, 8] = dy1[typical]
    geo[typical, 9] = dy2[typical]
    geo[typical, 10] = inv_area2[typical]
    two = np.nonzero(nbnd == 2)[0]
    if two.size:
        s = sn[two]
        j = np.where(s[:, 0] != two, 0, np.where(s[:, 1] != two, 1, 2))
        kn = s[np.arange(two.size), j]
        ddx = C[kn, 0] - x[two]
        ddy = C[kn, 1] - y[two]
        dist2 = ddx * ddx + ddy * ddy
        gdx = 1.0 / dist2
        gdy = gdx * ddy
        gdx = gdx * ddx
        geo[two, 6] = gdx
        geo[two, 7] = gdy
    inv_area = 1.0 / np.asarray(mesh.areas, np.float64)
    bslot = (3 * np.asarray(mesh.boundary_cells, np.int64) + np.asarray(mesh.boundary_edges, np.int64)).astype(np.int32)
    return dict(conn=np.ascontiguousarray(conn), surr=np.ascontiguousarray(surr),
                geo=np.ascontiguousarray(geo), edge_slot=np.ascontiguousarray(edge_slot),
                edge_opp=np.ascontiguousarray(edge_opp), normals=np.ascontiguousarray(normals.ravel()),
                edgelengths=np.ascontiguousarray(lengths.ravel()),
                radii=np.ascontiguousarray(np.asarray(mesh.radii, np.float64)),
                areas=np.ascontiguousarray(np.asarray(mesh.areas, np.float64)),
                inv_area=np.ascontiguousarray(inv_area), boundary_slot=np.ascontiguousarray(bslot),
                vertex_coordinates=np.ascontiguousarray(np.asarray(mesh.vertex_coordinates, np.float64).ravel()))
