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


def pack_tables_numpy(mesh, tri_full_flag=None, per_side_edges=None, order=None):
    """numpy restatement of :func:`pack_tables` (the tests' reference).

    Return a dict of numpy arrays for ``agx_scenario_create``.

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


def morton_order_numpy(points, bits=16):
    """Cell order along a Morton (Z-order) curve of the centroids, so that
    tiles of consecutive cells are compact patches of the mesh."""
    P = np.asarray(points, np.float64)
    lo = P.min(axis=0)
    span = np.maximum(P.max(axis=0) - lo, 1e-300)
    q = np.clip(((P - lo) / span * ((1 << bits) - 1)).astype(np.uint64), 0, (1 << bits) - 1)

    def spread(v):
        v = v & np.uint64(0xFFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
        return v
    key = spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1))
    return np.argsort(key, kind="stable")


def pack_mixed_numpy(mesh, order=None):
    """FP32 tables of the mixed-precision form, cells in Morton order.

    Returns conn int32 [N,4] (neighbours in the stored order, boundary edges as
    -(m+1) with the mesh's boundary index m, meta word), geo float32 [N,16]
    (jump matrix M row-major in g0.xyzw g1.xyzw g2.x, edge vectors in
    g2.yzw g3.xyz, radius in g3.w), area [N], radius [N] (FP64), order [N]
    (original index of each stored cell) and boundary_cell [B] (stored index).

    The jump matrix maps the differences to the three surrogate neighbours,
    Dq_j = q_{s_j} - q_k, to the provisional edge jumps; it is the linear
    gradient of sw_domain_openmp.c:1445-1484 (auxiliary triangle, one boundary
    or none) or :1684-1696 (two boundaries) evaluated at the edge midpoints.
    """
    N = len(mesh)
    nb = np.asarray(mesh.neighbours, np.int64)
    ne = np.asarray(mesh.neighbour_edges, np.int64)
    sn = np.asarray(mesh.surrogate_neighbours, np.int64)
    nbnd = np.asarray(mesh.number_of_boundaries, np.int64)
    cells = np.arange(N, dtype=np.int64)
    expected = np.where(nb >= 0, nb, cells[:, None])
    if not np.array_equal(expected, sn):
        raise NotImplementedError("the mixed-precision form needs surrogate neighbours equal to the "
                                  "flux neighbours (no internal boundary segments)")
    if order is None:
        order, _name, _costs = best_order_numpy(mesh)
    order = np.asarray(order, np.int64)
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    C = np.asarray(mesh.centroid_coordinates, np.float64)
    Em = np.asarray(mesh.edge_midpoint_coordinates, np.float64).reshape(N, 3, 2)
    V = np.asarray(mesh.vertex_coordinates, np.float64).reshape(N, 3, 2)
    dxv = Em[:, :, 0] - C[:, 0:1]
    dyv = Em[:, :, 1] - C[:, 1:2]
    M = np.zeros((N, 3, 3))
    x0, y0 = C[sn[:, 0], 0], C[sn[:, 0], 1]
    x1, y1 = C[sn[:, 1], 0], C[sn[:, 1], 1]
    x2, y2 = C[sn[:, 2], 0], C[sn[:, 2], 1]
    dx1, dx2, dy1, dy2 = x1 - x0, x2 - x0, y1 - y0, y2 - y0
    area2 = dy2 * dx1 - dy1 * dx2
    typ = nbnd <= 1
    with np.errstate(divide="ignore", invalid="ignore"):
        ia2 = np.where(typ, 1.0 / area2, 0.0)
    cx = np.stack([dy1 - dy2, dy2, -dy1], axis=1) * ia2[:, None]
    cy = np.stack([dx2 - dx1, -dx2, dx1], axis=1) * ia2[:, None]
    for i in range(3):
        M[:, i, :] = cx * dxv[:, i:i + 1] + cy * dyv[:, i:i + 1]
    M[~typ] = 0.0
    two = np.nonzero(nbnd == 2)[0]
    if two.size:
        s = sn[two]
        j = np.where(s[:, 0] != two, 0, np.where(s[:, 1] != two, 1, 2))
        kn = s[np.arange(two.size), j]
        ddx = C[kn, 0] - C[two, 0]
        ddy = C[kn, 1] - C[two, 1]
        dist2 = ddx * ddx + ddy * ddy
        gdx = ddx / dist2
        gdy = ddy / dist2
        for i in range(3):
            M[two, i, j] = gdx * dxv[two, i] + gdy * dyv[two, i]
    ev = np.stack([V[:, 2] - V[:, 1], V[:, 0] - V[:, 2], V[:, 1] - V[:, 0]], axis=1)   # [N,3,2]
    geo = np.zeros((N, 16), np.float32)
    Mf = M.reshape(N, 9)
    geo[:, 0:9] = Mf
    geo[:, 9] = ev[:, 0, 0]
    geo[:, 10] = ev[:, 0, 1]
    geo[:, 11] = ev[:, 1, 0]
    geo[:, 12] = ev[:, 1, 1]
    geo[:, 13] = ev[:, 2, 0]
    geo[:, 14] = ev[:, 2, 1]
    geo[:, 15] = np.asarray(mesh.radii, np.float64)
    meta = np.zeros(N, np.int64)
    for i in range(3):
        meta |= (np.where(nb[:, i] >= 0, ne[:, i], 0) & 3) << (2 * i)
    meta |= 1 << 8
    meta |= (nbnd & 3) << 16
    conn = np.empty((N, 4), np.int64)
    nbr_new = np.where(nb >= 0, inv[np.where(nb >= 0, nb, 0)], nb)
    conn[:, :3] = nbr_new
    conn[:, 3] = meta
    bcell = inv[np.asarray(mesh.boundary_cells, np.int64)]
    conn_s = np.ascontiguousarray(conn[order].astype(np.int32))
    lnk, hoff, hcnt, hcells = tile_halos_numpy(conn_s)
    return dict(conn=conn_s, lnk=lnk, halo_off=hoff, halo_cnt=hcnt, halo_cells=hcells,
                geo=np.ascontiguousarray(geo[order]),
                area=np.ascontiguousarray(np.asarray(mesh.areas, np.float64)[order]),
                radius=np.ascontiguousarray(np.asarray(mesh.radii, np.float64)[order]),
                order=np.ascontiguousarray(order.astype(np.int32)),
                boundary_cell=np.ascontiguousarray(bcell.astype(np.int32)))


TILE = 128
HALO_MAX = 128          # halo cells a tile can stage in shared memory
LNK_INLINE = 1023       # local index meaning "reconstruct this neighbour inline"


def tile_halos_numpy(conn, tile=TILE, halo_max=HALO_MAX):
    """Per tile of `tile` consecutive cells: the outside cells whose edges the
    tile's fluxes need (its halo), and for every cell slot the local index of
    the neighbour in the tile's staging area (own cells 0..tile-1, halo cells
    tile..tile+H-1, boundary edges LNK_INLINE, packed 10 bits per slot).

    Returns (lnk int32 [N], halo_off int32 [T], halo_cnt int32 [T],
    halo_cells int32 [sum H])."""
    N = conn.shape[0]
    T = (N + tile - 1) // tile
    nbr = conn[:, :3].astype(np.int64)
    cells = np.arange(N, dtype=np.int64)
    tcell = cells // tile
    local = np.full((N, 3), LNK_INLINE, np.int64)
    inside = (nbr >= 0) & (nbr // tile == tcell[:, None])
    local[inside] = (nbr - (tcell * tile)[:, None])[inside]
    ext = (nbr >= 0) & ~inside
    ek, ei = np.nonzero(ext)
    et = tcell[ek]
    en = nbr[ek, ei]
    key = et * (N + 1) + en
    uk, inv = np.unique(key, return_inverse=True)
    ut = uk // (N + 1)
    un = uk % (N + 1)
    cnt = np.bincount(ut, minlength=T)
    off = np.zeros(T, np.int64)
    off[1:] = np.cumsum(cnt)[:-1]
    pos = np.arange(uk.size) - off[ut]           # position of each halo cell in its tile's list
    hpos = pos[inv]
    ok = hpos < halo_max
    local[ek[ok], ei[ok]] = tile + hpos[ok]
    lnk = local[:, 0] | (local[:, 1] << 10) | (local[:, 2] << 20)
    cnt_clamped = np.minimum(cnt, halo_max)
    # keep only the first halo_max cells of each tile (the rest are reconstructed inline)
    keep = pos < halo_max
    hc = un[keep]
    off2 = np.zeros(T, np.int64)
    off2[1:] = np.cumsum(cnt_clamped)[:-1]
    return (lnk.astype(np.int32), off2.astype(np.int32), cnt_clamped.astype(np.int32), hc.astype(np.int32))


def hilbert_order_numpy(points, bits=16):
    """Cell order along a Hilbert curve of the centroids (better locality
    than Morton: consecutive cells are always adjacent patches)."""
    P = np.asarray(points, np.float64)
    lo = P.min(axis=0)
    span = np.maximum(P.max(axis=0) - lo, 1e-300)
    n = 1 << bits
    x = np.clip(((P[:, 0] - lo[0]) / span[0] * (n - 1)).astype(np.int64), 0, n - 1)
    y = np.clip(((P[:, 1] - lo[1]) / span[1] * (n - 1)).astype(np.int64), 0, n - 1)
    d = np.zeros(len(P), np.int64)
    s = n // 2
    while s > 0:
        rx = (x & s) > 0
        ry = (y & s) > 0
        d += s * s * ((3 * rx) ^ ry)
        # rotate the quadrant
        flip = ~ry
        swap_x = np.where(flip & rx, s - 1 - x, x)
        swap_y = np.where(flip & rx, s - 1 - y, y)
        x = np.where(flip, swap_y, swap_x)
        y = np.where(flip, swap_x, swap_y)
        s //= 2
    return np.argsort(d, kind="stable")


def halo_cost_numpy(mesh, order, tile=TILE):
    """Fraction of extra reconstructions (halo cells per own cell) of an order."""
    N = len(mesh)
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    nb = np.asarray(mesh.neighbours, np.int64)[order]
    conn = np.where(nb >= 0, inv[np.where(nb >= 0, nb, 0)], -1)
    k = np.arange(N)[:, None]
    ext = (conn >= 0) & (conn // tile != k // tile)
    pairs = np.unique((k // tile * (N + 1) + conn)[ext])
    return pairs.size / max(N, 1)


def best_order_numpy(mesh, tile=TILE):
    """numpy restatement of :func:`best_order`."""
    C = mesh.centroid_coordinates
    cands = {"hilbert": hilbert_order_numpy(C), "morton": morton_order_numpy(C)}
    costs = {k: halo_cost_numpy(mesh, v, tile) for k, v in cands.items()}
    name = min(costs, key=costs.get)
    return cands[name], name, costs


# ---------------------------------------------------------------------------
# Native builders (csrc/agx_mesh.cpp): the product path.  Each computes the
# same bits as its *_numpy restatement above.

def pack_tables(mesh, tri_full_flag=None, per_side_edges=None, order=None):
    """Return a dict of numpy arrays for ``agx_scenario_create``.

    per_side_edges: optional bool [N,3] forcing per-side evaluation of slots
    (used for low-Froude scaling and riverwalls, where the edge flux is not
    antisymmetric).  order: original index of each cell (for the ordering
    bits); defaults to the identity.
    """
    from . import native
    N = len(mesh)
    if N >= (1 << 29):
        raise ValueError("mesh too large for 32-bit slot indices")
    normals = np.asarray(mesh.normals, np.float64)
    lengths = np.asarray(mesh.edgelengths, np.float64)
    conn, surr, geo, edge_slot, edge_opp = native.pack_plain(
        N, mesh.neighbours, mesh.neighbour_edges, mesh.surrogate_neighbours, mesh.number_of_boundaries,
        tri_full_flag, per_side_edges, order, normals, lengths, mesh.centroid_coordinates,
        mesh.edge_midpoint_coordinates)
    inv_area = 1.0 / np.asarray(mesh.areas, np.float64)
    bslot = (3 * np.asarray(mesh.boundary_cells, np.int64) + np.asarray(mesh.boundary_edges, np.int64)).astype(np.int32)
    return dict(conn=conn, surr=surr, geo=geo, edge_slot=edge_slot, edge_opp=edge_opp,
                normals=np.ascontiguousarray(normals.ravel()), edgelengths=np.ascontiguousarray(lengths.ravel()),
                radii=np.ascontiguousarray(np.asarray(mesh.radii, np.float64)),
                areas=np.ascontiguousarray(np.asarray(mesh.areas, np.float64)),
                inv_area=np.ascontiguousarray(inv_area), boundary_slot=np.ascontiguousarray(bslot),
                vertex_coordinates=np.ascontiguousarray(np.asarray(mesh.vertex_coordinates, np.float64).ravel()))


def morton_order(points, bits=16):
    """Cell order along a Morton (Z-order) curve of the centroids, so that
    tiles of consecutive cells are compact patches of the mesh."""
    from . import native
    return native.sfc_order(points, "morton", bits)


def hilbert_order(points, bits=16):
    """Cell order along a Hilbert curve of the centroids (better locality
    than Morton: consecutive cells are always adjacent patches)."""
    from . import native
    return native.sfc_order(points, "hilbert", bits)


def tile_halos(conn, tile=TILE, halo_max=HALO_MAX):
    """Per tile of `tile` consecutive cells: the outside cells whose edges the
    tile's fluxes need (its halo), and for every cell slot the local index of
    the neighbour in the tile's staging area (own cells 0..tile-1, halo cells
    tile..tile+H-1, boundary edges LNK_INLINE, packed 10 bits per slot).

    Returns (lnk int32 [N], halo_off int32 [T], halo_cnt int32 [T],
    halo_cells int32 [sum H])."""
    from . import native
    lnk, off, cnt, hc, _unclamped = native.tile_halos(conn, tile, halo_max, LNK_INLINE)
    return lnk, off, cnt, hc


def _stored_conn(mesh, order):
    N = len(mesh)
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    nb = np.asarray(mesh.neighbours, np.int64)[order]
    conn = np.zeros((N, 4), np.int32)
    conn[:, :3] = np.where(nb >= 0, inv[np.where(nb >= 0, nb, 0)], -1)
    return conn


def halo_cost(mesh, order, tile=TILE):
    """Fraction of extra reconstructions (halo cells per own cell) of an order."""
    from . import native
    return native.tile_halos(_stored_conn(mesh, order), tile, HALO_MAX, LNK_INLINE, count_only=True) / max(len(mesh), 1)


def best_order(mesh, tile=TILE):
    """The cheaper of the Morton and Hilbert orders by halo cost (the
    reordering choice of the autotuner); returns (order, name, costs)."""
    C = mesh.centroid_coordinates
    cands = {"hilbert": hilbert_order(C), "morton": morton_order(C)}
    costs = {k: halo_cost(mesh, v, tile) for k, v in cands.items()}
    name = min(costs, key=costs.get)
    return cands[name], name, costs


def pack_mixed(mesh, order=None):
    """FP32 tables of the mixed-precision form, cells in a space-filling-curve
    order (see :func:`pack_mixed_numpy` for the layout; same arrays, built by
    the native builder)."""
    from . import native
    N = len(mesh)
    nb = np.asarray(mesh.neighbours, np.int64)
    sn = np.asarray(mesh.surrogate_neighbours, np.int64)
    cells = np.arange(N, dtype=np.int64)
    expected = np.where(nb >= 0, nb, cells[:, None])
    if not np.array_equal(expected, sn):
        raise NotImplementedError("the mixed-precision form needs surrogate neighbours equal to the "
                                  "flux neighbours (no internal boundary segments)")
    if order is None:
        order, _name, _costs = best_order(mesh)
    order = np.asarray(order, np.int64)
    conn_s, geo, area_s, order_s = native.pack_mixed(
        order, nb, mesh.neighbour_edges, sn, mesh.number_of_boundaries, mesh.centroid_coordinates,
        mesh.edge_midpoint_coordinates, mesh.vertex_coordinates, mesh.radii, mesh.areas)
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    bcell = inv[np.asarray(mesh.boundary_cells, np.int64)]
    lnk, hoff, hcnt, hcells = tile_halos(conn_s)
    return dict(conn=conn_s, lnk=lnk, halo_off=hoff, halo_cnt=hcnt, halo_cells=hcells, geo=geo, area=area_s,
                radius=np.ascontiguousarray(np.asarray(mesh.radii, np.float64)[order]),
                order=order_s, boundary_cell=np.ascontiguousarray(bcell.astype(np.int32)))
