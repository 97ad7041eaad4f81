"""Invariants of the device tables built on the host."""
import numpy as np
import pytest

from anuga_core_gb300.mesh import Mesh, rectangular_cross
from anuga_core_gb300.tables import pack_tables


def _delaunay(n, seed):
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 100, (n, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    return Mesh(pts, tri)


@pytest.mark.parametrize("mesh", [Mesh(*rectangular_cross(9, 7, 9.0, 7.0)), _delaunay(500, 2)],
                         ids=["rect", "delaunay"])
def test_every_slot_gets_exactly_one_flux(mesh):
    T = pack_tables(mesh)
    N = len(mesh)
    cover = np.zeros(3 * N, int)
    np.add.at(cover, T["edge_slot"], 1)
    opp = T["edge_opp"]
    np.add.at(cover, opp[opp >= 0], 1)
    assert cover.min() == 1 and cover.max() == 1
    # the opposite slot is the neighbour's back edge
    es = T["edge_slot"][opp >= 0]
    k, i = es // 3, es % 3
    n = mesh.neighbours[k, i]
    assert np.array_equal(opp[opp >= 0], 3 * n + mesh.neighbour_edges[k, i])


def test_meta_word_round_trips():
    mesh = _delaunay(400, 3)
    T = pack_tables(mesh)
    meta = T["conn"][:, 3].astype(np.int64)
    for i in range(3):
        ne = (meta >> (2 * i)) & 3
        interior = mesh.neighbours[:, i] >= 0
        assert np.array_equal(ne[interior], mesh.neighbour_edges[interior, i])
    assert np.array_equal((meta >> 16) & 3, mesh.number_of_boundaries)
    assert np.all(((meta >> 8) & 1) == 1)
    assert np.array_equal(T["surr"][:, :3], mesh.surrogate_neighbours)


def test_low_froude_forces_per_side_evaluation():
    mesh = Mesh(*rectangular_cross(4, 4, 4.0, 4.0))
    T = pack_tables(mesh, per_side_edges=np.ones((len(mesh), 3), bool))
    assert np.all(T["edge_opp"] == -1)
    assert T["edge_slot"].size == 3 * len(mesh)


@pytest.mark.parametrize("mesh", [Mesh(*rectangular_cross(60, 50, 60.0, 50.0)), _delaunay(3000, 4)],
                         ids=["rect", "delaunay"])
def test_mixed_tables_and_tile_halos(mesh):
    from anuga_core_gb300.tables import pack_mixed, TILE, LNK_INLINE
    T = pack_mixed(mesh)
    N = len(mesh)
    order = T["order"]
    assert np.array_equal(np.sort(order), np.arange(N))
    conn = T["conn"]
    inv = np.empty(N, np.int64)
    inv[order] = np.arange(N)
    # neighbours are the mesh's, renumbered
    nb = mesh.neighbours[order]
    assert np.array_equal(conn[:, :3][nb >= 0], inv[nb[nb >= 0]])
    lnk, off, cnt, hc = T["lnk"], T["halo_off"], T["halo_cnt"], T["halo_cells"]
    for k in range(0, N, 7):
        t = k // TILE
        for i in range(3):
            li = (int(lnk[k]) >> (10 * i)) & 1023
            n = conn[k, i]
            if n < 0:
                assert li == LNK_INLINE
            elif li < TILE:
                assert n == t * TILE + li
            elif li != LNK_INLINE:
                assert hc[off[t] + li - TILE] == n
    # the jump matrix reproduces a linear field exactly at the edge midpoints
    C = mesh.centroid_coordinates[order]
    E = mesh.edge_midpoint_coordinates.reshape(-1, 3, 2)[order]
    f = lambda x, y: 0.3 * x - 0.7 * y
    M = T["geo"][:, :9].astype(np.float64).reshape(-1, 3, 3)
    s = np.where(conn[:, :3] >= 0, conn[:, :3], np.arange(N)[:, None])
    D = f(C[s, 0], C[s, 1]) - f(C[:, 0], C[:, 1])[:, None]
    J = np.einsum("kij,kj->ki", M, D)
    exact = f(E[:, :, 0], E[:, :, 1]) - f(C[:, 0], C[:, 1])[:, None]
    typical = mesh.number_of_boundaries[order] == 0
    assert np.allclose(J[typical], exact[typical], atol=1e-4 * (1 + np.abs(exact[typical]).max()))
