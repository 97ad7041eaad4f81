"""The native host builders (csrc/agx_mesh.cpp) give the same bits as the
numpy restatements in mesh.py / tables.py (no GPU needed)."""
import copy

import numpy as np
import pytest

from anuga_core_gb300 import tables
from anuga_core_gb300.mesh import Mesh, rectangular_cross


def _meshes():
    from anuga_core_gb300.serve import delaunay_mesh
    from anuga_core_gb300.workloads import polygon_mesh
    p, e, b = rectangular_cross(37, 23, 370.0, 230.0)
    yield "rect", Mesh(p, e, b)
    yield "delaunay", delaunay_mesh(6000, seed=4)
    yield "polygon", polygon_mesh(8000, seed=3)[0]
    rng = np.random.default_rng(1)
    from scipy.spatial import Delaunay
    pts = rng.uniform(0, 100, (400, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    yield "random", Mesh(pts, tri)


MESHES = list(_meshes())


@pytest.mark.parametrize("name,mesh", MESHES, ids=[m[0] for m in MESHES])
def test_geometry_and_neighbours_match_numpy(name, mesh):
    ref = copy.copy(mesh)
    ref._geometry_numpy()
    ref._neighbours_numpy()
    for k in ("vertex_coordinates", "edge_midpoint_coordinates", "areas", "normals", "edgelengths",
              "centroid_coordinates", "radii", "neighbour_edges", "number_of_boundaries", "surrogate_neighbours"):
        assert np.array_equal(getattr(mesh, k), getattr(ref, k)), k
    nb = np.where(mesh.neighbours < 0, -1, mesh.neighbours)
    assert np.array_equal(nb, ref.neighbours), "neighbours"


@pytest.mark.parametrize("name,mesh", MESHES, ids=[m[0] for m in MESHES])
def test_tables_match_numpy(name, mesh):
    rng = np.random.default_rng(7)
    N = len(mesh)
    full = (rng.uniform(size=N) < 0.9).astype(np.int64)
    per_side = rng.uniform(size=(N, 3)) < 0.05
    order = rng.permutation(N)
    for kw in ({}, dict(tri_full_flag=full, per_side_edges=per_side, order=order)):
        a = tables.pack_tables(mesh, **kw)
        b = tables.pack_tables_numpy(mesh, **kw)
        for k in b:
            assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k], equal_nan=True), (k, kw.keys())
    C = mesh.centroid_coordinates
    assert np.array_equal(tables.hilbert_order(C), tables.hilbert_order_numpy(C))
    assert np.array_equal(tables.morton_order(C), tables.morton_order_numpy(C))
    for curve in (tables.hilbert_order(C), tables.morton_order(C)):
        assert tables.halo_cost(mesh, curve) == tables.halo_cost_numpy(mesh, curve)
    a = tables.pack_mixed(mesh)
    b = tables.pack_mixed_numpy(mesh)
    for k in b:
        assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k], equal_nan=True), k


def test_builder_errors_match_numpy():
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [2.0, 0.0]])
    with pytest.raises(ValueError, match="Degenerate"):
        Mesh(pts, [[0, 2, 1]])                      # clockwise: negative area
    with pytest.raises(ValueError, match="Inconsistent"):
        Mesh(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]]), [[0, 1, 2], [0, 1, 3]])
    with pytest.raises(ValueError):
        Mesh(pts, [[0, 1, 7]])
