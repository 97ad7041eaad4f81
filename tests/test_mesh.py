"""Mesh construction and geometry match the reference's arrays bit for bit
(golden fixtures written from the reference Domain)."""
import numpy as np
import pytest

from anuga_core_gb300.mesh import Mesh, rectangular_cross

KEYS = ["vertex_coordinates", "edge_midpoint_coordinates", "centroid_coordinates", "normals", "edgelengths",
        "areas", "radii", "neighbours", "neighbour_edges", "number_of_boundaries", "surrogate_neighbours",
        "boundary_cells", "boundary_edges"]


@pytest.mark.parametrize("name", ["mesh_rect_3x2.npz", "mesh_delaunay_300.npz"])
def test_mesh_arrays_match_reference(golden, name):
    f = golden(name)
    boundary = None
    if name.startswith("mesh_rect"):
        p, e, boundary = rectangular_cross(3, 2, 3.0, 2.0)
        assert np.array_equal(p, f["points"]) and np.array_equal(e, f["elements"])
    M = Mesh(f["points"], f["elements"], boundary)
    for k in KEYS:
        assert np.array_equal(np.asarray(getattr(M, k)), f[k]), k
    assert np.array_equal(np.array(sorted(M.boundary), np.int64).reshape(-1, 2), f["boundary_keys"])


def test_rectangular_cross_counts():
    p, e, b = rectangular_cross(7, 5, 70.0, 50.0)
    assert e.shape == (4 * 35, 3)
    assert p.shape == (8 * 6 + 35, 2)
    tags = {}
    for v in b.values():
        tags[v] = tags.get(v, 0) + 1
    assert tags == {"left": 5, "right": 5, "bottom": 7, "top": 7}
    M = Mesh(p, e, b)
    assert np.all(M.areas > 0)
    assert np.isclose(M.areas.sum(), 70.0 * 50.0)


def test_inconsistent_orientation_rejected():
    p = np.array([[0, 0], [1, 0], [0, 1], [1, 1.0]])
    e = np.array([[0, 1, 2], [1, 2, 3]])    # second triangle is clockwise -> degenerate area check
    with pytest.raises(ValueError):
        Mesh(p, e)


def test_polygon_mesh_meets_its_area_limits():
    from anuga_core_gb300.geometry import inside_polygon
    from anuga_core_gb300.workloads import polygon_mesh, value_noise
    mesh, info = polygon_mesh(2.0e4, seed=7)
    assert abs(len(mesh) - 2.0e4) < 0.15 * 2.0e4
    assert mesh.areas.min() > 0.0 and mesh.areas.max() <= 50.0 + 1e-9
    inner = np.array(info["refined"])
    fine = inside_polygon(mesh.centroid_coordinates, inner)
    assert fine.size > 0 and mesh.areas[fine].max() <= 12.5 + 1e-9
    assert "inflow" in mesh.tag_boundary_cells and "wall" in mesh.tag_boundary_cells
    z = value_noise(mesh.nodes[:, 0], mesh.nodes[:, 1], seed=7)
    assert abs(z.min() + 10.0) < 1e-9 and abs(z.max() - 30.0) < 1e-9
    again, _ = polygon_mesh(2.0e4, seed=7)
    assert np.array_equal(again.triangles, mesh.triangles)
