"""Triangle-mesh construction and geometry (host side).

Builds the same connectivity and geometry arrays as the reference's mesh
classes, with the same floating-point formulas so that every derived array is
bit-identical:

* ``rectangular_cross`` follows
  ``abstract_2d_finite_volumes/mesh_factory.py:138-175`` and
  ``mesh_factory_ext.pyx:8-90`` (4*m*n triangles, boundary tags on edge 1).
* ``Mesh`` follows ``general_mesh.py:134-267`` (areas, normals, edge lengths,
  centroids, radii, edge midpoints) and ``neighbour_mesh.py:70-505``
  (neighbours, neighbour edges, number of boundaries, surrogate neighbours,
  boundary dictionary and enumeration).

Geometry and neighbours are computed by the native builder
(``csrc/agx_mesh.cpp``: directed edges bucketed by their first vertex instead
of the reference's hash table in ``neighbour_table.cpp``; the result is
identical).  ``_geometry_numpy`` / ``_neighbours_numpy`` restate the same in
numpy for the tests.
"""
from __future__ import annotations

import numpy as np

DEFAULT_BOUNDARY_TAG = "exterior"   # anuga/config.py default_boundary_tag


def rectangular_cross(m, n, len1=1.0, len2=1.0, origin=(0.0, 0.0)):
    """Rectangular grid of m x n cells, each split into 4 triangles by its
    diagonals.  Returns ``(points, elements, boundary)`` like
    ``mesh_factory.rectangular_cross``."""
    m = int(m)
    n = int(n)
    len1 = float(len1)
    len2 = float(len2)
    ox, oy = float(origin[0]), float(origin[1])
    delta1 = len1 / m
    delta2 = len2 / n
    ngrid = (m + 1) * (n + 1)
    points = np.empty((ngrid + m * n, 2), dtype=float)
    ii, jj = np.meshgrid(np.arange(m + 1), np.arange(n + 1), indexing="ij")
    points[:ngrid, 0] = (ii.astype(float) * delta1 + ox).ravel()
    points[:ngrid, 1] = (jj.astype(float) * delta2 + oy).ravel()
    vid = np.arange(ngrid).reshape(m + 1, n + 1)
    ci, cj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    ci = ci.ravel()
    cj = cj.ravel()
    v1 = vid[ci, cj + 1]
    v2 = vid[ci, cj]
    v3 = vid[ci + 1, cj + 1]
    v4 = vid[ci + 1, cj]
    for d in range(2):
        s = points[v1, d] + points[v2, d]
        s = s + points[v3, d]
        s = s + points[v4, d]
        points[ngrid:, d] = s * 0.25
    v5 = ngrid + np.arange(m * n)
    elements = np.empty((4 * m * n, 3), dtype=np.int64)
    base = 4 * np.arange(m * n)
    elements[base + 0] = np.stack([v2, v5, v1], axis=1)   # left
    elements[base + 1] = np.stack([v4, v5, v2], axis=1)   # bottom
    elements[base + 2] = np.stack([v3, v5, v4], axis=1)   # right
    elements[base + 3] = np.stack([v1, v5, v3], axis=1)   # top
    boundary = {}
    cell = np.arange(m * n)
    for off, tag, mask in ((0, "left", ci == 0), (1, "bottom", cj == 0),
                           (2, "right", ci == m - 1), (3, "top", cj == n - 1)):
        for t in (4 * cell[mask] + off).tolist():
            boundary[(t, 1)] = tag
    return points, elements, boundary


class Mesh:
    """Connectivity and geometry of an unstructured triangle mesh.

    Attributes mirror the reference's ``Mesh`` object: ``nodes``,
    ``triangles``, ``vertex_coordinates`` [3N,2], ``edge_midpoint_coordinates``
    [3N,2], ``centroid_coordinates`` [N,2], ``normals`` [N,6],
    ``edgelengths`` [N,3], ``areas`` [N], ``radii`` [N], ``neighbours`` [N,3],
    ``neighbour_edges`` [N,3], ``number_of_boundaries`` [N],
    ``surrogate_neighbours`` [N,3], ``boundary`` {(vol, edge): tag},
    ``boundary_cells`` / ``boundary_edges`` [B], ``tag_boundary_cells``.
    """

    def __init__(self, coordinates, triangles, boundary=None, use_inscribed_circle=False):
        self.nodes = np.array(coordinates, dtype=float)
        self.triangles = np.array(triangles, dtype=np.int64)
        if self.triangles.ndim != 2 or self.triangles.shape[1] != 3:
            raise ValueError("triangles must be an N x 3 array")
        if self.triangles.size and self.triangles.max() >= self.nodes.shape[0]:
            raise ValueError("Vertex indices reference non-existing coordinate sets")
        self.use_inscribed_circle = use_inscribed_circle
        self.number_of_triangles = N = self.triangles.shape[0]
        self.number_of_nodes = self.nodes.shape[0]
        self._geometry()
        self._neighbours()
        self._boundary(boundary)

    def __len__(self):
        return self.number_of_triangles

    # general_mesh.py:134-267 (native: agx_mesh_geometry)
    def _geometry(self):
        from . import native
        g, bad = native.mesh_geometry(self.nodes, self.triangles, self.use_inscribed_circle)
        self.vertex_coordinates = g["V"]
        self.edge_midpoint_coordinates = g["E"]
        self.areas = g["areas"]
        if bad >= 0:
            raise ValueError("Degenerate Triangle(s) %s" % np.where(self.areas <= 0.0)[0][:20])
        self.normals = g["normals"]
        self.edgelengths = g["lengths"]
        self.centroid_coordinates = g["C"]
        self.radii = g["radii"]

    # neighbour_table.cpp + neighbour_mesh.py:296-346 (native: agx_mesh_neighbours)
    def _neighbours(self):
        from . import native
        N = self.number_of_triangles
        nb, ne, nbnd = native.mesh_neighbours(self.number_of_nodes, self.triangles)
        self.neighbours = nb
        self.neighbour_edges = ne
        self.number_of_boundaries = nbnd
        rng = np.arange(N, dtype=np.int64)[:, None]
        self.surrogate_neighbours = np.where(self.neighbours < 0, rng, self.neighbours)

    # numpy restatement of _geometry (the reference the native builder is tested against)
    def _geometry_numpy(self):
        N = self.number_of_triangles
        tri = self.triangles
        V = np.zeros((3 * N, 2), dtype=float)
        V[0::3] = self.nodes[tri[:, 0]]
        V[1::3] = self.nodes[tri[:, 1]]
        V[2::3] = self.nodes[tri[:, 2]]
        self.vertex_coordinates = V
        E = np.zeros((3 * N, 2), dtype=float)
        V0, V1, V2 = V[0::3], V[1::3], V[2::3]
        E[0::3] = 0.5 * (V1 + V2)
        E[1::3] = 0.5 * (V2 + V0)
        E[2::3] = 0.5 * (V0 + V1)
        self.edge_midpoint_coordinates = E
        x0, y0 = V0[:, 0], V0[:, 1]
        x1, y1 = V1[:, 0], V1[:, 1]
        x2, y2 = V2[:, 0], V2[:, 1]
        self.areas = -((x1 * y0 - x0 * y1) + (x2 * y1 - x1 * y2) + (x0 * y2 - x2 * y0)) / 2.0
        if N and not np.all(self.areas > 0.0):
            bad = np.where(self.areas <= 0.0)[0]
            raise ValueError("Degenerate Triangle(s) %s" % bad[:20])
        normals = np.zeros((N, 6), dtype=float)
        lengths = np.zeros((N, 3), dtype=float)
        for i, (xa, ya, xb, yb) in enumerate(((x1, y1, x2, y2), (x2, y2, x0, y0), (x0, y0, x1, y1))):
            xn = xb - xa
            yn = yb - ya
            ln = np.sqrt(xn * xn + yn * yn)
            xn = xn / ln
            yn = yn / ln
            normals[:, 2 * i] = yn
            normals[:, 2 * i + 1] = -xn
            lengths[:, i] = ln
        self.normals = normals
        self.edgelengths = lengths
        C = np.zeros((N, 2), dtype=float)
        C[:, 0] = (x0 + x1 + x2) / 3
        C[:, 1] = (y0 + y1 + y2) / 3
        self.centroid_coordinates = C
        if not self.use_inscribed_circle:
            xm0 = (x1 + x2) / 2
            ym0 = (y1 + y2) / 2
            xm1 = (x2 + x0) / 2
            ym1 = (y2 + y0) / 2
            xm2 = (x0 + x1) / 2
            ym2 = (y0 + y1) / 2
            d0 = np.sqrt((C[:, 0] - xm0) ** 2 + (C[:, 1] - ym0) ** 2)
            d1 = np.sqrt((C[:, 0] - xm1) ** 2 + (C[:, 1] - ym1) ** 2)
            d2 = np.sqrt((C[:, 0] - xm2) ** 2 + (C[:, 1] - ym2) ** 2)
            self.radii = np.minimum(np.minimum(d0, d1), d2)
        else:
            a = np.sqrt((x0 - x1) ** 2 + (y0 - y1) ** 2)
            b = np.sqrt((x1 - x2) ** 2 + (y1 - y2) ** 2)
            c = np.sqrt((x2 - x0) ** 2 + (y2 - y0) ** 2)
            self.radii = 2.0 * self.areas / (a + b + c)

    # numpy restatement of _neighbours (the reference the native builder is tested against)
    def _neighbours_numpy(self):
        N = self.number_of_triangles
        tri = self.triangles
        M = np.int64(max(self.number_of_nodes, 1))
        # directed edge i of triangle k: (v[(i+1)%3], v[(i+2)%3])
        a = np.stack([tri[:, 1], tri[:, 2], tri[:, 0]], axis=1).ravel()
        b = np.stack([tri[:, 2], tri[:, 0], tri[:, 1]], axis=1).ravel()
        key = a * M + b
        order = np.argsort(key, kind="stable")
        skey = key[order]
        if skey.size > 1 and np.any(skey[1:] == skey[:-1]):
            raise ValueError("Inconsistent mesh: a directed edge appears twice "
                             "(triangles not consistently oriented)")
        rkey = b * M + a
        pos = np.searchsorted(skey, rkey)
        pos = np.minimum(pos, max(skey.size - 1, 0))
        found = skey[pos] == rkey if skey.size else np.zeros(0, bool)
        nb = np.full(3 * N, -1, dtype=np.int64)
        ne = np.full(3 * N, -1, dtype=np.int64)
        hit = order[pos[found]]
        nb[found] = hit // 3
        ne[found] = hit % 3
        self.neighbours = nb.reshape(N, 3)
        self.neighbour_edges = ne.reshape(N, 3)
        self.number_of_boundaries = (3 - found.reshape(N, 3).sum(axis=1)).astype(np.int64)
        rng = np.arange(N, dtype=np.int64)[:, None]
        self.surrogate_neighbours = np.where(self.neighbours < 0, rng, self.neighbours)

    # neighbour_mesh.py:352-505 and neighbour_mesh_ext.pyx boundary_dictionary_construct
    def _boundary(self, boundary):
        N = self.number_of_triangles
        boundary = {} if boundary is None else dict(boundary)
        for (vol, edge) in boundary:
            if not (0 <= vol < N and 0 <= edge < 3):
                raise ValueError("Segment (%d, %d) does not exist" % (vol, edge))
        vols, edges = np.nonzero(self.neighbours < 0)
        for v, e in zip(vols.tolist(), edges.tolist()):
            boundary.setdefault((v, e), DEFAULT_BOUNDARY_TAG)
        self.boundary = boundary
        keys = sorted(boundary.keys())
        B = len(keys)
        self.boundary_length = B
        if B:
            arr = np.array(keys, dtype=np.int64)
            self.boundary_cells = arr[:, 0].copy()
            self.boundary_edges = arr[:, 1].copy()
        else:
            self.boundary_cells = np.zeros(0, np.int64)
            self.boundary_edges = np.zeros(0, np.int64)
        self.neighbours[self.boundary_cells, self.boundary_edges] = -np.arange(1, B + 1, dtype=np.int64)
        tags = sorted(set(boundary.values()))
        self.tag_boundary_cells = {t: [] for t in tags}
        tag_of = [boundary[k] for k in keys]
        for j, t in enumerate(tag_of):
            self.tag_boundary_cells[t].append(j)

    def get_boundary_tags(self):
        return sorted(set(self.boundary.values()))

    def get_vertex_coordinates(self):
        return self.vertex_coordinates

    def get_centroid_coordinates(self):
        return self.centroid_coordinates

    def get_edge_midpoint_coordinates(self):
        return self.edge_midpoint_coordinates

    def get_area(self):
        return float(np.sum(self.areas))
