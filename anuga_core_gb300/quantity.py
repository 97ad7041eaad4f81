"""Quantity: host mirror of one field of a Domain, backed by device memory.

Mirrors the public interface of the reference's
``abstract_2d_finite_volumes/quantity.py:28-117`` (``centroid_values``,
``edge_values``, ``vertex_values``, ``boundary_values``, ``explicit_update``,
``semi_implicit_update``, ``set_values``, ``get_values``).  The arrays live
on the GPU while the domain evolves; the host copies are refreshed on access
(and, for the conserved quantities, at every yield), and host edits are sent
back before the next device operation.
"""
from __future__ import annotations

import numpy as np

# which device fields back each quantity: (centroid, edge, vertex, boundary, explicit, semi)
DEVICE_FIELDS = {
    "stage": ("stage_c", "stage_e", "stage_v", "stage_b", "stage_x", "stage_s"),
    "xmomentum": ("xmom_c", "xmom_e", "xmom_v", "xmom_b", "xmom_x", "xmom_s"),
    "ymomentum": ("ymom_c", "ymom_e", "ymom_v", "ymom_b", "ymom_x", "ymom_s"),
    "elevation": ("elev_c", "elev_e", "elev_v", None, None, None),
    "friction": ("friction_c", None, None, None, None, None),
    "height": ("height_c", "height_e", "height_v", None, None, None),
}
_SLOTS = ("centroid_values", "edge_values", "vertex_values", "boundary_values", "explicit_update",
          "semi_implicit_update")


class Quantity:
    def __init__(self, domain, name):
        self.domain = domain
        self.name = name
        N = len(domain)
        B = domain.mesh.boundary_length
        self._arr = {
            "centroid_values": np.zeros(N),
            "edge_values": np.zeros((N, 3)),
            "vertex_values": np.zeros((N, 3)),
            "boundary_values": np.zeros(B),
            "explicit_update": np.zeros(N),
            "semi_implicit_update": np.zeros(N),
        }
        fields = DEVICE_FIELDS.get(name, (None,) * 6)
        self._field = dict(zip(_SLOTS, fields))

    def __len__(self):
        return len(self._arr["centroid_values"])

    # -- synchronised array access -----------------------------------------
    def _get(self, slot):
        f = self._field[slot]
        if f is not None:
            self.domain._host_view(f, self._arr[slot])
        elif self.name in ("xvelocity", "yvelocity"):
            self.domain._refresh_velocity(self, slot)
        return self._arr[slot]

    def _set(self, slot, value):
        a = self._arr[slot]
        a[...] = np.asarray(value, dtype=float).reshape(a.shape)
        f = self._field[slot]
        if f is not None:
            self.domain._host_modified(f)

    centroid_values = property(lambda s: s._get("centroid_values"), lambda s, v: s._set("centroid_values", v))
    edge_values = property(lambda s: s._get("edge_values"), lambda s, v: s._set("edge_values", v))
    vertex_values = property(lambda s: s._get("vertex_values"), lambda s, v: s._set("vertex_values", v))
    boundary_values = property(lambda s: s._get("boundary_values"), lambda s, v: s._set("boundary_values", v))
    explicit_update = property(lambda s: s._get("explicit_update"), lambda s, v: s._set("explicit_update", v))
    semi_implicit_update = property(lambda s: s._get("semi_implicit_update"),
                                    lambda s, v: s._set("semi_implicit_update", v))

    # -- setting values (quantity.py:709-1195) -----------------------------
    def set_values(self, numeric=None, quantity=None, function=None, location="vertices",
                   indices=None, polygon=None, **kwargs):
        if location not in ("vertices", "centroids", "unique vertices"):
            raise ValueError("Invalid location: %s" % location)
        if polygon is not None:
            if indices is not None:
                raise ValueError("Only one of polygon and indices can be specified")
            from .geometry import inside_polygon
            pts = self.domain.get_centroid_coordinates() if location == "centroids" else \
                self.domain.get_centroid_coordinates()
            indices = inside_polygon(pts, polygon)
        if quantity is not None:
            numeric = quantity
        if function is not None:
            numeric = function
        if isinstance(numeric, Quantity):
            src = numeric
            if location == "centroids":
                self._set_centroids(src.centroid_values if indices is None else src.centroid_values[indices], indices)
            else:
                self._set_vertices(src.vertex_values.ravel() if indices is None else src.vertex_values[indices].ravel(), indices)
        elif callable(numeric):
            if location == "centroids":
                C = self.domain.get_centroid_coordinates()
                idx = np.arange(len(self)) if indices is None else np.asarray(indices, int)
                res = numeric(C[idx, 0], C[idx, 1])
                self._set_centroids(res, None if indices is None else idx)
            else:
                V = self.domain.get_vertex_coordinates()
                vals = numeric(V[:, 0], V[:, 1])
                if np.isscalar(vals) or np.ndim(vals) == 0:
                    self._set_constant(float(vals), location, indices)
                else:
                    vals = np.asarray(vals, float).reshape(-1)
                    if indices is None:
                        self._set_vertices(vals, None)
                    else:
                        idx = np.asarray(indices, int)
                        self._set_vertices(vals.reshape(-1, 3)[idx].ravel(), idx)
        elif isinstance(numeric, (list, tuple, np.ndarray)):
            vals = np.asarray(numeric, float)
            if location == "centroids":
                self._set_centroids(vals, indices)
            else:
                if vals.ndim == 1 and indices is None and vals.size == len(self):
                    raise ValueError("vertex values must be N x 3")
                self._set_vertices(vals.reshape(-1), indices)
        elif numeric is not None:
            self._set_constant(float(numeric), location, indices)
        else:
            raise ValueError("no values given")
        self.domain._quantity_changed(self.name)

    def _set_constant(self, X, location, indices):
        if location == "centroids":
            c = self._get("centroid_values").copy()
            if indices is None:
                c[:] = X
            else:
                c[np.asarray(indices, int)] = X
            self._set_centroids(c, None)
        else:
            v = self._get("vertex_values").copy()
            if indices is None:
                v[:] = X
            else:
                v[np.asarray(indices, int)] = X
            self._set_vertices(v.ravel(), None)

    def _set_centroids(self, vals, indices):
        c = self._get("centroid_values").copy()
        vals = np.asarray(vals, float).reshape(-1)
        if indices is None:
            if vals.size != c.size:
                raise ValueError("Number of values must match number of elements")
            c[:] = vals
        else:
            c[np.asarray(indices, int)] = vals
        # extrapolate_first_order: edges and vertices take the centroid value
        self._set("centroid_values", c)
        if self._field["edge_values"] is not None or self.name not in DEVICE_FIELDS:
            self._set("edge_values", np.repeat(c[:, None], 3, 1))
            self._set("vertex_values", np.repeat(c[:, None], 3, 1))

    def _set_vertices(self, vals, indices):
        v = self._get("vertex_values").copy()
        if indices is None:
            v[:] = np.asarray(vals, float).reshape(-1, 3)
        else:
            v[np.asarray(indices, int)] = np.asarray(vals, float).reshape(-1, 3)
        self._set("vertex_values", v)
        self.interpolate()

    def interpolate(self):
        """centroid = vertex mean, edges = mid-edge means (quantity.c:665-688)."""
        v = self._get("vertex_values")
        q0, q1, q2 = v[:, 0], v[:, 1], v[:, 2]
        self._set("centroid_values", (q0 + q1 + q2) / 3.0)
        e = np.empty_like(v)
        e[:, 0] = 0.5 * (q1 + q2)
        e[:, 1] = 0.5 * (q0 + q2)
        e[:, 2] = 0.5 * (q0 + q1)
        self._set("edge_values", e)

    def get_values(self, location="vertices", indices=None):
        if location == "centroids":
            a = self.centroid_values
        elif location == "edges":
            a = self.edge_values
        elif location == "vertices":
            a = self.vertex_values
        else:
            raise ValueError("Invalid location: %s" % location)
        return a.copy() if indices is None else a[np.asarray(indices, int)].copy()

    def get_vertex_values(self, xy=True, smooth=False, precision=None):
        v = self.vertex_values
        out = v.ravel().copy()
        if precision is not None:
            out = out.astype(precision)
        return out

    def get_integral(self):
        return float(np.sum(self.domain.mesh.areas * self.centroid_values))

    def get_maximum_value(self):
        return float(np.max(self.centroid_values))

    def get_minimum_value(self):
        return float(np.min(self.centroid_values))
