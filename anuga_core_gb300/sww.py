"""SWW (NetCDF) output of a Domain at yieldsteps.

Follows the layout written by the reference's ``file/sww.py`` (SWW_file,
Write_sww: dimensions number_of_volumes / number_of_vertices /
number_of_points / number_of_timesteps; variables x, y, volumes, time,
elevation, friction, stage, xmomentum, ymomentum in single precision, the
``*_c`` centroid variables when centroids are stored, and the
``minimum_storable_height`` mask on stage, file/sww.py:352-368).  Vertex
values are stored smoothed (averaged per node), the reference's default
(``set_store_vertices_uniquely(False)``).

On the plain FP64 form the frame is formed on the device (agx_sww_frame:
storable-height mask, node means summed in the same order as numpy's
bincount, single precision) and read back with one copy of 3 floats per node
and 3 per cell; the mixed form builds it on the host from the quantities'
vertex values.  NetCDF classic format is written with scipy.io.netcdf_file
(the netCDF4 package is not required).
"""
from __future__ import annotations

import os

import numpy as np

STATIC = ("elevation", "friction")
DYNAMIC = ("stage", "xmomentum", "ymomentum")


class SWW_file:
    def __init__(self, domain, store_centroids=True):
        from scipy.io import netcdf_file
        self.domain = domain
        self.filename = os.path.join(domain.datadir, domain.get_name() + ".sww")
        self.store_centroids = store_centroids
        self._netcdf_file = netcdf_file
        mesh = domain.mesh
        tri = mesh.triangles
        self.N = len(tri)
        self.P = mesh.number_of_nodes
        self._tri = tri
        self._count = np.bincount(tri.ravel(), minlength=self.P).astype(float)
        self._count[self._count == 0] = 1.0

    def __getstate__(self):
        state = self.__dict__.copy()
        state.pop("_bound_to", None)
        return state

    def _device_frame(self):
        """(vertex [3, P], centroid [3, N]) float32 from the device, or None."""
        d = self.domain
        scn = d._scn
        if scn is None or not hasattr(scn, "sww_frame"):
            return None
        if getattr(self, "_bound_to", None) is not scn:      # a new device scenario needs the node map
            slots = np.argsort(self._tri.ravel(), kind="stable")
            counts = np.bincount(self._tri.ravel(), minlength=self.P)
            off = np.zeros(self.P + 1, np.int64)
            off[1:] = np.cumsum(counts)
            scn.sww_bind(off, slots)
            self._bound_to = scn
        d._push_dirty()
        return scn.sww_frame(d.minimum_storable_height)

    def _smooth(self, vertex_values):
        acc = np.bincount(self._tri.ravel(), weights=vertex_values.ravel(), minlength=self.P)
        return acc / self._count

    def store_connectivity(self):
        d = self.domain
        f = self._netcdf_file(self.filename, "w", version=2)
        f.institution = "anuga_core_gb300"
        f.description = "Output from anuga_core_gb300 (DE timestep on GPU)"
        f.starttime = d.starttime
        f.createDimension("number_of_timesteps", None)      # the record dimension comes first
        f.createDimension("number_of_volumes", self.N)
        f.createDimension("number_of_vertices", 3)
        f.createDimension("number_of_points", self.P)
        f.createDimension("numbers_in_range", 2)
        x = f.createVariable("x", "f", ("number_of_points",))
        y = f.createVariable("y", "f", ("number_of_points",))
        x[:] = d.mesh.nodes[:, 0].astype(np.float32)
        y[:] = d.mesh.nodes[:, 1].astype(np.float32)
        vol = f.createVariable("volumes", "i", ("number_of_volumes", "number_of_vertices"))
        vol[:] = self._tri.astype(np.int32)
        f.createVariable("time", "d", ("number_of_timesteps",))
        for q in STATIC:
            v = f.createVariable(q, "f", ("number_of_points",))
            v[:] = self._smooth(d.quantities[q].vertex_values).astype(np.float32)
            r = f.createVariable(q + "_range", "f", ("numbers_in_range",))
            vals = d.quantities[q].centroid_values
            r[:] = np.array([vals.min(), vals.max()], np.float32) if vals.size else np.zeros(2, np.float32)
            if self.store_centroids:
                c = f.createVariable(q + "_c", "f", ("number_of_volumes",))
                c[:] = vals.astype(np.float32)
        for q in DYNAMIC:
            f.createVariable(q, "f", ("number_of_timesteps", "number_of_points"))
            r = f.createVariable(q + "_range", "f", ("numbers_in_range",))
            r[:] = np.array([np.inf, -np.inf], np.float32)
            if self.store_centroids:
                f.createVariable(q + "_c", "f", ("number_of_timesteps", "number_of_volumes"))
        f.close()

    def store_timestep(self):
        d = self.domain
        f = self._netcdf_file(self.filename, "a", version=2)
        t = f.variables["time"]
        i = t.shape[0]
        t[i] = d.get_time() - d.starttime
        frame = self._device_frame()
        Q = d.quantities
        zv = Q["elevation"].vertex_values if frame is None else None
        for j, q in enumerate(DYNAMIC):
            if frame is not None:
                A = frame[0][j]
            else:
                vv = Q[q].vertex_values
                if q == "stage":
                    # minimum_storable_height mask (file/sww.py:352-368)
                    vv = np.where(vv - zv < d.minimum_storable_height, zv, vv)
                A = self._smooth(vv).astype(np.float32)
            f.variables[q][i, :] = A
            r = f.variables[q + "_range"]
            r[0] = min(float(r[0]), float(A.min()) if A.size else np.inf)
            r[1] = max(float(r[1]), float(A.max()) if A.size else -np.inf)
            if self.store_centroids:
                if frame is not None:
                    c = frame[1][j]
                else:
                    c = Q[q].centroid_values
                    if q == "stage":
                        zc = Q["elevation"].centroid_values
                        c = np.where(c - zc < d.minimum_storable_height, zc, c)
                f.variables[q + "_c"][i, :] = np.asarray(c, np.float32)
        f.close()

    def host_frame(self):
        """The same frame formed on the host from the quantities (reference)."""
        d = self.domain
        Q = d.quantities
        zv = Q["elevation"].vertex_values
        zc = Q["elevation"].centroid_values
        V, C = [], []
        for q in DYNAMIC:
            vv = Q[q].vertex_values
            c = Q[q].centroid_values
            if q == "stage":
                vv = np.where(vv - zv < d.minimum_storable_height, zv, vv)
                c = np.where(c - zc < d.minimum_storable_height, zc, c)
            V.append(self._smooth(vv).astype(np.float32))
            C.append(c.astype(np.float32))
        return np.array(V), np.array(C)


def read_sww(filename):
    """Small reader returning a dict of numpy arrays (for tests and tools)."""
    from scipy.io import netcdf_file
    f = netcdf_file(filename, "r", mmap=False)
    out = {k: np.array(v[:]) for k, v in f.variables.items()}
    f.close()
    return out
