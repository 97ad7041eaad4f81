"""SWW (NetCDF) output of a Domain at yieldsteps.

Follows what the reference's ``file/sww.py`` writes (SWW_file, Write_sww:
dimensions number_of_volumes / number_of_vertices / number_of_points /
number_of_timesteps; variables x, y, volumes, time, elevation, friction,
stage, xmomentum, ymomentum in single precision, their ``*_range`` and the
``*_c`` centroid variables).  A frame is formed as SWW_file.store_timestep
does (file/sww.py:352-410): per node the mean over its vertex slots, summed in
the order of the mesh's vertex_value_indices (general_mesh.py:830, the
default numpy argsort of the triangles) and divided by their count, of the
centroid values of the slots' triangles (the centroid averaging that every
DE flow algorithm switches on, shallow_water_domain.py:596; quantity.c:872-915)
or, with centroid averaging off, of the slots' vertex values
(quantity.c:823-870); where the mean stage minus the mean bed is below
minimum_storable_height the node's stage is its bed and its momenta are zero;
centroid values are stored as they are.

Both forms build the frame on the device (agx_sww_frame_async: node means,
mask and conversion to single precision in one kernel pair) and copy it into
page-locked memory without blocking the host.  The netCDF append then runs
on a writer thread while the host issues the next yieldstep; the file is
complete once the next frame starts, when evolve returns, or after
``flush()``.  NetCDF classic format is written with scipy.io.netcdf_file (the
netCDF4 package is not required).
"""
from __future__ import annotations

import concurrent.futures
import os

import numpy as np

STATIC = ("elevation", "friction")
DYNAMIC = ("stage", "xmomentum", "ymomentum")


class SWW_file:
    def __init__(self, domain, store_centroids=True, asynchronous=True):
        from scipy.io import netcdf_file
        self.domain = domain
        self.filename = os.path.join(domain.datadir, domain.get_name() + ".sww")
        self.store_centroids = store_centroids
        self.asynchronous = asynchronous
        self._netcdf_file = netcdf_file
        mesh = domain.mesh
        tri = np.asarray(mesh.triangles, np.int64)
        self.N = len(tri)
        self.P = mesh.number_of_nodes
        self._tri = tri
        flat = tri.ravel()
        self._counts = np.bincount(flat, minlength=self.P)
        # vertex slots grouped by node, in the order of the reference's
        # vertex_value_indices
        self._vvi = np.argsort(flat).astype(np.int64)
        self._off = np.zeros(self.P + 1, np.int64)
        self._off[1:] = np.cumsum(self._counts)
        self._exec = None
        self._pending = None

    def __getstate__(self):
        self.flush()
        state = self.__dict__.copy()
        state.pop("_bound_to", None)
        state["_exec"] = None
        state["_pending"] = None
        return state

    # ------------------------------------------------------------------
    def _device_scn(self):
        """The domain's device scenario, bound to this file's node map."""
        d = self.domain
        scn = d._scn
        if scn is None or not hasattr(scn, "sww_frame_async"):
            return None
        if getattr(self, "_bound_to", None) is not scn:      # a new device scenario needs the node map
            scn.sww_bind(self._off, self._vvi)
            self._bound_to = scn
        d._push_dirty()
        return scn

    def _device_frame(self):
        """(vertex [3, P], centroid [3, N]) float32 formed on the device, or None."""
        scn = self._device_scn()
        if scn is None:
            return None
        self.flush()
        d = self.domain
        scn.sww_frame_async(d.minimum_storable_height, d.get_using_centroid_averaging())
        return scn.sww_frame_wait()

    def _smooth(self, vertex_values, centroid_values=None):
        """Node means as quantity.c:823-915 forms them: the values of the
        node's vertex slots (the centroid value of the slot's triangle when
        centroid_values is given, else the slot's vertex value) added one at a
        time in vertex_value_indices order, the total divided by the count."""
        if centroid_values is not None:
            v = np.asarray(centroid_values, float)[self._vvi // 3]
        else:
            v = np.asarray(vertex_values, float).ravel()[self._vvi]
        acc = np.zeros(self.P)
        start = self._off[:-1]
        for j in range(int(self._counts.max()) if self.P else 0):
            sel = self._counts > j
            acc[sel] = acc[sel] + v[start[sel] + j]
        nz = self._counts > 0
        acc[nz] = acc[nz] / self._counts[nz]
        return acc

    def _node_values(self, q):
        Q = self.domain.quantities[q]
        if self.domain.get_using_centroid_averaging():
            return self._smooth(None, Q.centroid_values)
        return self._smooth(Q.vertex_values)

    def host_frame(self):
        """The same frame formed on the host from the quantities."""
        d = self.domain
        Q = d.quantities
        wn = self._node_values("stage")
        zn = self._node_values("elevation")
        storable = wn - zn >= d.minimum_storable_height
        V = [np.where(storable, wn.astype(np.float32), zn.astype(np.float32)).astype(np.float32)]
        for q in ("xmomentum", "ymomentum"):
            A = self._node_values(q).astype(np.float32)
            V.append(np.where(storable, A, np.float32(0.0)).astype(np.float32))
        C = [Q[q].centroid_values.astype(np.float32) for q in DYNAMIC]
        return np.array(V), np.array(C)

    # ------------------------------------------------------------------
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
            A = self._node_values(q).astype(np.float32)
            v[:] = A
            r = f.createVariable(q + "_range", "f", ("numbers_in_range",))
            r[:] = np.array([A.min(), A.max()], np.float32) if A.size else np.zeros(2, np.float32)
            if self.store_centroids:
                c = f.createVariable(q + "_c", "f", ("number_of_volumes",))
                c[:] = d.quantities[q].centroid_values.astype(np.float32)
        big = np.finfo(np.float32).max
        for q in DYNAMIC:
            f.createVariable(q, "f", ("number_of_timesteps", "number_of_points"))
            r = f.createVariable(q + "_range", "f", ("numbers_in_range",))
            r[:] = np.array([big, -big], np.float32)
            if self.store_centroids:
                f.createVariable(q + "_c", "f", ("number_of_timesteps", "number_of_volumes"))
        f.close()

    def _append(self, t, V, C):
        f = self._netcdf_file(self.filename, "a", version=2)
        tv = f.variables["time"]
        i = tv.shape[0]
        tv[i] = t
        for j, q in enumerate(DYNAMIC):
            A = V[j]
            f.variables[q][i, :] = A
            r = f.variables[q + "_range"]
            if A.size:
                r[0] = min(float(r[0]), float(A.min()))
                r[1] = max(float(r[1]), float(A.max()))
            if self.store_centroids:
                f.variables[q + "_c"][i, :] = C[j]
        f.close()

    def _write_device_frame(self, t, scn):
        V, C = scn.sww_frame_wait()
        self._append(t, V, C)

    def store_timestep(self):
        d = self.domain
        t = d.get_time() - d.starttime
        self.flush()
        scn = self._device_scn()
        if scn is None:
            V, C = self.host_frame()
            self._append(t, V, C)
            return
        scn.sww_frame_async(d.minimum_storable_height, d.get_using_centroid_averaging())
        if self.asynchronous:
            if self._exec is None:
                self._exec = concurrent.futures.ThreadPoolExecutor(max_workers=1)
            self._pending = self._exec.submit(self._write_device_frame, t, scn)
        else:
            self._write_device_frame(t, scn)

    def flush(self):
        """Wait until the last frame is in the file (raises its error, if any)."""
        if self._pending is not None:
            fut, self._pending = self._pending, None
            fut.result()


def read_sww(filename):
    """Small reader returning a dict of numpy arrays (for tests and tools)."""
    from scipy.io import netcdf_file
    f = netcdf_file(filename, "r", mmap=False)
    out = {k: np.array(v[:]) for k, v in f.variables.items()}
    f.close()
    return out
