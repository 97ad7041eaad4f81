"""Riverwalls: levees along mesh edges whose flux follows the weir equation
(structures/riverwall.py, the weir branch of sw_domain_openmp.c:324-426 and
:581-650).

``domain.create_riverwalls(riverwalls, riverwallPar={}, default_riverwallPar={})``
finds the mesh edges lying on each named 3-D polyline (x, y, crest elevation),
gives each the crest elevation interpolated along its segment and the
riverwall's hydraulic parameters, and marks them ``edge_flux_type == 1``.  The
tables have the reference's layout so that the same flux arithmetic reads
them:

* ``domain.edge_flux_type[3N]``: 1 on a riverwall edge (both cells' slots of an
  interior edge share the midpoint, so both are marked), else 0;
* ``domain.edge_river_wall_counter[3N]``: 1-based rank of a marked slot in slot
  order, 0 elsewhere;
* ``riverwall_elevation[n]``, ``hydraulic_properties_rowIndex[n]`` per marked
  slot in slot order, ``hydraulic_properties[n_walls, 5]`` with the columns
  ``Qfactor, s1, s2, h1, h2``.

On the device the marked slots are evaluated from each side (the weir
correction uses each side's own upstream and downstream heads, so the flux is
not antisymmetric) and the weir correction is applied inside the flux kernel.
"""
from __future__ import annotations

import numpy as np

HYDRAULIC_VARIABLES = ("Qfactor", "s1", "s2", "h1", "h2")
DEFAULT_PARAMETERS = {"Qfactor": 1.0, "s1": 0.9, "s2": 0.95, "h1": 1.0, "h2": 1.5}
_NO_ELEVATION = -1.0e36                     # -max_float (anuga/config.py), unmarked slots


class RiverWall:
    """Riverwall tables of one domain (empty until create_riverwalls)."""

    hydraulic_variable_names = HYDRAULIC_VARIABLES
    ncol_hydraulic_properties = len(HYDRAULIC_VARIABLES)

    def __init__(self, domain):
        self.domain = domain
        self.names = []
        self.default_riverwallPar = dict(DEFAULT_PARAMETERS)
        self.riverwall_elevation = np.array([-9.0e20])
        self.hydraulic_properties_rowIndex = np.array([-1000000000], dtype=np.int64)
        self.hydraulic_properties = np.array([[-9.0e20]])
        self.riverwall_edges = np.array([-1000000000], dtype=np.int64)
        self.input_riverwall_geo = None
        self.input_riverwallPar = None

    @property
    def active(self):
        return len(self.names) > 0 and int(self.domain.number_of_riverwall_edges) > 0

    def _offsets(self):
        g = getattr(self.domain, "geo_reference", None)
        if g is None:
            return 0.0, 0.0
        x = g.get_xllcorner() if hasattr(g, "get_xllcorner") else getattr(g, "xllcorner", 0.0)
        y = g.get_yllcorner() if hasattr(g, "get_yllcorner") else getattr(g, "yllcorner", 0.0)
        return float(x), float(y)

    def create_riverwalls(self, riverwalls, riverwallPar={}, default_riverwallPar={}, tol=1.0e-4,
                          verbose=False, output_dir=None):
        """Marks the edges on each riverwall polyline (within ``tol`` of a
        segment, measured at the edge midpoint) and fills the tables.  The
        walls must coincide with mesh edges (build the mesh with them as
        breaklines)."""
        d = self.domain
        if getattr(d, "flow_algorithm", "DE0")[:2] != "DE":
            raise Exception("Riverwalls are currently only supported for discontinuous elevation flow algorithms")
        if self.names:
            self.__init__(d)
        self.input_riverwall_geo = riverwalls
        self.input_riverwallPar = riverwallPar
        for k, v in default_riverwallPar.items():
            if k not in self.default_riverwallPar:
                raise Exception("Key %s in default_riverwallPar not recognized" % k)
            self.default_riverwallPar[k] = v
        for name, par in riverwallPar.items():
            if name not in riverwalls:
                raise Exception("Key %s in riverwallPar has no corresponding key in riverwall" % name)
            for k in par:
                if k not in self.default_riverwallPar:
                    raise Exception("Hydraulic parameter %s for riverwall %s not recognised in "
                                    "default_riverwallPar" % (k, name))

        exy = np.asarray(d.edge_coordinates)
        llx, lly = self._offsets()
        n_slots = exy.shape[0]
        flux_type = np.zeros(n_slots, dtype=np.int64)
        elevation = np.full(n_slots, _NO_ELEVATION)
        row = np.full(n_slots, -1.0)
        names = list(riverwalls.keys())
        for wall, name in enumerate(names):
            points = riverwalls[name]
            for a, b in zip(points[:-1], points[1:]):
                if len(a) != 3 or len(b) != 3:
                    raise Exception("Riverwall %s: points must be [x, y, z]" % name)
                seg_len = ((a[0] - b[0]) ** 2 + (a[1] - b[1]) ** 2) ** 0.5
                if seg_len < tol:
                    continue
                ux = -(a[0] - b[0]) / seg_len
                uy = -(a[1] - b[1]) / seg_len
                px = exy[:, 0] - (a[0] - llx)
                py = exy[:, 1] - (a[1] - lly)
                dist = (px ** 2 + py ** 2) ** 0.5
                along = px * ux + py * uy
                perp_sq = dist ** 2. - along ** 2.
                on = ((perp_sq < tol ** 2) * (along > 0. - tol) * (along < seg_len + tol)).nonzero()[0]
                if len(on) == 0:
                    continue
                flux_type[on] = 1
                w = along[on] / seg_len
                w = w * (w >= 0.0)
                w = w * (w <= 1.0) + 1.0 * (w > 1.0)
                elevation[on] = a[2] * (1.0 - w) + w * b[2]
                row[on] = wall

        marked = (flux_type == 1).nonzero()[0]
        d.edge_flux_type = flux_type
        counter = np.zeros(n_slots, dtype=np.int64)
        counter[marked] = np.arange(1, len(marked) + 1)
        d.edge_river_wall_counter = counter
        d.number_of_riverwall_edges = len(marked)
        self.riverwall_elevation = elevation[marked]
        self.hydraulic_properties_rowIndex = row[marked].astype(np.int64)
        self.riverwall_edges = marked
        self.names = names

        table = np.full((len(names), len(HYDRAULIC_VARIABLES)), np.nan)
        for wall, name in enumerate(names):
            par = riverwallPar.get(name, {})
            for j, var in enumerate(HYDRAULIC_VARIABLES):
                table[wall, j] = par[var] if var in par else self.default_riverwallPar[var]
        for wall in range(len(names)):
            if table[wall, 1] >= table[wall, 2]:
                raise Exception("s1 must be less than s2 for riverwall %s" % names[wall])
            if table[wall, 1] < 0.0 or table[wall, 2] < 0.0:
                raise Exception("s1 and s2 must be positive, with s1<s2")
            if table[wall, 3] >= table[wall, 4]:
                raise Exception("h1 must be less than h2 for riverwall %s" % names[wall])
            if table[wall, 3] < 0.0 or table[wall, 4] < 0.0:
                raise Exception("h1 and h2 must be positive, with h1<h2")
        self.hydraulic_properties = table
        if verbose:
            print("Riverwalls: %d edges on %d walls" % (len(marked), len(names)))
        d._riverwalls_changed()
