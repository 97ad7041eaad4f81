"""Small host-side polygon helpers (point selection for quantities and
operators), vectorised with numpy.  Same semantics as the reference's
``geometry/polygon.py`` inside_polygon for points strictly inside or on the
boundary (closed=True)."""
from __future__ import annotations

import numpy as np


def inside_polygon(points, polygon, closed=True):
    """Indices of points inside the polygon (even-odd rule, boundary counts
    as inside when closed)."""
    P = np.asarray(points, float).reshape(-1, 2)
    poly = np.asarray(polygon, float).reshape(-1, 2)
    x, y = P[:, 0], P[:, 1]
    inside = np.zeros(len(P), bool)
    on_edge = np.zeros(len(P), bool)
    n = len(poly)
    for i in range(n):
        x0, y0 = poly[i]
        x1, y1 = poly[(i + 1) % n]
        cond = (y0 > y) != (y1 > y)
        with np.errstate(divide="ignore", invalid="ignore"):
            xin = x0 + (y - y0) * (x1 - x0) / (y1 - y0)
        inside ^= cond & (x < xin)
        # on-segment test
        cross = (x1 - x0) * (y - y0) - (y1 - y0) * (x - x0)
        within = (np.minimum(x0, x1) <= x) & (x <= np.maximum(x0, x1)) & \
                 (np.minimum(y0, y1) <= y) & (y <= np.maximum(y0, y1))
        on_edge |= (np.abs(cross) <= 1e-12 * max(1.0, abs(x1 - x0) + abs(y1 - y0))) & within
    if closed:
        inside |= on_edge
    else:
        inside &= ~on_edge
    return np.nonzero(inside)[0]


def polygon_area(polygon):
    p = np.asarray(polygon, float).reshape(-1, 2)
    x, y = p[:, 0], p[:, 1]
    return 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))
