"""ctypes bindings of the native host builders (include/agx_mesh.h).

Mesh geometry and neighbours, space-filling-curve orders, tile halos and the
packed device tables are computed in C++ with OpenMP over the host cores; the
numpy restatements in mesh.py and tables.py compute the same bits and are
kept as the references the tests compare against.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32

_bound = None


def _L():
    global _bound
    if _bound is None:
        L = _lib.load()
        sig = {
            "agx_mesh_geometry": [_I64, _f64p, _I64, _i64p, _I32, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                  _f64p, _i64p],
            "agx_mesh_neighbours": [_I64, _I64, _i64p, _i64p, _i64p, _i64p],
            "agx_sfc_order": [_I64, _f64p, _I32, _I32, _i64p],
            "agx_tile_halos": [_I64, _i32p, _I32, _I32, _I32, _i32p, _i32p, _i32p, _i32p, _I64, _i64p, _i64p],
            "agx_pack_plain": [_I64, _i64p, _i64p, _i64p, _i64p, _i64p, _u8p, _i64p, _f64p, _f64p, _f64p, _f64p,
                               _i32p, _i32p, _f64p, _i32p, _i32p, _i64p],
            "agx_pack_mixed": [_I64, _i64p, _i64p, _i64p, _i64p, _i64p, _f64p, _f64p, _f64p, _f64p, _f64p, _i32p,
                               _f32p, _f64p, _i32p],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int32
        L.agx_mesh_threads.argtypes = [_I32]
        L.agx_mesh_threads.restype = _I32
        _bound = L
    return _bound


def _p(a, t):
    if a is None:
        return ctypes.cast(None, t)
    return a.ctypes.data_as(t)


def _c(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype))


def threads(n=0):
    """Host threads of the builders (n > 0 sets it)."""
    return int(_L().agx_mesh_threads(int(n)))


def mesh_geometry(nodes, triangles, use_inscribed_circle=False):
    nodes = _c(nodes, np.float64)
    tri = _c(triangles, np.int64)
    N = tri.shape[0]
    out = dict(V=np.empty((3 * N, 2)), E=np.empty((3 * N, 2)), C=np.empty((N, 2)), normals=np.empty((N, 6)),
               lengths=np.empty((N, 3)), areas=np.empty(N), radii=np.empty(N))
    bad = ctypes.c_int64(-1)
    rc = _L().agx_mesh_geometry(nodes.shape[0], _p(nodes, _f64p), N, _p(tri, _i64p), 1 if use_inscribed_circle else 0,
                                *[_p(out[k], _f64p) for k in ("V", "E", "C", "normals", "lengths", "areas", "radii")],
                                ctypes.byref(bad))
    if rc != 0:
        raise ValueError("Vertex indices reference non-existing coordinate sets")
    return out, int(bad.value)


def mesh_neighbours(n_nodes, triangles):
    tri = _c(triangles, np.int64)
    N = tri.shape[0]
    nb = np.empty((N, 3), np.int64)
    ne = np.empty((N, 3), np.int64)
    nbnd = np.empty(N, np.int64)
    rc = _L().agx_mesh_neighbours(int(n_nodes), N, _p(tri, _i64p), _p(nb, _i64p), _p(ne, _i64p), _p(nbnd, _i64p))
    if rc == -4:                     # AGX_E_STATE
        raise ValueError("Inconsistent mesh: a directed edge appears twice (triangles not consistently oriented)")
    if rc != 0:
        raise ValueError("Vertex indices reference non-existing coordinate sets")
    return nb, ne, nbnd


def sfc_order(points, curve, bits=16):
    P = _c(points, np.float64).reshape(-1, 2)
    order = np.empty(P.shape[0], np.int64)
    rc = _L().agx_sfc_order(P.shape[0], _p(P, _f64p), {"morton": 0, "hilbert": 1}[curve], int(bits), _p(order, _i64p))
    if rc != 0:
        raise ValueError("bad arguments to agx_sfc_order")
    return order


def tile_halos(conn, tile, halo_max, inline_id, count_only=False):
    conn = _c(conn, np.int32).reshape(-1, 4)
    N = conn.shape[0]
    T = (N + tile - 1) // tile
    lnk = np.empty(N, np.int32)
    off = np.empty(T, np.int32)
    cnt = np.empty(T, np.int32)
    nh = ctypes.c_int64()
    nu = ctypes.c_int64()
    cap = 3 * N
    hc = None if count_only else np.empty(cap, np.int32)
    rc = _L().agx_tile_halos(N, _p(conn, _i32p), tile, halo_max, inline_id, _p(lnk, _i32p), _p(off, _i32p),
                             _p(cnt, _i32p), _p(hc, _i32p), cap, ctypes.byref(nh), ctypes.byref(nu))
    if rc != 0:
        raise ValueError("bad arguments to agx_tile_halos")
    if count_only:
        return int(nu.value)
    return lnk, off, cnt, hc[:nh.value].copy(), int(nu.value)


def pack_plain(N, nb, ne, sn, nbnd, full, per_side, orig, normals, lengths, C, Em):
    arr = dict(nb=_c(nb, np.int64), ne=_c(ne, np.int64), sn=_c(sn, np.int64), nbnd=_c(nbnd, np.int64))
    full = None if full is None else _c(full, np.int64)
    per_side = None if per_side is None else _c(per_side, np.uint8)
    orig = None if orig is None else _c(orig, np.int64)
    normals = _c(normals, np.float64)
    lengths = _c(lengths, np.float64)
    C = _c(C, np.float64)
    Em = _c(Em, np.float64)
    conn = np.empty((N, 4), np.int32)
    surr = np.empty((N, 4), np.int32)
    geo = np.empty((N, 11), np.float64)
    es = np.empty(3 * N, np.int32)
    eo = np.empty(3 * N, np.int32)
    ne_out = ctypes.c_int64()
    rc = _L().agx_pack_plain(N, _p(arr["nb"], _i64p), _p(arr["ne"], _i64p), _p(arr["sn"], _i64p),
                             _p(arr["nbnd"], _i64p), _p(full, _i64p), _p(per_side, _u8p), _p(orig, _i64p),
                             _p(normals, _f64p), _p(lengths, _f64p), _p(C, _f64p), _p(Em, _f64p), _p(conn, _i32p),
                             _p(surr, _i32p), _p(geo, _f64p), _p(es, _i32p), _p(eo, _i32p), ctypes.byref(ne_out))
    if rc != 0:
        raise ValueError("mesh too large for 32-bit slot indices" if N >= (1 << 29) else "bad mesh tables")
    n = ne_out.value
    return conn, surr, geo, es[:n].copy(), eo[:n].copy()


def pack_mixed(order, nb, ne, sn, nbnd, C, Em, V, radii, areas):
    order = _c(order, np.int64)
    N = order.shape[0]
    a = [_c(x, np.int64) for x in (nb, ne, sn, nbnd)]
    f = [_c(x, np.float64) for x in (C, Em, V, radii, areas)]
    conn = np.empty((N, 4), np.int32)
    geo = np.empty((N, 16), np.float32)
    area_s = np.empty(N, np.float64)
    order_s = np.empty(N, np.int32)
    rc = _L().agx_pack_mixed(N, _p(order, _i64p), *[_p(x, _i64p) for x in a], *[_p(x, _f64p) for x in f],
                             _p(conn, _i32p), _p(geo, _f32p), _p(area_s, _f64p), _p(order_s, _i32p))
    if rc != 0:
        raise ValueError("bad arguments to agx_pack_mixed")
    return conn, geo, area_s, order_s
