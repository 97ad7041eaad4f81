"""The oracle restatement against the reference's own DE kernels compiled from
their sources (oracle/_ref, built by `make -C oracle ref` where the reference
tree exists).  Random non-trivial states on a Delaunay mesh; bit-exact."""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libswref_domain.so")

pytestmark = pytest.mark.skipif(not os.path.exists(REF), reason="reference kernels not compiled here")


I = ctypes.c_int64
D = ctypes.c_double
PI = ctypes.POINTER(ctypes.c_int64)
PD = ctypes.POINTER(ctypes.c_double)


class RefDomain(ctypes.Structure):
    """struct domain of shallow_water/sw_domain.h:14-121 (field order kept)."""
    _fields_ = [("number_of_elements", I), ("boundary_length", I), ("number_of_riverwall_edges", I),
                ("epsilon", D), ("H0", D), ("g", D), ("optimise_dry_cells", I), ("evolve_max_timestep", D),
                ("extrapolate_velocity_second_order", I), ("minimum_allowed_height", D),
                ("maximum_allowed_speed", D), ("low_froude", I), ("timestep_fluxcalls", I),
                ("beta_w", D), ("beta_w_dry", D), ("beta_uh", D), ("beta_uh_dry", D), ("beta_vh", D),
                ("beta_vh_dry", D), ("max_flux_update_frequency", I), ("ncol_riverwall_hydraulic_properties", I)] + \
               [(n, PI) for n in ("neighbours", "neighbour_edges", "surrogate_neighbours")] + \
               [(n, PD) for n in ("normals", "edgelengths", "radii", "areas")] + \
               [("edge_flux_type", PI), ("tri_full_flag", PI), ("already_computed_flux", PI), ("max_speed", PD)] + \
               [(n, PD) for n in ("vertex_coordinates", "edge_coordinates", "centroid_coordinates")] + \
               [("number_of_boundaries", PI)] + \
               [(n, PD) for n in ("stage_edge_values", "xmom_edge_values", "ymom_edge_values", "bed_edge_values",
                                  "height_edge_values", "stage_centroid_values", "xmom_centroid_values",
                                  "ymom_centroid_values", "bed_centroid_values", "height_centroid_values",
                                  "stage_vertex_values", "xmom_vertex_values", "ymom_vertex_values",
                                  "bed_vertex_values", "height_vertex_values", "stage_boundary_values",
                                  "xmom_boundary_values", "ymom_boundary_values", "bed_boundary_values",
                                  "stage_explicit_update", "xmom_explicit_update", "ymom_explicit_update")] + \
               [(n, PI) for n in ("flux_update_frequency", "update_next_flux", "update_extrapolation")] + \
               [(n, PD) for n in ("edge_timestep", "edge_flux_work", "neigh_work", "pressuregrad_work",
                                  "x_centroid_work", "y_centroid_work", "boundary_flux_sum")] + \
               [("allow_timestep_increase", PI), ("edge_river_wall_counter", PI), ("riverwall_elevation", PD),
                ("riverwall_rowIndex", PI), ("riverwall_hydraulic_properties", PD)] + \
               [(n, PD) for n in ("stage_semi_implicit_update", "xmom_semi_implicit_update",
                                  "ymom_semi_implicit_update")]


def _mesh(seed):
    from scipy.spatial import Delaunay
    from anuga_core_gb300.mesh import Mesh
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 200, (1500, 2))
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    return Mesh(pts, tri)


@pytest.mark.parametrize("alg,seed", [("DE0", 1), ("DE1", 2), ("DE1", 3)])
def test_oracle_matches_compiled_reference(oracle_mod, alg, seed):
    from helpers import random_state
    mesh = _mesh(seed)
    st = random_state(mesh, seed)
    kinds = {"exterior": ("reflective", None)}
    od = oracle_mod.OracleDomain(mesh, alg)
    od.set_centroid_state(st["stage"], st["xmom"], st["ymom"], st["elevation"], st["friction"])
    od.set_boundaries([(mesh.tag_boundary_cells[t], "reflective", None) for t in mesh.tag_boundary_cells])
    ref = ctypes.CDLL(REF)
    ref._openmp_protect.restype = ctypes.c_double
    ref._openmp_compute_fluxes_central.restype = ctypes.c_double
    ref._openmp_compute_fluxes_central.argtypes = [ctypes.c_void_p, ctypes.c_double]
    # an independent copy of the arrays for the reference
    N, B = od.N, od.B
    arr = {k: getattr(od, k).copy() for k in ("stage_c", "xmom_c", "ymom_c", "bed_c", "height_c")}
    e = {k: np.zeros(3 * N) for k in ("stage_e", "xmom_e", "ymom_e", "bed_e", "height_e",
                                       "stage_v", "xmom_v", "ymom_v", "bed_v", "height_v")}
    bnd = {k: np.zeros(B) for k in ("stage_b", "xmom_b", "ymom_b", "bed_b")}
    upd = {k: np.zeros(N) for k in ("stage_x", "xmom_x", "ymom_x", "stage_s", "xmom_s", "ymom_s",
                                    "max_speed", "xw", "yw")}
    zeros_i = np.zeros(3 * N, np.int64)
    bfs = np.zeros(3)
    D = RefDomain()  # noqa: N806
    D.number_of_elements, D.boundary_length = N, B
    D.epsilon, D.H0, D.g = 1e-12, 1e-5, 9.8
    D.evolve_max_timestep = 1e3
    D.extrapolate_velocity_second_order = 1
    D.minimum_allowed_height = od.D.minimum_allowed_height
    D.timestep_fluxcalls = 1
    for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
        setattr(D, k, getattr(od.D, k))
    D.max_flux_update_frequency = 1
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64) if a.dtype == np.int64 else ctypes.POINTER(ctypes.c_double))
    D.neighbours, D.neighbour_edges, D.surrogate_neighbours = P(od.neighbours), P(od.neighbour_edges), P(od.surrogate_neighbours)
    D.normals, D.edgelengths, D.radii, D.areas = P(od.normals), P(od.edgelengths), P(od.radii), P(od.areas)
    D.edge_flux_type, D.tri_full_flag, D.already_computed_flux = P(zeros_i), P(od.tri_full_flag), P(zeros_i)
    D.max_speed = P(upd["max_speed"])
    D.vertex_coordinates, D.edge_coordinates, D.centroid_coordinates = P(od.vertex_coordinates), P(od.edge_coordinates), P(od.centroid_coordinates)
    D.number_of_boundaries = P(od.number_of_boundaries)
    for q, a in (("stage", "stage"), ("xmom", "xmom"), ("ymom", "ymom"), ("bed", "bed"), ("height", "height")):
        setattr(D, q + "_edge_values", P(e[a + "_e"]))
        setattr(D, q + "_vertex_values", P(e[a + "_v"]))
        setattr(D, q + "_centroid_values", P(arr[a + "_c"]))
    for q in ("stage", "xmom", "ymom", "bed"):
        setattr(D, q + "_boundary_values", P(bnd[q + "_b"]))
    for q in ("stage", "xmom", "ymom"):
        setattr(D, q + "_explicit_update", P(upd[q + "_x"]))
        setattr(D, q + "_semi_implicit_update", P(upd[q + "_s"]))
    D.x_centroid_work, D.y_centroid_work = P(upd["xw"]), P(upd["yw"])
    D.boundary_flux_sum = P(bfs)
    D.edge_river_wall_counter = P(zeros_i)
    oracle_mod.set_threads(1)      # one OpenMP runtime serves both libraries
    m_ref = ref._openmp_protect(ctypes.byref(D))
    m_orc = od.protect()
    assert m_ref == m_orc
    ref._openmp_extrapolate_second_order_edge_sw(ctypes.byref(D))
    od.extrapolate()
    for k in ("stage_e", "xmom_e", "ymom_e", "bed_e", "height_e"):
        assert np.array_equal(e[k], getattr(od, k)), k
    od.update_boundary()
    for k in ("stage_b", "xmom_b", "ymom_b"):
        bnd[k][:] = getattr(od, k)
    dt_ref = ref._openmp_compute_fluxes_central(ctypes.byref(D), 1e3)
    dt_orc = od.compute_fluxes(0)
    assert dt_ref == dt_orc
    for k in ("stage_x", "xmom_x", "ymom_x"):
        assert np.array_equal(upd[k], getattr(od, k)), k
    assert np.array_equal(upd["max_speed"], od.max_speed)
