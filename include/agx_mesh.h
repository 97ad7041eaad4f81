/*
 * agx_mesh.h -- native host builders of mesh connectivity, geometry and the
 * device tables (libagx.so; C++ with OpenMP over the host cores).
 *
 * These replace the host-side setup the reference does when a Domain is built:
 * the geometry of abstract_2d_finite_volumes/general_mesh.py:134-267, the
 * neighbour structure of neighbour_mesh.py:296-346 (built in the reference by
 * abstract_2d_finite_volumes/neighbour_table.cpp), and the packing of the
 * arrays the kernels read.  All arrays are host memory, row-major, int64 or
 * double unless stated.  Results are bit-identical to the numpy restatement in
 * anuga_core_gb300/mesh.py and tables.py.
 */
#ifndef AGX_MESH_H
#define AGX_MESH_H
#include <stdint.h>
#include "agx.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry of N counter-clockwise triangles tri[N*3] over nodes[n_nodes*2]:
 * vertex coordinates V[N*6], edge midpoints E[N*6] (edge i opposite vertex i),
 * centroids C[N*2], outward normals[N*6], edge lengths[N*3], areas[N], radii[N]
 * (centroid to nearest edge midpoint, or the inscribed circle).  *first_bad is
 * the first triangle whose area is not positive (-1 if none). */
agx_status agx_mesh_geometry(int64_t n_nodes, const double* nodes, int64_t N, const int64_t* tri,
                             int32_t use_inscribed_circle, double* V, double* E, double* C, double* normals,
                             double* lengths, double* areas, double* radii, int64_t* first_bad);

/* Neighbour across each edge nb[N*3] (-1: boundary), the neighbour's edge
 * number ne[N*3], and the number of boundary edges per triangle.
 * AGX_E_STATE if a directed edge appears twice (inconsistent orientation). */
agx_status agx_mesh_neighbours(int64_t n_nodes, int64_t N, const int64_t* tri, int64_t* nb, int64_t* ne,
                               int64_t* n_boundaries);

/* Order of n points pts[n*2] along a space-filling curve (curve 0: Morton,
 * 1: Hilbert) quantised to `bits` bits per axis; ties keep index order. */
agx_status agx_sfc_order(int64_t n, const double* pts, int32_t curve, int32_t bits, int64_t* order);

/* Per tile of `tile` consecutive cells (conn[N*4] in the stored order): the
 * outside cells its fluxes need (sorted, at most halo_max staged), and for
 * every slot the staging index of its neighbour packed 10 bits per slot
 * (inline_id for boundary edges and unstaged cells).  halo_cells may be NULL
 * to count only; *n_halo_unclamped counts every (tile, outside cell) pair. */
agx_status agx_tile_halos(int64_t N, const int32_t* conn, int32_t tile, int32_t halo_max, int32_t inline_id,
                          int32_t* lnk, int32_t* halo_off, int32_t* halo_cnt, int32_t* halo_cells,
                          int64_t halo_capacity, int64_t* n_halo, int64_t* n_halo_unclamped);

/* Tables of the plain FP64 path (agx_mesh_desc): conn/surr int32[N*4] with
 * the meta word, extrapolation geometry geo[N*11] and the edge-once lists
 * edge_slot/edge_opp int32 (capacity 3N, *n_edges used).  full[N] (NULL: all
 * full), per_side_in uint8[N*3] (NULL: none) and orig[N] (NULL: identity) are
 * optional. */
agx_status agx_pack_plain(int64_t N, const int64_t* nb, const int64_t* ne, const int64_t* sn, const int64_t* nbnd,
                          const int64_t* full, const uint8_t* per_side_in, const int64_t* orig,
                          const double* normals, const double* lengths, const double* C, const double* Em,
                          int32_t* conn, int32_t* surr, double* geo, int32_t* edge_slot, int32_t* edge_opp,
                          int64_t* n_edges);

/* Tables of the mixed-precision pool in the stored order `order[N]`:
 * conn int32[N*4], geo float[N*16] (jump matrix, edge vectors, radius),
 * area_s[N], order_s int32[N]. */
agx_status agx_pack_mixed(int64_t N, const int64_t* order, const int64_t* nb, const int64_t* ne, const int64_t* sn,
                          const int64_t* nbnd, const double* C, const double* Em, const double* V,
                          const double* radii, const double* areas, int32_t* conn, float* geo, double* area_s,
                          int32_t* order_s);

/* Host threads the builders use (n > 0 sets it); returns the current count. */
int32_t agx_mesh_threads(int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* AGX_MESH_H */
