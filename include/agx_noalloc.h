/*
 * agx_noalloc.h -- edge fluxes into caller-owned device buffers, with no
 * device allocation (libagx.so).
 *
 * No counterpart in the reference: the reference computes fluxes only on the
 * arrays of its own domain object (compute_fluxes_ext_central,
 * shallow_water/sw_domain_openmp_ext.pyx:371).  This entry point gives the same
 * results as agx_compute_fluxes (include/agx.h) for device arrays that the
 * caller owns, and it allocates nothing: its scratch is a fixed-size device
 * array inside libagx.so.
 */
#ifndef AGX_NOALLOC_H
#define AGX_NOALLOC_H
#include <stdint.h>
#include "agx.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Largest mesh (triangles) the built-in scratch holds: six FP64 values and a
 * 32-bit stamp per edge slot, 3 slots per triangle, i.e. 9.75 MiB of device
 * memory on every device that loads the library, held until the process
 * exits. */
#define AGX_NOALLOC_MAX_CELLS 65536

/* Device pointers, laid out as the tables of anuga_core_gb300/tables.py
 * pack_tables() and the fields of include/agx.h. */
typedef struct {
  int64_t N;                    /* triangles, 1 .. AGX_NOALLOC_MAX_CELLS */
  int64_t B;                    /* boundary edges */
  int64_t E;                    /* entries of the edge list, <= 3N: together the listed slots and
                                   their opposite slots must name each of the 3N slots exactly
                                   once (the edge list of pack_tables does); a list that misses
                                   or repeats a slot is rejected with AGX_E_INVALID */
  const int32_t* conn;          /* [N*4] neighbours + meta word; 16-byte aligned */
  const int32_t* edge_slot;     /* [E] slot 3k+i of each listed edge */
  const int32_t* edge_opp;      /* [E] slot on the other side, -1 on the boundary */
  const double* normals;        /* [N*6] */
  const double* edgelengths;    /* [N*3] */
  const double* radii;          /* [N] */
  const double* inv_area;       /* [N] */
  const double* stage_e;        /* [3N] edge values */
  const double* xmom_e;
  const double* ymom_e;
  const double* elev_e;
  const double* height_e;
  const double* stage_b;        /* [B] boundary values */
  const double* xmom_b;
  const double* ymom_b;
  const double* stage_c;        /* [N] centroid values */
  const double* height_c;
  const double* elev_c;
  double* stage_x;              /* [N] explicit updates, written */
  double* xmom_x;
  double* ymom_x;
  double* max_speed;            /* [N] written when substep == 0 */
} agx_flux_buffers;

/* compute_fluxes (shallow_water_domain.py:1828-1877) on caller-owned arrays:
 * the explicit updates, the max speeds (substep 0) and the flux timestep and
 * boundary flux sum, as agx_compute_fluxes returns them (flux_timestep and
 * boundary_flux_sum are host pointers and may be NULL).  Work is issued on
 * `stream` (NULL: the legacy default stream) and the call waits for it, then
 * reports a table index found out of range as AGX_E_INVALID.
 *
 * Limits: N above AGX_NOALLOC_MAX_CELLS is rejected with AGX_E_INVALID and a
 * message in err.  The scratch is one per device, so calls that overlap on
 * the same device (two host threads, or two streams whose work is in flight
 * together) race on it and give wrong results; serialise them.  The first call
 * on each device looks up the scratch address (cudaGetSymbolAddress, which
 * may load the module); make that first call before any stream capture.
 * With lazy module loading (the CUDA default) that first call is also when
 * the scratch itself is committed on the device, so it needs 9.75 MiB of
 * free device memory: make it (a warm-up call on a small mesh will do)
 * before a host framework's caching allocator reserves the free memory.
 * Riverwalls are not applied: every edge takes the plain central flux.
 * err (may be NULL) receives a message of at most err_len bytes on failure. */
agx_status agx_compute_fluxes_noalloc(const agx_params* params, const agx_flux_buffers* buf, int32_t substep,
                                      void* stream, double* flux_timestep, double* boundary_flux_sum,
                                      char* err, int32_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* AGX_NOALLOC_H */
