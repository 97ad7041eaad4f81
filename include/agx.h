/*
 * agx.h -- C ABI of the GB300 DE-timestep library (libagx.so).
 *
 * Plain pointers and sizes only; every function returns an agx_status
 * (0 = success, negative = error; agx_last_error() gives the message).
 * A scenario is one mesh with its state resident in device memory; handles
 * are not thread-safe (one caller thread per handle).
 *
 * Each entry point names the reference interface it replaces (paths in the
 * anuga_core project).  The reference's plugin seam is the multiprocessor_mode
 * dispatch of shallow_water/shallow_water_domain.py:1855-1874, 1893-1915,
 * 2022-2039, 2114-2154 and shallow_water/friction.py:23-29; its native calls
 * are the Cython wrappers of shallow_water/sw_domain_openmp_ext.pyx:366-459
 * over struct domain (shallow_water/sw_domain.h:14-121).
 */
#ifndef AGX_H
#define AGX_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t agx_status;
#define AGX_OK 0
#define AGX_E_INVALID   (-1)   /* bad argument or size */
#define AGX_E_CUDA      (-2)   /* a CUDA call failed */
#define AGX_E_NOMEM     (-3)   /* device allocation failed */
#define AGX_E_STATE     (-4)   /* call not valid in the scenario's current state */
#define AGX_E_NUMERIC   (-5)   /* non-positive semi-implicit denominator (quantity.c:800-806) */
#define AGX_E_TIMESTEP  (-6)   /* too small timestep at first order (generic_domain.py:2369-2395) */
#define AGX_E_OVERSHOOT (-7)   /* time overshot finaltime (generic_domain.py:1869-1875) */
#define AGX_E_TIMEOUT   (-8)   /* a bounded device wait gave up */

typedef struct agx_scenario* agx_handle;

/* Mesh tables (host pointers, copied at creation).  Built from the mesh
 * arrays of abstract_2d_finite_volumes/general_mesh.py:134-267 and
 * neighbour_mesh.py:70-505 by anuga_core_gb300/tables.py. */
typedef struct {
  int64_t n_cells;             /* N triangles */
  int64_t n_boundary;          /* B boundary edges */
  int64_t n_edges;             /* E flux evaluations (edge_slot / edge_opp length) */
  const int32_t* conn;         /* [N*4] neighbours + meta word */
  const int32_t* surr;         /* [N*4] surrogate neighbours + number_of_boundaries */
  const double* geo;           /* [N*11] extrapolation geometry */
  const int32_t* edge_slot;    /* [E] */
  const int32_t* edge_opp;     /* [E] */
  const double* normals;       /* [N*6] */
  const double* edgelengths;   /* [N*3] */
  const double* radii;         /* [N] */
  const double* areas;         /* [N] */
  const double* inv_area;      /* [N] */
  const int32_t* boundary_slot;/* [B] 3*cell + edge */
  const double* vertex_coordinates; /* [N*6] */
} agx_mesh_desc;

/* Algorithm parameters: the scalar part of struct domain
 * (sw_domain.h:16-38) plus the time-stepping settings of
 * generic_domain.py:2349-2415. */
typedef struct {
  double g, epsilon, minimum_allowed_height;
  double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
  double CFL, evolve_max_timestep, evolve_min_timestep;
  int32_t extrapolate_velocity_second_order;
  int32_t low_froude;
  int32_t timestepping_method;   /* 1 = euler (DE0, DE0_7), 2 = rk2 (DE1, DE1_7), 3 = rk3 (DE2) */
  int32_t protect_zero_ymom;     /* 0: sw_domain_openmp.c:1139-1140 (xmom only); 1: orig (both) */
  int32_t use_sloped_mannings;
  int32_t max_smallsteps;
  int32_t precision;             /* AGX_PREC_FP64 or AGX_PREC_MIXED */
  int32_t reserved;
} agx_params;

#define AGX_PREC_FP64  0
#define AGX_PREC_MIXED 1

/* Field identifiers for agx_set_field / agx_get_field / agx_device_ptr.
 * Centroid fields have N doubles, edge/vertex fields 3N, boundary fields B. */
enum {
  AGX_STAGE_C = 0, AGX_XMOM_C, AGX_YMOM_C, AGX_ELEV_C, AGX_FRICTION_C, AGX_HEIGHT_C,
  AGX_STAGE_E, AGX_XMOM_E, AGX_YMOM_E, AGX_ELEV_E, AGX_HEIGHT_E,
  AGX_STAGE_V, AGX_XMOM_V, AGX_YMOM_V, AGX_ELEV_V, AGX_HEIGHT_V,
  AGX_STAGE_B, AGX_XMOM_B, AGX_YMOM_B,
  AGX_STAGE_X, AGX_XMOM_X, AGX_YMOM_X,      /* explicit_update */
  AGX_STAGE_S, AGX_XMOM_S, AGX_YMOM_S,      /* semi_implicit_update */
  AGX_MAX_SPEED,
  AGX_FIELD_COUNT
};

/* Boundary kinds for agx_set_boundary (one per boundary edge). */
#define AGX_BC_NONE            0  /* segment bound to None: values untouched */
#define AGX_BC_REFLECTIVE      1  /* shallow_water/boundaries.py:235-292 */
#define AGX_BC_TRANSMISSIVE    2  /* generic_boundary_conditions.py:173-195 (edge values) */
#define AGX_BC_TRANSMISSIVE_C  3  /* same, centroid_transmissive_bc */
#define AGX_BC_DIRICHLET       4  /* generic_boundary_conditions.py:221-264 */
#define AGX_BC_TIME_SERIES     5  /* Time_boundary as a piecewise-linear table (generic_boundary_conditions.py:297-416) */
#define AGX_BC_TRANSMISSIVE_N0 6  /* stage given, normal momentum of the edge, tangential zero (shallow_water/boundaries.py:384-519) */
#define AGX_BC_TRANSMISSIVE_SET_STAGE 7  /* stage given, momenta of the edge (boundaries.py:295-383) */
#define AGX_BC_TRANSMISSIVE_ZERO_MOM  8  /* stage of the edge, momenta zero (boundaries.py:520-552) */
#define AGX_BC_FLATHER         9  /* outside stage given, zero outside velocity (boundaries.py:1096-1330) */
#define AGX_BC_CHARACTERISTIC 10  /* stage given, incoming-wave momentum (boundaries.py:639-848) */
#define AGX_BC_INFLOW         11  /* stage = edge bed + value 0 (a depth), momenta given (boundaries.py:902-992) */

/* Per-step statistics returned by agx_advance (generic_domain.py:1200
 * timestepping_statistics and the evolve bookkeeping). */
typedef struct {
  double time;                 /* relative time after the last step */
  double last_timestep;
  double min_timestep, max_timestep;   /* recorded over the call */
  double flux_timestep;
  double mass_added;           /* cumulative mass added by protection */
  double boundary_flux_sum[3];
  int64_t steps;               /* steps taken by this call */
  int64_t total_steps;
  int64_t negative_cells;      /* cumulative fix_negative_cells count */
  int32_t reason;              /* AGX_STOP_* */
  int32_t order;
  /* cumulative time integral of the boundary flux sums, accumulated after
   * every step as boundary_flux_integral_operator.__call__ does
   * (operators/boundary_flux_integral_operator.py:44-62) */
  double boundary_flux_integral;
  int64_t nonfinite_cells;     /* cell updates that produced NaN or Inf (the loop stops on the first) */
} agx_step_stats;

#define AGX_STOP_YIELD    1
#define AGX_STOP_FINAL    2
#define AGX_STOP_MAXSTEPS 3
#define AGX_STOP_ERROR    4

/* ---- lifetime ------------------------------------------------------------ */

/* Create a scenario on the current CUDA device: uploads the mesh tables and
 * allocates the state.  Replaces the Domain/Quantity numpy storage of
 * abstract_2d_finite_volumes/quantity.py:59-103 and the per-call marshalling
 * of sw_domain_openmp_ext.pyx:112-365. */
agx_status agx_scenario_create(const agx_mesh_desc* mesh, const agx_params* params, agx_handle* out);
agx_status agx_scenario_destroy(agx_handle h);

/* Device bytes a scenario with these sizes occupies (admission control). */
int64_t agx_scenario_footprint(int64_t n_cells, int64_t n_boundary, int64_t n_edges, int32_t precision);

/* ---- state ----------------------------------------------------------------- */

/* Copy a field between host memory and the device.  Quantity.set_values /
 * centroid_values access (quantity.py:709-1055). */
agx_status agx_set_field(agx_handle h, int32_t field, const double* host, int64_t n);
agx_status agx_get_field(agx_handle h, int32_t field, double* host, int64_t n);
/* Device address of a field (for zero-copy torch views).  Valid until destroy. */
agx_status agx_device_ptr(agx_handle h, int32_t field, void** ptr, int64_t* n);
/* The conserved centroid state (stage, xmomentum, ymomentum; N values each)
 * in one call with one synchronisation: the per-yield exchange of
 * Domain.get_conserved_quantities / set_quantity (quantity.py:709-1055). */
agx_status agx_set_state(agx_handle h, const double* w, const double* uh, const double* vh, int64_t n);
agx_status agx_get_state(agx_handle h, double* w, double* uh, double* vh, int64_t n);

/* Bind boundary conditions: kind[B] and values[B*3] (w, uh, vh) for
 * Dirichlet.  Domain.set_boundary + update_boundary (generic_domain.py:2288-2306). */
agx_status agx_set_boundary(agx_handle h, const int32_t* kind, const double* values, int64_t B);
/* Time series for AGX_BC_TIME_SERIES edges: rows of (t, w, uh, vh). */
agx_status agx_set_boundary_series(agx_handle h, const double* rows, int64_t n_rows);

/* Fractional-step rain/extraction: Rate_operator.__call__ with a constant
 * rate (operators/rate_operators.py:149-258).  indices == NULL: all cells. */
agx_status agx_add_rate_operator(agx_handle h, const int32_t* indices, int64_t n, double rate, double factor);
agx_status agx_clear_operators(agx_handle h);
/* Inlet_operator (structures/inlet_operator.py:17-165, inlet.py:107-226):
 * discharge Q (m^3/s) into the cells `indices` (at most 2048) of total area
 * `area`; flags & 1: momenta from the velocity (velocity_u, velocity_v);
 * flags & 2: zero velocity.  Applied after each step with the other
 * operators, in registration order. */
agx_status agx_add_inlet_operator(agx_handle h, const int32_t* indices, int64_t n, double Q, double area,
                                  int32_t flags, double velocity_u, double velocity_v);
/* One application of registered operator `op` (in registration order) with
 * the values and timestep the caller gives: for a Rate_operator the rate and
 * factor, for an Inlet_operator Q(t) and Q(t + timestep); used when these are
 * functions of time evaluated by the host. */
agx_status agx_apply_operator(agx_handle h, int32_t op, double rate, double factor, double timestep);
/* Cumulative influx (m^3) of operator `op` (Rate_operator.cumulative_influx). */
agx_status agx_operator_influx(agx_handle h, int32_t op, double* influx);

/* ---- per-phase calls (the reference's per-call plugin surface) ---------- */

/* protect_new -> _openmp_protect (sw_domain_openmp_ext.pyx:398-411). */
agx_status agx_protect(agx_handle h, double* mass_error);
/* extrapolate_second_order_edge_sw (sw_domain_openmp_ext.pyx:384-396),
 * including the protect step of distribute_to_vertices_and_edges when
 * with_protect != 0 (shallow_water_domain.py:1879-1915). */
agx_status agx_distribute(agx_handle h, int32_t with_protect);
/* Domain.update_boundary (generic_domain.py:2288-2306) at relative time t. */
agx_status agx_update_boundary(agx_handle h, double t);
/* compute_fluxes_ext_central (sw_domain_openmp_ext.pyx:371-382): returns the
 * flux timestep on substep 0 and evolve_max_timestep otherwise. */
agx_status agx_compute_fluxes(agx_handle h, int32_t substep, double* flux_timestep);
/* manning_friction_implicit (shallow_water/friction.py:23-72). */
agx_status agx_compute_forcing(agx_handle h);
/* update_conserved_quantities (shallow_water_domain.py:2089-2163). */
agx_status agx_update_conserved(agx_handle h, double timestep, int64_t* negative_cells);
/* backup_conserved_quantities / saxpy_conserved_quantities
 * (generic_domain.py:2187-2199). */
agx_status agx_backup(agx_handle h);
agx_status agx_saxpy(agx_handle h, double a, double b);
/* Riverwalls (structures/riverwall.py create_riverwalls; the weir branch of
 * the flux, sw_domain_openmp.c:324-426, 581-650): edge_counter[n_slots = 3N]
 * is the reference's edge_river_wall_counter (1-based riverwall edge of each
 * slot, 0 for ordinary edges); elevation and row_index[n_riverwall_edges] the
 * crest elevation and hydraulic-table row of each riverwall edge;
 * hydraulic[n_rows * ncol] the table (columns Qfactor, s1, s2, h1, h2).  The
 * mesh tables must evaluate riverwall slots per side (agx_mesh_desc edge
 * list: no shared edge flux for them).  n_riverwall_edges = 0 removes them. */
agx_status agx_set_riverwalls(agx_handle h, const int32_t* edge_counter, int64_t n_slots, int64_t n_riverwall_edges,
                              const double* elevation, const int32_t* row_index, int32_t n_rows, int32_t ncol,
                              const double* hydraulic);
/* Conserved centroid values divided by `divisor`: the last stage of
 * evolve_one_rk3_step, Q.centroid_values / 3.0 (generic_domain.py:2160-2166). */
agx_status agx_divide_conserved(agx_handle h, double divisor);

/* ---- device step loop ------------------------------------------------------ */

/* Fixed flux timestep in place of the CFL minimum (0: variable timestepping
 * again).  Domain.set_fixed_flux_timestep, generic_domain.py:2332-2346;
 * applied as update_timestep does, :2358-2359. */
agx_status agx_set_fixed_flux_timestep(agx_handle h, double flux_timestep);

/* Set the evolve clock: relative time, next yield time and final time
 * (final_time < 0: none).  _evolve_base bookkeeping (generic_domain.py:1715-1826). */
agx_status agx_set_clock(agx_handle h, double time, double yield_time, double final_time);
/* Advance on the device until the next yield time, the final time or
 * max_steps steps (whichever first), without host round trips: the step
 * loop of generic_domain.py:1835-1912 with evolve_one_euler_step (:1914) or
 * evolve_one_rk2_step (:1974).  The loop is captured once as a CUDA graph
 * with a device-side while node. */
agx_status agx_advance(agx_handle h, int64_t max_steps, agx_step_stats* out);
/* Issue all further work of this scenario on `stream` (a cudaStream_t such as
 * torch.cuda.current_stream().cuda_stream); NULL restores its own stream. */
agx_status agx_set_stream(agx_handle h, void* stream);
/* Per-kernel CUDA-event timing of `reps` steps issued as individual launches:
 * ms[c] is the average time per step of kernel category c (AGX_PHASE_*).
 * The state advances by `reps` steps. */
#define AGX_PHASE_PREP    0
#define AGX_PHASE_EXTRAP  1
#define AGX_PHASE_BC      2
#define AGX_PHASE_FLUX    3
#define AGX_PHASE_ACCUM   4
#define AGX_PHASE_UPDATE  5
#define AGX_PHASE_RATE    6
#define AGX_PHASE_SMALL   7
#define AGX_PHASE_COUNT   8
agx_status agx_time_phases(agx_handle h, int32_t reps, double* ms, int32_t n_cat);
/* Read the statistics without stepping. */
agx_status agx_get_stats(agx_handle h, agx_step_stats* out);

/* ---- sww output (file/sww.py:260-435 store_timestep, smoothed vertices) ------- */
/* Node -> vertex-slot map: the vertex slots 3k+i of node p are
 * node_slots[node_offsets[p] .. node_offsets[p+1]), summed in that order
 * (the reference's vertex_value_indices, general_mesh.py:740-850). */
agx_status agx_sww_bind(agx_handle h, int64_t P, const int32_t* node_offsets, const int32_t* node_slots);
/* One output frame from the device state, as SWW_file.store_timestep forms
 * it (file/sww.py:352-410): vertex_out[3P] = stage, xmomentum, ymomentum per
 * node, each the mean over the node's vertex slots of the centroid values of
 * their triangles (centroid_averaging = 1, what the DE algorithms set,
 * shallow_water_domain.py:596; quantity.c:872-915) or of the slots' vertex
 * values as last distributed (0; quantity.c:823-870); where the mean stage
 * minus the mean bed is below min_storable_height the stage is the bed and
 * the momenta are zero.  centroid_out[3N] = the centroid values as they
 * are.  Single precision, one device-to-host copy each. */
agx_status agx_sww_frame(agx_handle h, double min_storable_height, int32_t centroid_averaging, float* vertex_out,
                         float* centroid_out);
/* The same frame, formed and copied into a page-locked buffer of the library
 * on the scenario's stream without waiting, so that the host can write the
 * previous frame or issue the next yieldstep meanwhile. */
agx_status agx_sww_frame_async(agx_handle h, double min_storable_height, int32_t centroid_averaging);
/* Wait for the frame started last; *vertex [3P] and *centroid [3N] point
 * into the page-locked buffer, valid until the next agx_sww_frame_async,
 * agx_sww_bind or destroy. */
agx_status agx_sww_frame_wait(agx_handle h, const float** vertex, const float** centroid);

/* ---- diagnostics ------------------------------------------------------------- */
int32_t agx_last_error(char* buf, int32_t n);
int32_t agx_version(void);
/* Number of kernels this library launched since load (launch accounting). */
int64_t agx_kernel_launches(void);
/* FP64 throughput of the current device in G operations/s (DFMA, IEEE DDIV,
 * IEEE DSQRT), measured with dependent chains of 8-way ILP over the whole
 * device: the compute ceiling of the plain FP64 path.  No counterpart in the
 * reference (measurement only); allocates and frees a small result buffer. */
agx_status agx_fp64_throughput(double* dfma_gops, double* ddiv_gops, double* dsqrt_gops);
/* Throughput (G op/s) of binary64 add, multiply, divide and square root on
 * the FP64 pipe (out[0..3]), done with integer instructions with exact IEEE
 * rounding (out[4..7]; anuga_core_gb300/csrc/soft64.cuh) and split half and
 * half between the two (divide out[8], multiply out[9]).  No counterpart in
 * the reference (a GPU measurement). */
agx_status agx_soft64_throughput(double* out10);
/* n cases of each integer-instruction binary64 operation (add, sub, mul,
 * div, sqrt) run on the device against the FP64 pipe's IEEE results; writes
 * the number of mismatches of each to mism5 (a NaN result only has to be a
 * NaN).  No counterpart in the reference (a self-check of this library). */
agx_status agx_soft64_check(long long n, unsigned long long seed, unsigned long long* mism5);

#ifdef __cplusplus
}
#endif
#endif /* AGX_H */
