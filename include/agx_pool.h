/*
 * agx_pool.h -- C ABI of the mixed-precision scenario pool (libagx.so).
 *
 * A pool is one device arena holding many scenarios; every active scenario
 * advances together (one CUDA graph launch runs a device-side step loop over
 * all of them).  The mixed-precision form computes edge extrapolation and
 * fluxes in FP32 and accumulates the conserved quantities, the stage-minus-bed
 * depth and the timestep reduction in FP64.  It backs
 * Domain.set_gpu_options(precision='mixed'), the batched form and the serving
 * loop.  The reference has one domain per process and no pool; each entry
 * point names the reference interface whose role it takes for a scenario.
 *
 * Cells of a scenario are passed in the stored (space-filling-curve) order
 * built by anuga_core_gb300/tables.py pack_mixed(); fields are read and
 * written in the caller's original cell order.
 */
#ifndef AGX_POOL_H
#define AGX_POOL_H
#include <stdint.h>
#include "agx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct agx_pool_s* agx_pool;

/* Create a pool with room for cap_cells cells, cap_boundary boundary edges
 * and cap_scenarios scenarios (one cudaMalloc).  Replaces, per scenario, the
 * Domain/Quantity storage of abstract_2d_finite_volumes/quantity.py:59-103. */
agx_status agx_pool_create(int64_t cap_cells, int64_t cap_boundary, int32_t cap_scenarios, agx_pool* out);
agx_status agx_pool_destroy(agx_pool p);
/* Device bytes of a pool with these capacities (admission control). */
int64_t agx_pool_footprint(int64_t cap_cells, int64_t cap_boundary, int32_t cap_scenarios);
int64_t agx_pool_bytes_per_cell(void);
agx_status agx_pool_set_stream(agx_pool p, void* stream);

/* Add a scenario (Domain construction, shallow_water_domain.py:231):
 * conn[N*4], geo[N*16], area[N], radius[N] (FP64 inscribed-circle radii,
 * neighbour_mesh.py radii, in the stored order), order[N], boundary_cell[B],
 * lnk[N], halo_off/halo_cnt per tile of 128 cells, halo_cells[n_halo]. */
agx_status agx_pool_add(agx_pool p, int64_t N, int64_t B, const int32_t* conn, const float* geo,
                        const double* area, const double* radius, const int32_t* order,
                        const int32_t* boundary_cell,
                        const int32_t* lnk, const int32_t* halo_off, const int32_t* halo_cnt, int64_t n_halo,
                        const int32_t* halo_cells, const agx_params* params, int32_t* sid_out);
agx_status agx_pool_remove(agx_pool p, int32_t sid);
/* Free contiguous capacity. */
agx_status agx_pool_capacity(agx_pool p, int64_t* free_cells, int64_t* free_boundary, int64_t* free_halo,
                             int32_t* free_scenarios);

/* Quantity values (Quantity.set_values / centroid_values, quantity.py:709-1055):
 * AGX_STAGE_C, AGX_XMOM_C, AGX_YMOM_C, AGX_ELEV_C, AGX_FRICTION_C to set;
 * those, AGX_HEIGHT_C, AGX_MAX_SPEED, the explicit updates and the edge and
 * vertex fields to get. */
agx_status agx_pool_set_field(agx_pool p, int32_t sid, int32_t field, const double* host, int64_t n);
agx_status agx_pool_get_field(agx_pool p, int32_t sid, int32_t field, double* host, int64_t n);

/* The conserved state (stage, xmomentum, ymomentum; N values each) in one
 * call with one synchronisation.  Page-locked host buffers the device maps at
 * the same address are read or written by one kernel directly; other buffers
 * go through copies. */
agx_status agx_pool_set_state(agx_pool p, int32_t sid, const double* w, const double* uh, const double* vh, int64_t n);
agx_status agx_pool_get_state(agx_pool p, int32_t sid, double* w, double* uh, double* vh, int64_t n);

/* Boundary conditions (Domain.set_boundary, generic_domain.py:2288-2306). */
agx_status agx_pool_set_boundary(agx_pool p, int32_t sid, const int32_t* kind, const double* values, int64_t B);
agx_status agx_pool_set_boundary_series(agx_pool p, int32_t sid, const double* rows, int64_t n_rows);
/* Rate_operator with a constant rate (operators/rate_operators.py:149-258). */
agx_status agx_pool_add_rate(agx_pool p, int32_t sid, const int32_t* idx, int64_t n, double rate, double factor);
/* Inlet_operator (structures/inlet_operator.py:17-165, inlet.py:107-226):
 * discharge Q (m^3/s) into the cells idx[n] (at most 2048) of total area
 * `area`; flags & 1: momenta from (velocity_u, velocity_v); flags & 2: zero
 * velocity.  Same meaning as agx_add_inlet_operator. */
agx_status agx_pool_add_inlet(agx_pool p, int32_t sid, const int32_t* idx, int64_t n, double Q, double area,
                              int32_t flags, double velocity_u, double velocity_v);
/* on != 0: the scenario's operators are left out of the step loop and the
 * caller applies them after each step with agx_pool_apply_operator (rates,
 * factors or discharges that are functions of time, evaluated by the host). */
agx_status agx_pool_operators_from_host(agx_pool p, int32_t sid, int32_t on);
/* One application of registered operator `op` (registration order) with the
 * caller's values and timestep: a Rate_operator's rate and factor, an
 * Inlet_operator's Q(t) and Q(t + timestep).  Same meaning as
 * agx_apply_operator. */
agx_status agx_pool_apply_operator(agx_pool p, int32_t sid, int32_t op, double rate, double factor,
                                   double timestep);
/* Riverwalls of one scenario, with the arguments of agx_set_riverwalls
 * (edge_counter in the caller's cell order, 3 slots per cell); the pool's
 * flux kernels take the weir branch on the marked slots (FP32). */
agx_status agx_pool_set_riverwalls(agx_pool p, int32_t sid, const int32_t* edge_counter, int64_t n_slots,
                                   int64_t n_riverwall_edges, const double* elevation, const int32_t* row_index,
                                   int32_t n_rows, int32_t ncol, const double* hydraulic);
agx_status agx_pool_clear_operators(agx_pool p, int32_t sid);
agx_status agx_pool_operator_influx(agx_pool p, int32_t sid, int32_t op, double* influx);
/* distribute_to_vertices_and_edges (shallow_water_domain.py:1879-1915). */
agx_status agx_pool_distribute(agx_pool p, int32_t sid);

/* Fixed flux timestep of one scenario (0: variable timestepping again);
 * generic_domain.py:2332-2359. */
agx_status agx_pool_set_fixed_flux_timestep(agx_pool p, int32_t sid, double flux_timestep);

/* sww frames of one scenario formed on the device (agx_sww_frame of
 * include/agx.h: node means of centroid or vertex values in the given slot
 * order, storable-height mask at the nodes, centroid values as they are;
 * file/sww.py:352-410).  Vertex values are those of the mixed reconstruction
 * from the current state; slots are 3k+i in the original cell order. */
agx_status agx_pool_sww_bind(agx_pool p, int32_t sid, int64_t P, const int32_t* node_offsets,
                             const int32_t* node_slots);
agx_status agx_pool_sww_frame_async(agx_pool p, int32_t sid, double min_storable_height, int32_t centroid_averaging);
agx_status agx_pool_sww_frame_wait(agx_pool p, int32_t sid, const float** vertex, const float** centroid);

/* Evolve clock of one scenario (generic_domain.py:1715-1826): relative time,
 * next yield time, final time (< 0: none), step target (0: none). */
agx_status agx_pool_set_clock(agx_pool p, int32_t sid, double time, double yield_time, double final_time,
                              int64_t max_steps);
agx_status agx_pool_deactivate(agx_pool p, int32_t sid);
/* Step loop (generic_domain.py:1835-1912) for every active scenario until
 * each reaches its yield time, final time or step target; one graph launch. */
agx_status agx_pool_advance(agx_pool p, int32_t* n_done);
/* One step of every active scenario in two calls, without the graph, for
 * boundary values the host evaluates at each RK2 stage's time
 * (generic_domain.py:1974-2051 updates the boundary at t and at t + dt):
 * agx_pool_step_begin runs the first stage (flux, timestep, first update;
 * Euler scenarios are complete after it), after which agx_pool_get_stats
 * gives each scenario's timestep; agx_pool_step_end runs the second stage,
 * the operators of the step loop and the clocks. */
agx_status agx_pool_step_begin(agx_pool p);
/* Runs stage 2, then (rk3 scenarios) stage 3 of the split step on its own,
 * so that boundary values for the stage's time (t + dt, then t + dt/2) can
 * be set before it; agx_pool_step_end runs the stages not run yet.
 * AGX_E_STATE if called out of order. */
agx_status agx_pool_step_stage(agx_pool p, int32_t stage);
agx_status agx_pool_step_end(agx_pool p, int32_t* n_done);
/* Continuous batching: up to max_steps more steps for every running scenario,
 * launched without waiting; agx_pool_wait completes it. */
agx_status agx_pool_launch_chunk(agx_pool p, int64_t max_steps);
agx_status agx_pool_wait(agx_pool p, int32_t* n_running);
agx_status agx_pool_get_stats(agx_pool p, int32_t sid, agx_step_stats* out);
agx_status agx_pool_stats_all(agx_pool p, int32_t n, const int32_t* sids, agx_step_stats* out, int32_t* running);

/* Autotuning and checkpoints: kernel variant, state snapshot / restore. */
agx_status agx_pool_set_variant(agx_pool p, int32_t variant, int32_t grid_mode);
agx_status agx_pool_snapshot(agx_pool p);
agx_status agx_pool_restore(agx_pool p);
agx_status agx_pool_time_phases(agx_pool p, int32_t reps, double* ms, int32_t n_cat);
int32_t agx_pool_grid(agx_pool p);
/* Keep the work records the flux kernels gather resident in L2 through an
 * access policy window (1) or not (0, the default); timed by the autotuner.
 * Switching it on sets this context's persisting L2 size to the device's
 * maximum.  No counterpart in the reference (a GPU cache policy). */
agx_status agx_pool_set_l2_window(agx_pool p, int32_t on);
int32_t agx_pool_last_error(char* buf, int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* AGX_POOL_H */
