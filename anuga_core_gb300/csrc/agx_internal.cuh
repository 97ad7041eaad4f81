// agx_internal.cuh -- scenario object shared by the translation units of libagx.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <cstring>
#include "../../include/agx.h"
#include "de_plain.cuh"

namespace agx {

constexpr int MAX_OPS = 16;

// Device-resident clock and reductions of one scenario (all times relative).
struct Clock {
  double time, yield_time, final_time;   // final_time < 0: none
  double timestep, flux_timestep;
  float timestep32, pad_ts;              // (float)timestep, for the mixed-precision kernels
  double recorded_min, recorded_max;
  double cfl, max_dt, min_dt;
  double mass_added;
  double bfs[3];
  double bfs_acc;
  unsigned long long dt_key;             // ~bits(dt) of the running minimum (0 = none)
  long long steps_call, total_steps, steps_target, negative_cells;
  long long nonfinite_cells;             // cell updates that produced a NaN or an infinity
  int smallsteps, max_smallsteps, order, default_order;
  int error, reason, fluxcalls, pad1;    // fluxcalls: stages per step (1 euler, 2 rk2, 3 rk3)
  double bf_integral;                    // time integral of the boundary flux sums
  double fixed_flux_dt;                  // > 0: set_fixed_flux_timestep (replaces the CFL minimum)
  double op_influx[MAX_OPS];
};

enum ErrorBits { ERR_NUMERIC = 1, ERR_TIMESTEP = 2, ERR_OVERSHOOT = 4, ERR_NAN = 8, ERR_STEPCAP = 16,
                 ERR_NONFINITE = 32, ERR_BARRIER = 64 };

// A double that is NaN or an infinity (biased exponent all ones), tested on
// the high word with integer operations.
__host__ __device__ inline bool nonfinite64(double x) {
  long long b;
  memcpy(&b, &x, 8);
  return ((b >> 52) & 0x7ff) == 0x7ff;
}
// hard cap on the steps one agx_advance call may take on the device
constexpr long long MAX_STEPS_PER_CALL = 20000000;

// The timestep update_timestep takes from a flux timestep, without changing
// the clock (generic_domain.py:2349-2415): CFL scaling, the minimum timestep
// where the small-step count runs out at first order, the clamps to the final
// and the next yield time.  timestep_logic below applies the same steps with
// their bookkeeping; both give the same value for the same clock.
__host__ __device__ inline double timestep_value(const Clock* c, double flux_dt) {
  if (c->fixed_flux_dt > 0.0) flux_dt = c->fixed_flux_dt;
  double ts = fmin(c->cfl * flux_dt, c->max_dt);
  if (ts < c->min_dt && c->smallsteps + 1 > c->max_smallsteps && c->order == 1) ts = c->min_dt;
  if (c->final_time >= 0.0 && c->time + ts > c->final_time) ts = c->final_time - c->time;
  if (c->time + ts > c->yield_time) ts = c->yield_time - c->time;
  return ts;
}

// update_timestep (abstract_2d_finite_volumes/generic_domain.py:2349-2415):
// CFL scaling, small-step fallback to first order, clamp to the final and the
// next yield time.  Also publishes the flux timestep of the reduction key.
__host__ __device__ inline void timestep_logic(Clock* c) {
  const unsigned long long key = c->dt_key;
  double flux_dt = 1.0e100;
  if (key) {
    const unsigned long long bits = ~key;
    double v;
    memcpy(&v, &bits, 8);
    flux_dt = v;
  }
  if (c->fixed_flux_dt > 0.0) flux_dt = c->fixed_flux_dt;     // generic_domain.py:2358-2359
  c->flux_timestep = flux_dt;
  double ts = fmin(c->cfl * flux_dt, c->max_dt);
  c->recorded_max = fmax(ts, c->recorded_max);
  c->recorded_min = fmin(ts, c->recorded_min);
  if (ts < c->min_dt) {
    c->smallsteps += 1;
    if (c->smallsteps > c->max_smallsteps) {
      c->smallsteps = 0;
      if (c->order == 1) {
        c->error |= ERR_TIMESTEP;
        ts = c->min_dt;
      } else {
        c->order = 1;
      }
    }
  } else {
    c->smallsteps = 0;
    if (c->order == 1 && c->default_order == 2) c->order = 2;
  }
  if (c->final_time >= 0.0 && c->time + ts > c->final_time) ts = c->final_time - c->time;
  if (c->time + ts > c->yield_time) ts = c->yield_time - c->time;
  c->timestep = ts;
  c->timestep32 = (float)ts;
}

// End of one step (generic_domain.py:1851-1912): advance time, count, and
// decide whether the loop continues.  Returns the stop reason (0 = go on).
// Guards keep the device loop finite: a NaN time or timestep, a non-positive
// timestep or the per-call step cap end it with an error.
__host__ __device__ inline int clock_logic(Clock* c) {
  // boundary_flux_integral_operator.__call__ (operators/boundary_flux_integral_operator.py:44-62),
  // which the reference's Domain applies after every step: the step's
  // boundary flux sums weighted by its stages
  if (c->fluxcalls == 1) {
    c->bf_integral = c->bf_integral + c->timestep * c->bfs[0];
  } else if (c->fluxcalls == 2) {
    c->bf_integral = c->bf_integral + 0.5 * c->timestep * (c->bfs[0] + c->bfs[1]);
  } else if (c->fluxcalls == 3) {
    c->bf_integral = c->bf_integral + 1.0 / 6.0 * c->timestep * (c->bfs[0] + c->bfs[1] + 4.0 * c->bfs[2]);
  }
  c->time = c->time + c->timestep;
  c->steps_call += 1;
  c->total_steps += 1;
  int reason = 0;
  if (!(c->time == c->time) || !(c->timestep == c->timestep)) c->error |= ERR_NAN;
  if (!(c->timestep > 0.0) && !(c->final_time >= 0.0 && c->time >= c->final_time - 1.0e-12) &&
      !(c->time >= c->yield_time))
    c->error |= ERR_NAN;
  if (c->steps_call >= MAX_STEPS_PER_CALL) c->error |= ERR_STEPCAP;
  // A step that reaches the final or the yield time reports that even when it
  // is also the last step of the target count, so the next call does not
  // take a zero-length step.
  if (c->error) {
    reason = AGX_STOP_ERROR;
  } else if (c->final_time >= 0.0 && c->time >= c->final_time - 1.0e-12) {
    if (c->time > c->final_time) c->error |= ERR_OVERSHOOT;
    c->time = c->final_time;
    reason = AGX_STOP_FINAL;
  } else if (c->time >= c->yield_time) {
    reason = AGX_STOP_YIELD;
  } else if (c->steps_target > 0 && c->steps_call >= c->steps_target) {
    reason = AGX_STOP_MAXSTEPS;
  }
  c->reason = reason;
  return reason;
}

// A fractional-step operator: Rate_operator (kind 0) or Inlet_operator
// (kind 1: rate = constant discharge Q, vu/vv the imposed velocity when
// flags & 1, zero velocity when flags & 2, area = the inlet's total area).
struct RateOp {
  int* idx;        // device indices (nullptr: all cells)
  int n;
  double rate, factor;
  int kind = 0;
  int flags = 0;
  double vu = 0.0, vv = 0.0, area = 0.0;
};
constexpr int INLET_MAX = 2048;     // cells of one inlet region (one block sorts them)

// Everything a kernel needs, passed by value.
struct Dev {
  int N, B, E;
  Params P;
  const int4* conn;
  const int4* surr;
  const double* geo;
  const int* edge_slot;
  const int* edge_opp;
  const double* normals;
  const double* lengths;
  const double* radii;
  const double* areas;
  const double* inv_area;
  const double* vcoord;
  const int* bslot;
  const int* bkind;
  const double* bval;
  const double* bseries;
  int nseries;
  double *w, *uh, *vh, *z, *eta, *h, *u, *v;
  double *w0, *uh0, *vh0;
  double *we, *uhe, *vhe, *ze, *he;
  double *wv, *uhv, *vhv, *zv, *hv;
  double *wb, *uhb, *vhb;
  double *xw, *xuh, *xvh;
  double *sw, *suh, *svh;
  double *max_speed;
  double *sl0, *sl1, *sl2, *slsp, *slpf, *slhl;
  // the extrapolation's cell order: cells grouped by the branches they took
  // in the previous extrapolation (cls), so that the lanes of a warp follow
  // the same path; cls_count[0..255] counts, [256..511] scatter cursors
  int* order;
  unsigned char* cls;
  unsigned int* cls_count;
  Clock* clock;
  // riverwalls (structures/riverwall.py): per slot the 1-based riverwall
  // edge (0: ordinary edge), crest elevation and hydraulic-table row per
  // riverwall edge, the table [rows][rw_ncol]; all null without riverwalls
  const int* rw_counter;
  const double* rw_elev;
  const int* rw_row;
  const double* rw_hyd;
  int rw_ncol;
};

struct Scenario {
  int device = 0;
  int N = 0, B = 0, E = 0;
  // sww output: node -> vertex-slot CSR and a float staging buffer
  int P = 0;
  int* node_off = nullptr;
  int* node_slot = nullptr;
  float* frame = nullptr;
  float* frame_host = nullptr;           // pinned copy of the last frame (asynchronous output)
  cudaEvent_t frame_done = nullptr;      // recorded after that copy
  cudaEvent_t frame_ready = nullptr;     // recorded after the frame kernels
  cudaStream_t copy_stream = nullptr;    // the copy's own stream: the next steps need not wait for it
  agx_params prm{};
  Dev d{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  double* field[AGX_FIELD_COUNT] = {};
  int64_t field_len[AGX_FIELD_COUNT] = {};
  int* bkind = nullptr;
  double* bval = nullptr;
  double* bseries = nullptr;
  int nseries = 0;
  std::vector<RateOp> ops;
  Clock* clock_dev = nullptr;
  Clock* clock_host = nullptr;           // pinned
  cudaStream_t stream = nullptr;         // stream all work is issued on
  cudaStream_t own_stream = nullptr;     // the scenario's own (used for capture)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_valid = false;
  int kernels_per_step = 0;
  void* rw_mem = nullptr;                // riverwall tables (one allocation)
};

// NVTX ranges around the library's entry points (a no-op unless a profiler
// such as Nsight Systems is attached; generic_domain.py:47-54 wraps its step
// phases the same way)
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
#define AGX_TRACE(name) ::agx::TraceRange agx_trace_range_(name)

// launch accounting
void count_launch(int64_t n = 1);

// per-kernel event timing (agx_time_phases): categories of step kernels
enum Phase { PH_PREP = 0, PH_EXTRAP, PH_BC, PH_FLUX, PH_ACCUM, PH_UPDATE, PH_RATE, PH_SMALL, PH_COUNT };
void phase_mark(cudaStream_t st, int cat);
void set_capturing(bool on);
// start collecting events for one timed iteration / accumulate its per-category times
void begin_phase_timer();
void end_phase_timer(double* ms, int reps, cudaEvent_t start, int abort);

// implemented in agx_plain.cu
cudaError_t enqueue_step(Scenario* s, cudaStream_t st, unsigned long long cond_handle, bool set_cond);
cudaError_t enqueue_distribute(Scenario* s, cudaStream_t st, bool with_protect, bool vertices);
cudaError_t enqueue_rate_once(Scenario* s, cudaStream_t st, int op, double rate, double factor, double dt);
cudaError_t enqueue_op(Scenario* s, cudaStream_t st, int op, double rate, double factor, double dt);
cudaError_t enqueue_sww_frame(Scenario* s, cudaStream_t st, double min_storable_height, int centroid_avg);
cudaError_t enqueue_protect(Scenario* s, cudaStream_t st);
cudaError_t enqueue_boundary(Scenario* s, cudaStream_t st, double t_override, bool stage2);
cudaError_t enqueue_fluxes(Scenario* s, cudaStream_t st, int substep);
cudaError_t enqueue_update(Scenario* s, cudaStream_t st, int stage, bool use_clock_dt, double dt);
cudaError_t enqueue_forcing(Scenario* s, cudaStream_t st);
cudaError_t enqueue_backup(Scenario* s, cudaStream_t st);
cudaError_t enqueue_saxpy(Scenario* s, cudaStream_t st, double a, double b);
cudaError_t enqueue_divide(Scenario* s, cudaStream_t st, double divisor);
cudaError_t enqueue_reset_accum(Scenario* s, cudaStream_t st);
cudaError_t enqueue_order_init(Scenario* s, cudaStream_t st);

}  // namespace agx
