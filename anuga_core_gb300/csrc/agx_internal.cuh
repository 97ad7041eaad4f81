// agx_internal.cuh -- scenario object shared by the translation units of libagx.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/agx.h"
#include "de_plain.cuh"

namespace agx {

constexpr int MAX_OPS = 16;

// Device-resident clock and reductions of one scenario (all times relative).
struct Clock {
  double time, yield_time, final_time;   // final_time < 0: none
  double timestep, flux_timestep;
  double recorded_min, recorded_max;
  double cfl, max_dt, min_dt;
  double mass_added;
  double bfs[3];
  double bfs_acc;
  unsigned long long dt_key;             // ~bits(dt) of the running minimum (0 = none)
  long long steps_call, total_steps, steps_target, negative_cells;
  int smallsteps, max_smallsteps, order, default_order;
  int error, reason, pad0, pad1;
  double op_influx[MAX_OPS];
};

enum ErrorBits { ERR_NUMERIC = 1, ERR_TIMESTEP = 2, ERR_OVERSHOOT = 4, ERR_NAN = 8, ERR_STEPCAP = 16 };
// hard cap on the steps one agx_advance call may take on the device
constexpr long long MAX_STEPS_PER_CALL = 20000000;

struct RateOp {
  int* idx;        // device indices (nullptr: all cells)
  int n;
  double rate, factor;
};

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
  Clock* clock;
};

struct Scenario {
  int device = 0;
  int N = 0, B = 0, E = 0;
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
};

// launch accounting
void count_launch(int64_t n = 1);

// per-kernel event timing (agx_time_phases): categories of step kernels
enum Phase { PH_PREP = 0, PH_EXTRAP, PH_BC, PH_FLUX, PH_ACCUM, PH_UPDATE, PH_RATE, PH_SMALL, PH_COUNT };
void phase_mark(cudaStream_t st, int cat);

// implemented in agx_plain.cu
cudaError_t enqueue_step(Scenario* s, cudaStream_t st, unsigned long long cond_handle, bool set_cond);
cudaError_t enqueue_distribute(Scenario* s, cudaStream_t st, bool with_protect, bool vertices);
cudaError_t enqueue_protect(Scenario* s, cudaStream_t st);
cudaError_t enqueue_boundary(Scenario* s, cudaStream_t st, double t_override, bool stage2);
cudaError_t enqueue_fluxes(Scenario* s, cudaStream_t st, int substep);
cudaError_t enqueue_update(Scenario* s, cudaStream_t st, int stage, bool use_clock_dt, double dt);
cudaError_t enqueue_forcing(Scenario* s, cudaStream_t st);
cudaError_t enqueue_backup(Scenario* s, cudaStream_t st);
cudaError_t enqueue_saxpy(Scenario* s, cudaStream_t st, double a, double b);
cudaError_t enqueue_reset_accum(Scenario* s, cudaStream_t st);

}  // namespace agx
