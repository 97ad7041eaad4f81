// agx_api.cu -- C ABI of libagx: scenario lifetime, state access, per-phase
// calls and the graph-captured device step loop.
#include "agx_internal.cuh"
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace agx {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};
static thread_local bool g_capturing = false;

void count_launch(int64_t n) {
  if (!g_capturing) g_launches += n;
}

// Event timer used by agx_time_phases: an event after every launch.
struct PhaseTimer {
  std::vector<cudaEvent_t> ev;
  std::vector<int> cat;
  size_t used = 0;
};
static thread_local PhaseTimer* g_timer = nullptr;

void set_capturing(bool on) { g_capturing = on; }

static thread_local PhaseTimer g_shared_timer;

void begin_phase_timer() {
  g_shared_timer.used = 0;
  g_timer = &g_shared_timer;
}

void end_phase_timer(double* ms, int reps, cudaEvent_t start, int abort) {
  g_timer = nullptr;
  if (abort || !ms) return;
  cudaEvent_t prev = start;
  for (size_t i = 0; i < g_shared_timer.used; i++) {
    float t = 0.f;
    cudaEventElapsedTime(&t, prev, g_shared_timer.ev[i]);
    ms[g_shared_timer.cat[i]] += t / reps;
    prev = g_shared_timer.ev[i];
  }
}

void phase_mark(cudaStream_t st, int c) {
  if (!g_timer) return;
  PhaseTimer& T = *g_timer;
  if (T.used == T.ev.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    T.ev.push_back(e);
    T.cat.push_back(0);
  }
  T.cat[T.used] = c;
  cudaEventRecord(T.ev[T.used], st);
  T.used++;
}

static agx_status fail(agx_status code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(AGX_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),   \
                  __FILE__, __LINE__);                                                  \
  } while (0)

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Layout of the scenario arena: returns total bytes and (if base != null)
// assigns the pointers.
static size_t layout(Scenario* s, char* base) {
  const size_t N = s->N, B = s->B, E = s->E;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += align_up(bytes ? bytes : 8);
    return p;
  };
  Dev& d = s->d;
  d.conn = (const int4*)take(N * sizeof(int4));
  d.surr = (const int4*)take(N * sizeof(int4));
  d.geo = (const double*)take(N * GEO_STRIDE * 8);
  d.edge_slot = (const int*)take(E * 4);
  d.edge_opp = (const int*)take(E * 4);
  d.normals = (const double*)take(N * 6 * 8);
  d.lengths = (const double*)take(N * 3 * 8);
  d.radii = (const double*)take(N * 8);
  d.areas = (const double*)take(N * 8);
  d.inv_area = (const double*)take(N * 8);
  d.vcoord = (const double*)take(N * 6 * 8);
  d.bslot = (const int*)take(B * 4);
  s->bkind = (int*)take(B * 4);
  s->bval = (double*)take(B * 3 * 8);
  double** cen[] = {&d.w, &d.uh, &d.vh, &d.z, &d.eta, &d.h, &d.u, &d.v, &d.w0, &d.uh0, &d.vh0,
                    &d.xw, &d.xuh, &d.xvh, &d.sw, &d.suh, &d.svh, &d.max_speed};
  for (double** p : cen) *p = (double*)take(N * 8);
  double** edg[] = {&d.we, &d.uhe, &d.vhe, &d.ze, &d.he, &d.wv, &d.uhv, &d.vhv, &d.zv, &d.hv,
                    &d.sl0, &d.sl1, &d.sl2, &d.slsp, &d.slpf, &d.slhl};
  for (double** p : edg) *p = (double*)take(N * 3 * 8);
  double** bnd[] = {&d.wb, &d.uhb, &d.vhb};
  for (double** p : bnd) *p = (double*)take(B * 8);
  d.order = (int*)take(N * 4);
  d.cls = (unsigned char*)take(N);
  d.cls_count = (unsigned int*)take(512 * 4);
  d.clock = (Clock*)take(sizeof(Clock));
  return off;
}

static void bind_fields(Scenario* s) {
  Dev& d = s->d;
  const int64_t N = s->N, B = s->B;
  double* f[AGX_FIELD_COUNT] = {d.w, d.uh, d.vh, d.z, d.eta, d.h, d.we, d.uhe, d.vhe, d.ze, d.he,
                                d.wv, d.uhv, d.vhv, d.zv, d.hv, d.wb, d.uhb, d.vhb, d.xw, d.xuh,
                                d.xvh, d.sw, d.suh, d.svh, d.max_speed};
  for (int i = 0; i < AGX_FIELD_COUNT; i++) {
    s->field[i] = f[i];
    int64_t n = N;
    if (i >= AGX_STAGE_E && i <= AGX_HEIGHT_V) n = 3 * N;
    if (i >= AGX_STAGE_B && i <= AGX_YMOM_B) n = B;
    s->field_len[i] = n;
  }
}

static void init_clock(Clock* c, const agx_params& p) {
  memset(c, 0, sizeof(Clock));
  c->final_time = -1.0;
  c->yield_time = 1.0e300;
  c->cfl = p.CFL;
  c->max_dt = p.evolve_max_timestep;
  c->min_dt = p.evolve_min_timestep;
  c->recorded_min = p.evolve_max_timestep;
  c->recorded_max = p.evolve_min_timestep;
  c->max_smallsteps = p.max_smallsteps;
  c->order = 2;
  c->default_order = 2;
  c->flux_timestep = p.evolve_max_timestep;
  c->fluxcalls = p.timestepping_method;
}

static agx_status sync(Scenario* s) {
  CK(cudaStreamSynchronize(s->stream));
  return AGX_OK;
}

static agx_status pull_clock(Scenario* s) {
  CK(cudaMemcpyAsync(s->clock_host, s->d.clock, sizeof(Clock), cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

static agx_status push_clock(Scenario* s) {
  CK(cudaMemcpyAsync(s->d.clock, s->clock_host, sizeof(Clock), cudaMemcpyHostToDevice, s->stream));
  return sync(s);
}

static agx_status check_errors(Scenario* s) {
  const int e = s->clock_host->error;
  if (e & ERR_NONFINITE)
    return fail(AGX_E_NUMERIC, "non-finite conserved quantity (NaN or Inf) in %lld cell updates; the step loop "
                "stopped", (long long)s->clock_host->nonfinite_cells);
  if (e & ERR_NUMERIC) return fail(AGX_E_NUMERIC, "update: non-positive semi-implicit denominator");
  if (e & ERR_TIMESTEP) return fail(AGX_E_TIMESTEP, "too small timestep reached after %d steps at first order", s->prm.max_smallsteps);
  if (e & ERR_OVERSHOOT) return fail(AGX_E_OVERSHOOT, "time overshot finaltime");
  if (e & ERR_NAN) return fail(AGX_E_NUMERIC, "non-finite or non-positive timestep (state diverged)");
  if (e & ERR_STEPCAP) return fail(AGX_E_STATE, "device loop hit the per-call step cap");
  return AGX_OK;
}

static void destroy_graph(Scenario* s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->exec = nullptr;
  s->graph = nullptr;
  s->graph_valid = false;
}

static agx_status build_graph(Scenario* s) {
  destroy_graph(s);
  CK(cudaGraphCreate(&s->graph, 0));
  cudaGraphConditionalHandle handle;
  CK(cudaGraphConditionalHandleCreate(&handle, s->graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = handle;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, s->graph, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  // capture on the scenario's own stream (the caller's may be the legacy default stream)
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaStreamBeginCaptureToGraph(s->own_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  g_capturing = true;
  cudaError_t e = enqueue_step(s, s->own_stream, (unsigned long long)handle, true);
  g_capturing = false;
  cudaGraph_t captured = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s->own_stream, &captured);
  if (e != cudaSuccess) return fail(AGX_E_CUDA, "step capture failed: %s", cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(AGX_E_CUDA, "end capture failed: %s", cudaGetErrorString(e2));
  CK(cudaGraphInstantiate(&s->exec, s->graph, 0));
  // kernels per body iteration
  size_t nn = 0;
  CK(cudaGraphGetNodes(body, nullptr, &nn));
  s->kernels_per_step = (int)nn;
  s->graph_valid = true;
  return AGX_OK;
}

}  // namespace agx

struct agx_scenario : public agx::Scenario {};

using namespace agx;

extern "C" {

int32_t agx_version(void) { return 1; }

int64_t agx_kernel_launches(void) { return g_launches.load(); }

int32_t agx_last_error(char* buf, int32_t n) {
  if (buf && n > 0) {
    strncpy(buf, g_err, (size_t)n - 1);
    buf[n - 1] = 0;
  }
  return (int32_t)strlen(g_err);
}

int64_t agx_scenario_footprint(int64_t n_cells, int64_t n_boundary, int64_t n_edges, int32_t precision) {
  Scenario tmp;
  tmp.N = (int)n_cells;
  tmp.B = (int)n_boundary;
  tmp.E = (int)n_edges;
  (void)precision;
  return (int64_t)layout(&tmp, nullptr);
}

agx_status agx_scenario_create(const agx_mesh_desc* m, const agx_params* p, agx_handle* out) {
  AGX_TRACE("agx_scenario_create");
  if (!m || !p || !out) return fail(AGX_E_INVALID, "null argument");
  *out = nullptr;
  if (m->n_cells < 0 || m->n_cells >= (1ll << 29) || m->n_boundary < 0 || m->n_edges < 0)
    return fail(AGX_E_INVALID, "mesh sizes out of range");
  if (p->timestepping_method < 1 || p->timestepping_method > 3)
    return fail(AGX_E_INVALID, "timestepping_method must be 1 (euler), 2 (rk2) or 3 (rk3)");
  if (p->precision != AGX_PREC_FP64)
    return fail(AGX_E_INVALID, "this entry point builds the plain FP64 form; use agx_mixed_create for mixed precision");
  agx_scenario* s = new agx_scenario();
  s->N = (int)m->n_cells;
  s->B = (int)m->n_boundary;
  s->E = (int)m->n_edges;
  s->prm = *p;
  CK(cudaGetDevice(&s->device));
  size_t bytes = layout(s, nullptr);
  void* arena = nullptr;
  cudaError_t e = cudaMalloc(&arena, bytes);
  if (e != cudaSuccess) {
    delete s;
    return fail(AGX_E_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  s->arena = arena;
  s->arena_bytes = bytes;
  layout(s, (char*)arena);
  bind_fields(s);
  Params& P = s->d.P;
  P.g = p->g;
  P.epsilon = p->epsilon;
  P.hmin = p->minimum_allowed_height;
  P.beta_w = p->beta_w;
  P.beta_w_dry = p->beta_w_dry;
  P.beta_uh = p->beta_uh;
  P.beta_uh_dry = p->beta_uh_dry;
  P.beta_vh = p->beta_vh;
  P.beta_vh_dry = p->beta_vh_dry;
  P.c_tmp = 1.0 / (0.3 - 0.1);
  P.d_tmp = 1.0 - (P.c_tmp * 0.3);
  P.velocity_extrapolation = p->extrapolate_velocity_second_order == 1;
  P.low_froude = p->low_froude;
  P.protect_zero_ymom = p->protect_zero_ymom;
  P.sloped_mannings = p->use_sloped_mannings;
  finish_params(P);
  s->d.N = s->N;
  s->d.B = s->B;
  s->d.E = s->E;
  s->d.bkind = s->bkind;
  s->d.bval = s->bval;
  s->d.bseries = nullptr;
  s->d.nseries = 0;
  *out = s;
  agx_status st = AGX_OK;
  auto fin = [&](agx_status code) {
    agx_scenario_destroy(s);
    *out = nullptr;
    return code;
  };
  if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess) return fin(fail(AGX_E_CUDA, "stream create failed"));
  s->stream = s->own_stream;
  if (cudaMallocHost(&s->clock_host, sizeof(Clock)) != cudaSuccess) return fin(fail(AGX_E_NOMEM, "pinned clock alloc failed"));
  if (cudaMemsetAsync(arena, 0, bytes, s->stream) != cudaSuccess) return fin(fail(AGX_E_CUDA, "memset failed"));
  if (enqueue_order_init(s, s->stream) != cudaSuccess) return fin(fail(AGX_E_CUDA, "order init failed"));
  const size_t N = s->N, B = s->B, E = s->E;
  struct Up { const void* src; const void* dst; size_t bytes; } ups[] = {
      {m->conn, s->d.conn, N * 16}, {m->surr, s->d.surr, N * 16}, {m->geo, s->d.geo, N * GEO_STRIDE * 8},
      {m->edge_slot, s->d.edge_slot, E * 4}, {m->edge_opp, s->d.edge_opp, E * 4},
      {m->normals, s->d.normals, N * 48}, {m->edgelengths, s->d.lengths, N * 24},
      {m->radii, s->d.radii, N * 8}, {m->areas, s->d.areas, N * 8}, {m->inv_area, s->d.inv_area, N * 8},
      {m->vertex_coordinates, s->d.vcoord, N * 48}, {m->boundary_slot, s->d.bslot, B * 4}};
  for (auto& u : ups) {
    if (!u.bytes) continue;
    if (!u.src) return fin(fail(AGX_E_INVALID, "mesh table missing"));
    if (cudaMemcpyAsync((void*)u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
      return fin(fail(AGX_E_CUDA, "table upload failed"));
  }
  init_clock(s->clock_host, *p);
  if ((st = push_clock(s)) != AGX_OK) return fin(st);
  return AGX_OK;
}

agx_status agx_scenario_destroy(agx_handle h) {
  if (!h) return AGX_OK;
  agx_scenario* s = h;
  destroy_graph(s);
  for (auto& op : s->ops)
    if (op.idx) cudaFree(op.idx);
  if (s->node_off) cudaFree(s->node_off);
  if (s->node_slot) cudaFree(s->node_slot);
  if (s->frame) cudaFree(s->frame);
  if (s->copy_stream) {
    cudaStreamSynchronize(s->copy_stream);
    cudaStreamDestroy(s->copy_stream);
  }
  if (s->frame_host) cudaFreeHost(s->frame_host);
  if (s->frame_done) cudaEventDestroy(s->frame_done);
  if (s->frame_ready) cudaEventDestroy(s->frame_ready);
  if (s->bseries) cudaFree(s->bseries);
  if (s->rw_mem) cudaFree(s->rw_mem);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->own_stream) cudaStreamSynchronize(s->own_stream);
  if (s->arena) cudaFree(s->arena);
  if (s->clock_host) cudaFreeHost(s->clock_host);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return AGX_OK;
}

agx_status agx_set_field(agx_handle h, int32_t f, const double* host, int64_t n) {
  if (!h || f < 0 || f >= AGX_FIELD_COUNT) return fail(AGX_E_INVALID, "bad handle or field");
  if (n != h->field_len[f]) return fail(AGX_E_INVALID, "field %d expects %lld values, got %lld", f, (long long)h->field_len[f], (long long)n);
  if (n == 0) return AGX_OK;
  CK(cudaMemcpyAsync(h->field[f], host, (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

agx_status agx_get_field(agx_handle h, int32_t f, double* host, int64_t n) {
  if (!h || f < 0 || f >= AGX_FIELD_COUNT) return fail(AGX_E_INVALID, "bad handle or field");
  if (n != h->field_len[f]) return fail(AGX_E_INVALID, "field %d holds %lld values, asked for %lld", f, (long long)h->field_len[f], (long long)n);
  if (n == 0) return AGX_OK;
  CK(cudaMemcpyAsync(host, h->field[f], (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

// The conserved centroid state (stage, xmomentum, ymomentum) in one call:
// three copies on the scenario's stream and one synchronisation.
agx_status agx_set_state(agx_handle h, const double* w, const double* uh, const double* vh, int64_t n) {
  AGX_TRACE("agx_set_state");
  if (!h || !w || !uh || !vh) return fail(AGX_E_INVALID, "bad arguments");
  if (n != h->N) return fail(AGX_E_INVALID, "the state has %d cells, got %lld", h->N, (long long)n);
  if (n == 0) return AGX_OK;
  CK(cudaMemcpyAsync(h->field[AGX_STAGE_C], w, (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->field[AGX_XMOM_C], uh, (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->field[AGX_YMOM_C], vh, (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

agx_status agx_get_state(agx_handle h, double* w, double* uh, double* vh, int64_t n) {
  AGX_TRACE("agx_get_state");
  if (!h || !w || !uh || !vh) return fail(AGX_E_INVALID, "bad arguments");
  if (n != h->N) return fail(AGX_E_INVALID, "the state has %d cells, asked for %lld", h->N, (long long)n);
  if (n == 0) return AGX_OK;
  CK(cudaMemcpyAsync(w, h->field[AGX_STAGE_C], (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(uh, h->field[AGX_XMOM_C], (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(vh, h->field[AGX_YMOM_C], (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

agx_status agx_sww_bind(agx_handle h, int64_t P, const int32_t* node_offsets, const int32_t* node_slots) {
  if (!h || P < 0 || (P > 0 && (!node_offsets || !node_slots))) return fail(AGX_E_INVALID, "bad arguments");
  if (node_offsets[0] != 0 || node_offsets[P] != 3 * (int64_t)h->N)
    return fail(AGX_E_INVALID, "node offsets must run from 0 to 3N");
  for (int64_t p = 0; p < P; p++)
    if (node_offsets[p + 1] < node_offsets[p]) return fail(AGX_E_INVALID, "node offsets must not decrease");
  for (int64_t q = 0; q < 3 * (int64_t)h->N; q++)
    if (node_slots[q] < 0 || node_slots[q] >= 3 * h->N) return fail(AGX_E_INVALID, "vertex slot out of range");
  agx_status st = sync(h);
  if (st) return st;
  if (h->node_off) cudaFree(h->node_off);
  if (h->node_slot) cudaFree(h->node_slot);
  if (h->frame) cudaFree(h->frame);
  if (h->copy_stream) CK(cudaStreamSynchronize(h->copy_stream));
  if (h->frame_host) cudaFreeHost(h->frame_host);
  if (h->frame_done) cudaEventDestroy(h->frame_done);
  if (h->frame_ready) cudaEventDestroy(h->frame_ready);
  h->node_off = h->node_slot = nullptr;
  h->frame = h->frame_host = nullptr;
  h->frame_done = h->frame_ready = nullptr;
  h->P = (int)P;
  const size_t fbytes = ((size_t)3 * P + 3 * (size_t)h->N) * 4 + 4;
  CK(cudaMalloc(&h->node_off, (size_t)(P + 1) * 4));
  CK(cudaMalloc(&h->node_slot, (size_t)3 * h->N * 4 + 4));
  CK(cudaMalloc(&h->frame, fbytes));
  CK(cudaMallocHost(&h->frame_host, fbytes));
  CK(cudaEventCreateWithFlags(&h->frame_done, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->frame_ready, cudaEventDisableTiming));
  if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  CK(cudaMemcpyAsync(h->node_off, node_offsets, (size_t)(P + 1) * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->node_slot, node_slots, (size_t)3 * h->N * 4, cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

agx_status agx_sww_frame(agx_handle h, double min_storable_height, int32_t centroid_averaging, float* vertex_out,
                         float* centroid_out) {
  AGX_TRACE("agx_sww_frame");
  if (!h || !vertex_out || !centroid_out) return fail(AGX_E_INVALID, "bad arguments");
  if (!h->frame) return fail(AGX_E_STATE, "agx_sww_bind first");
  CK(cudaStreamWaitEvent(h->stream, h->frame_done, 0));     // an earlier asynchronous copy of the buffer
  CK(enqueue_sww_frame(h, h->stream, min_storable_height, centroid_averaging ? 1 : 0));
  if (h->P > 0) CK(cudaMemcpyAsync(vertex_out, h->frame, (size_t)3 * h->P * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(centroid_out, h->frame + 3 * (size_t)h->P, (size_t)3 * h->N * 4, cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

agx_status agx_sww_frame_async(agx_handle h, double min_storable_height, int32_t centroid_averaging) {
  AGX_TRACE("agx_sww_frame_async");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  if (!h->frame) return fail(AGX_E_STATE, "agx_sww_bind first");
  // the frame kernels wait for the previous frame's copy to leave the buffer;
  // the copy runs on its own stream, so the steps enqueued next overlap it
  CK(cudaStreamWaitEvent(h->stream, h->frame_done, 0));
  CK(enqueue_sww_frame(h, h->stream, min_storable_height, centroid_averaging ? 1 : 0));
  CK(cudaEventRecord(h->frame_ready, h->stream));
  CK(cudaStreamWaitEvent(h->copy_stream, h->frame_ready, 0));
  CK(cudaMemcpyAsync(h->frame_host, h->frame, ((size_t)3 * h->P + 3 * (size_t)h->N) * 4, cudaMemcpyDeviceToHost,
                     h->copy_stream));
  CK(cudaEventRecord(h->frame_done, h->copy_stream));
  return AGX_OK;
}

agx_status agx_sww_frame_wait(agx_handle h, const float** vertex, const float** centroid) {
  if (!h || !vertex || !centroid) return fail(AGX_E_INVALID, "bad arguments");
  if (!h->frame_host) return fail(AGX_E_STATE, "agx_sww_bind first");
  CK(cudaEventSynchronize(h->frame_done));
  *vertex = h->frame_host;
  *centroid = h->frame_host + 3 * (size_t)h->P;
  return AGX_OK;
}

agx_status agx_device_ptr(agx_handle h, int32_t f, void** ptr, int64_t* n) {
  if (!h || f < 0 || f >= AGX_FIELD_COUNT || !ptr) return fail(AGX_E_INVALID, "bad handle or field");
  *ptr = h->field[f];
  if (n) *n = h->field_len[f];
  return AGX_OK;
}

agx_status agx_set_boundary(agx_handle h, const int32_t* kind, const double* values, int64_t B) {
  if (!h || B != h->B) return fail(AGX_E_INVALID, "boundary arrays must have B=%d entries", h ? h->B : -1);
  if (B == 0) return AGX_OK;
  for (int64_t i = 0; i < B; i++)
    if (kind[i] < AGX_BC_NONE || kind[i] > AGX_BC_INFLOW)
      return fail(AGX_E_INVALID, "bad boundary kind %d at %lld", kind[i], (long long)i);
  CK(cudaMemcpyAsync(h->bkind, kind, (size_t)B * 4, cudaMemcpyHostToDevice, h->stream));
  if (values) CK(cudaMemcpyAsync(h->bval, values, (size_t)B * 24, cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

agx_status agx_set_boundary_series(agx_handle h, const double* rows, int64_t n_rows) {
  if (!h || n_rows < 0) return fail(AGX_E_INVALID, "bad arguments");
  agx_status st = sync(h);
  if (st) return st;
  if (h->bseries) cudaFree(h->bseries);
  h->bseries = nullptr;
  h->nseries = 0;
  if (n_rows > 0) {
    CK(cudaMalloc(&h->bseries, (size_t)n_rows * 32));
    CK(cudaMemcpyAsync(h->bseries, rows, (size_t)n_rows * 32, cudaMemcpyHostToDevice, h->stream));
    h->nseries = (int)n_rows;
  }
  h->d.bseries = h->bseries;
  h->d.nseries = h->nseries;
  h->graph_valid = false;
  return sync(h);
}

agx_status agx_add_rate_operator(agx_handle h, const int32_t* indices, int64_t n, double rate, double factor) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  if ((int)h->ops.size() >= MAX_OPS) return fail(AGX_E_INVALID, "at most %d operators", MAX_OPS);
  RateOp op{nullptr, h->N, rate, factor};
  if (indices) {
    for (int64_t i = 0; i < n; i++)
      if (indices[i] < 0 || indices[i] >= h->N) return fail(AGX_E_INVALID, "operator index %d out of range", indices[i]);
    op.n = (int)n;
    if (n > 0) {
      CK(cudaMalloc(&op.idx, (size_t)n * 4));
      CK(cudaMemcpyAsync(op.idx, indices, (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
    }
  }
  h->ops.push_back(op);
  h->graph_valid = false;
  return sync(h);
}

agx_status agx_add_inlet_operator(agx_handle h, const int32_t* indices, int64_t n, double Q, double area,
                                  int32_t flags, double velocity_u, double velocity_v) {
  if (!h || !indices || n <= 0) return fail(AGX_E_INVALID, "an inlet needs at least one cell");
  if (n > INLET_MAX) return fail(AGX_E_INVALID, "an inlet region holds at most %d cells, got %lld", INLET_MAX, (long long)n);
  if (!(area > 0.0)) return fail(AGX_E_INVALID, "inlet area must be positive");
  if ((int)h->ops.size() >= MAX_OPS) return fail(AGX_E_INVALID, "at most %d operators", MAX_OPS);
  for (int64_t i = 0; i < n; i++)
    if (indices[i] < 0 || indices[i] >= h->N) return fail(AGX_E_INVALID, "inlet index %d out of range", indices[i]);
  RateOp op{nullptr, (int)n, Q, 1.0};
  op.kind = 1;
  op.flags = flags;
  op.vu = velocity_u;
  op.vv = velocity_v;
  op.area = area;
  CK(cudaMalloc(&op.idx, (size_t)n * 4));
  CK(cudaMemcpyAsync(op.idx, indices, (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
  h->ops.push_back(op);
  h->graph_valid = false;
  return sync(h);
}

agx_status agx_apply_operator(agx_handle h, int32_t op, double rate, double factor, double timestep) {
  AGX_TRACE("agx_apply_operator");
  if (!h || op < 0 || op >= (int)h->ops.size() || !(timestep >= 0.0))
    return fail(AGX_E_INVALID, "bad operator %d or timestep", op);
  CK(enqueue_rate_once(h, h->stream, op, rate, factor, timestep));
  return sync(h);
}

agx_status agx_clear_operators(agx_handle h) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = sync(h);
  if (st) return st;
  for (auto& op : h->ops)
    if (op.idx) cudaFree(op.idx);
  h->ops.clear();
  h->graph_valid = false;
  return AGX_OK;
}

agx_status agx_operator_influx(agx_handle h, int32_t op, double* influx) {
  if (!h || op < 0 || op >= MAX_OPS || !influx) return fail(AGX_E_INVALID, "bad arguments");
  agx_status st = pull_clock(h);
  if (st) return st;
  *influx = h->clock_host->op_influx[op];
  return AGX_OK;
}

agx_status agx_protect(agx_handle h, double* mass_error) {
  AGX_TRACE("agx_protect");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = pull_clock(h);
  if (st) return st;
  const double before = h->clock_host->mass_added;
  CK(enqueue_protect(h, h->stream));
  if ((st = pull_clock(h))) return st;
  if (mass_error) *mass_error = h->clock_host->mass_added - before;
  return AGX_OK;
}

agx_status agx_distribute(agx_handle h, int32_t with_protect) {
  AGX_TRACE("agx_distribute");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_distribute(h, h->stream, with_protect != 0, true));
  return sync(h);
}

agx_status agx_update_boundary(agx_handle h, double t) {
  AGX_TRACE("agx_update_boundary");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_boundary(h, h->stream, t, false));
  return sync(h);
}

agx_status agx_compute_fluxes(agx_handle h, int32_t substep, double* flux_timestep) {
  AGX_TRACE("agx_compute_fluxes");
  if (!h || substep < 0 || substep > 2) return fail(AGX_E_INVALID, "bad arguments");
  CK(enqueue_fluxes(h, h->stream, substep));
  agx_status st = pull_clock(h);
  if (st) return st;
  Clock* c = h->clock_host;
  if (substep == 0) {
    const unsigned long long key = c->dt_key;
    double v;
    if (key) {
      long long bits = (long long)~key;
      memcpy(&v, &bits, 8);
    } else {
      v = 1.0e100;
    }
    c->flux_timestep = v;
  } else {
    c->flux_timestep = h->prm.evolve_max_timestep;
  }
  if ((st = push_clock(h))) return st;
  if (flux_timestep) *flux_timestep = c->flux_timestep;
  return AGX_OK;
}

agx_status agx_compute_forcing(agx_handle h) {
  AGX_TRACE("agx_compute_forcing");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_forcing(h, h->stream));
  return sync(h);
}

agx_status agx_update_conserved(agx_handle h, double timestep, int64_t* negative_cells) {
  AGX_TRACE("agx_update_conserved");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = pull_clock(h);
  if (st) return st;
  const long long before = h->clock_host->negative_cells;
  CK(enqueue_update(h, h->stream, -1, false, timestep));
  if ((st = pull_clock(h))) return st;
  if (negative_cells) *negative_cells = h->clock_host->negative_cells - before;
  if ((st = check_errors(h))) {
    h->clock_host->error = 0;
    push_clock(h);
    return st;
  }
  return AGX_OK;
}

agx_status agx_backup(agx_handle h) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_backup(h, h->stream));
  return sync(h);
}

agx_status agx_saxpy(agx_handle h, double a, double b) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_saxpy(h, h->stream, a, b));
  return sync(h);
}

agx_status agx_set_riverwalls(agx_handle h, const int32_t* edge_counter, int64_t n_slots, int64_t n_riverwall_edges,
                              const double* elevation, const int32_t* row_index, int32_t n_rows, int32_t ncol,
                              const double* hydraulic) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  if (n_slots != 3 * (int64_t)h->N) return fail(AGX_E_INVALID, "edge_counter has %lld slots, the mesh %lld",
                                                (long long)n_slots, 3 * (long long)h->N);
  if (n_riverwall_edges < 0 || (n_riverwall_edges > 0 && (!edge_counter || !elevation || !row_index || !hydraulic)) ||
      n_rows <= 0 || ncol < 5)
    return fail(AGX_E_INVALID, "bad riverwall tables (need 5 hydraulic columns: Qfactor s1 s2 h1 h2)");
  for (int64_t s = 0; n_riverwall_edges > 0 && s < n_slots; s++)
    if (edge_counter[s] < 0 || edge_counter[s] > n_riverwall_edges)
      return fail(AGX_E_INVALID, "riverwall counter %d at slot %lld out of range", edge_counter[s], (long long)s);
  for (int64_t r = 0; r < n_riverwall_edges; r++)
    if (row_index[r] < 0 || row_index[r] >= n_rows)
      return fail(AGX_E_INVALID, "riverwall row index %d out of range", row_index[r]);
  agx_status st = sync(h);
  if (st) return st;
  if (h->rw_mem) cudaFree(h->rw_mem);
  h->rw_mem = nullptr;
  h->d.rw_counter = nullptr;
  h->d.rw_elev = nullptr;
  h->d.rw_row = nullptr;
  h->d.rw_hyd = nullptr;
  h->d.rw_ncol = 0;
  h->graph_valid = false;
  if (n_riverwall_edges == 0) return AGX_OK;
  const size_t b_counter = ((size_t)n_slots * 4 + 255) & ~(size_t)255;
  const size_t b_elev = ((size_t)n_riverwall_edges * 8 + 255) & ~(size_t)255;
  const size_t b_row = ((size_t)n_riverwall_edges * 4 + 255) & ~(size_t)255;
  const size_t b_hyd = (size_t)n_rows * ncol * 8;
  char* m = nullptr;
  CK(cudaMalloc((void**)&m, b_counter + b_elev + b_row + b_hyd));
  h->rw_mem = m;
  CK(cudaMemcpyAsync(m, edge_counter, (size_t)n_slots * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(m + b_counter, elevation, (size_t)n_riverwall_edges * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(m + b_counter + b_elev, row_index, (size_t)n_riverwall_edges * 4, cudaMemcpyHostToDevice,
                     h->stream));
  CK(cudaMemcpyAsync(m + b_counter + b_elev + b_row, hydraulic, b_hyd, cudaMemcpyHostToDevice, h->stream));
  h->d.rw_counter = (const int*)m;
  h->d.rw_elev = (const double*)(m + b_counter);
  h->d.rw_row = (const int*)(m + b_counter + b_elev);
  h->d.rw_hyd = (const double*)(m + b_counter + b_elev + b_row);
  h->d.rw_ncol = ncol;
  return sync(h);
}

agx_status agx_divide_conserved(agx_handle h, double divisor) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  CK(enqueue_divide(h, h->stream, divisor));
  return sync(h);
}

agx_status agx_set_fixed_flux_timestep(agx_handle h, double flux_timestep) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  if (!(flux_timestep >= 0.0)) return fail(AGX_E_INVALID, "flux_timestep needs to be greater than 0.0");
  agx_status st = pull_clock(h);
  if (st) return st;
  h->clock_host->fixed_flux_dt = flux_timestep;
  return push_clock(h);
}

agx_status agx_set_clock(agx_handle h, double time, double yield_time, double final_time) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = pull_clock(h);
  if (st) return st;
  Clock* c = h->clock_host;
  c->time = time;
  c->yield_time = yield_time;
  c->final_time = final_time;
  return push_clock(h);
}

static void fill_stats(const Clock* c, agx_step_stats* o) {
  o->time = c->time;
  o->last_timestep = c->timestep;
  o->min_timestep = c->recorded_min;
  o->max_timestep = c->recorded_max;
  o->flux_timestep = c->flux_timestep;
  o->mass_added = c->mass_added;
  for (int i = 0; i < 3; i++) o->boundary_flux_sum[i] = c->bfs[i];
  o->steps = c->steps_call;
  o->total_steps = c->total_steps;
  o->negative_cells = c->negative_cells;
  o->reason = c->reason;
  o->order = c->order;
  o->boundary_flux_integral = c->bf_integral;
  o->nonfinite_cells = c->nonfinite_cells;
}

agx_status agx_set_stream(agx_handle h, void* stream) {
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = sync(h);
  if (st) return st;
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return AGX_OK;
}

agx_status agx_time_phases(agx_handle h, int32_t reps, double* ms, int32_t n_cat) {
  if (!h || !ms || reps <= 0 || n_cat < PH_COUNT) return fail(AGX_E_INVALID, "bad arguments");
  agx_status st = pull_clock(h);
  if (st) return st;
  Clock saved = *h->clock_host;
  Clock* c = h->clock_host;
  c->yield_time = 1.0e300;
  c->final_time = -1.0;
  c->steps_target = 0;
  if ((st = push_clock(h))) return st;
  for (int i = 0; i < n_cat; i++) ms[i] = 0.0;
  PhaseTimer T;
  g_timer = &T;
  cudaEvent_t start;
  cudaEventCreate(&start);
  for (int r = 0; r < reps; r++) {
    T.used = 0;
    cudaEventRecord(start, h->stream);
    cudaError_t e = enqueue_step(h, h->stream, 0ull, false);
    if (e != cudaSuccess) {
      g_timer = nullptr;
      return fail(AGX_E_CUDA, "timed step failed: %s", cudaGetErrorString(e));
    }
    CK(cudaStreamSynchronize(h->stream));
    cudaEvent_t prev = start;
    for (size_t i = 0; i < T.used; i++) {
      float t = 0.f;
      cudaEventElapsedTime(&t, prev, T.ev[i]);
      ms[T.cat[i]] += t / reps;
      prev = T.ev[i];
    }
  }
  g_timer = nullptr;
  for (auto e : T.ev) cudaEventDestroy(e);
  cudaEventDestroy(start);
  // restore the clock bookkeeping (the state itself has advanced)
  if ((st = pull_clock(h))) return st;
  c->yield_time = saved.yield_time;
  c->final_time = saved.final_time;
  c->steps_target = saved.steps_target;
  return push_clock(h);
}

agx_status agx_get_stats(agx_handle h, agx_step_stats* out) {
  if (!h || !out) return fail(AGX_E_INVALID, "bad arguments");
  agx_status st = pull_clock(h);
  if (st) return st;
  fill_stats(h->clock_host, out);
  return AGX_OK;
}

agx_status agx_advance(agx_handle h, int64_t max_steps, agx_step_stats* out) {
  AGX_TRACE("agx_advance");
  if (!h) return fail(AGX_E_INVALID, "null handle");
  agx_status st = pull_clock(h);
  if (st) return st;
  Clock* c = h->clock_host;
  c->steps_call = 0;
  c->steps_target = max_steps > 0 ? max_steps : 0;
  c->reason = 0;
  c->recorded_min = h->prm.evolve_max_timestep;
  c->recorded_max = h->prm.evolve_min_timestep;
  if ((st = push_clock(h))) return st;
  if (h->N > 0) {
    if (!h->graph_valid && (st = build_graph(h)) != AGX_OK) return st;
    CK(cudaGraphLaunch(h->exec, h->stream));
  }
  if ((st = pull_clock(h))) return st;
  g_launches += (long long)c->steps_call * h->kernels_per_step;
  if (out) fill_stats(c, out);
  if ((st = check_errors(h))) return st;
  return AGX_OK;
}

}  // extern "C"
