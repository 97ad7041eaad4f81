// agx_noalloc.cu -- agx_compute_fluxes_noalloc: the plain FP64 edge-flux and
// accumulation kernels on device arrays owned by the caller, with their
// scratch in a file-scope device array instead of an allocation.
//
// Who needs this: a caller that cannot allocate device memory at the moment
// it needs the fluxes.  A host framework whose caching allocator already holds
// the device's free memory leaves nothing for a cudaMalloc from this library,
// so the call would fail; a coupled model may have to keep its device
// footprint fixed once it has started; and a step loop with a latency budget
// cannot afford cudaMalloc/cudaFree, which synchronise the device.  Such a
// caller owns every input and output array, and this file only reads and
// writes them plus the fixed scratch below.
//
// Compiled with --fmad=false, like agx_plain.cu, and built on the same
// per-edge and per-cell functions (de_plain.cuh), so the explicit updates,
// max speeds and flux timestep equal those of agx_compute_fluxes bit for bit;
// the boundary flux sum is added with atomics across blocks and its last
// place depends on their order.
#include "agx_internal.cuh"
#include "../../include/agx_noalloc.h"
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <mutex>

namespace {

using agx::Params;
using agx::SlotResult;
using agx::CellFlux;
using agx::Riverwall;

constexpr int NA_TPB = 256;
constexpr long long NA_SLOTS = 3LL * AGX_NOALLOC_MAX_CELLS;
constexpr long long NA_STAMP = 6 * NA_SLOTS;              // u32 stamps, NA_SLOTS / 2 doubles
constexpr long long NA_TAIL = NA_STAMP + NA_SLOTS / 2;
constexpr int NA_MAX_DEVICES = 64;

// Scratch, one copy per device (a __device__ variable exists on every device
// the module is loaded on).  Layout in doubles: six slot arrays of NA_SLOTS
// values each (flux components of w, uh, vh; wave speed; pressure flux; left
// depth), then one 32-bit stamp per slot (the number of the call that last
// wrote the slot), then a tail of 32: [0] the timestep reduction key (u64
// bits), [1] the boundary flux sum, [2] u64 flags (1: a table index out of
// range, 2: a slot the edge list did not write in this call), [3] the count
// of slots written.  The tail must start at zero on every call (k_na_reset).
// The slot arrays and stamps keep the last call's contents: the stamps show
// which slots this call wrote, so they need no clearing either.
static __device__ __align__(256) double g_na_scratch[NA_TAIL + 32];

std::mutex g_na_mu;
double* g_na_ptr[NA_MAX_DEVICES] = {};
unsigned g_na_call[NA_MAX_DEVICES] = {};     // call number per device (stamps), never 0

agx_status na_fail(agx_status code, char* err, int32_t err_len, const char* fmt, ...) {
  if (err && err_len > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, (size_t)err_len, fmt, ap);
    va_end(ap);
  }
  return code;
}

// Address of the current device's scratch.  Looked up once per device, with
// that device current; later calls read the cached pointer.
agx_status na_scratch(double** out, unsigned* call, char* err, int32_t err_len) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(AGX_E_CUDA, err, err_len, "cudaGetDevice failed: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= NA_MAX_DEVICES)
    return na_fail(AGX_E_INVALID, err, err_len, "device %d is beyond the %d devices the scratch table covers", dev,
                   NA_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess || p == nullptr)
      return na_fail(AGX_E_CUDA, err, err_len, "cudaGetSymbolAddress of the flux scratch failed on device %d: %s", dev,
                     cudaGetErrorString(e));
    g_na_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_na_ptr[dev];
  if (++g_na_call[dev] == 0) g_na_call[dev] = 1;     // after 2^32 calls a stale stamp could match again
  *call = g_na_call[dev];
  return AGX_OK;
}

struct NaArgs {
  Params P;
  agx_flux_buffers b;
  int N, B, E;
  unsigned call;       // stamp of this call
};

// Neighbour indices of a cell inside the mesh or the boundary, and
// neighbour-edge numbers 0..2, so that no load leaves the caller's arrays.
__device__ __forceinline__ bool na_cell_ok(const int4& c, int N, int B) {
  const int nb[3] = {c.x, c.y, c.z};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int n = nb[i];
    if (n >= N) return false;
    if (n < 0 && -(long long)n - 1 >= B) return false;
    if (n >= 0 && agx::meta_nedge(c.w, i) > 2) return false;
  }
  return true;
}

__device__ __forceinline__ unsigned long long* na_flag(double* scr) {
  return reinterpret_cast<unsigned long long*>(scr + NA_TAIL) + 2;
}

__global__ void k_na_reset(double* scr) {
  unsigned long long* t = reinterpret_cast<unsigned long long*>(scr + NA_TAIL);
  t[0] = 0ull;   // key: no timestep yet
  t[1] = 0ull;   // boundary flux sum: +0.0
  t[2] = 0ull;   // no bad index, no slot missed
  t[3] = 0ull;   // slots written
}

__device__ __forceinline__ unsigned* na_stamps(double* scr) { return reinterpret_cast<unsigned*>(scr + NA_STAMP); }

// One thread per listed edge: the flux from the listed slot's side, and its
// exact negation for the slot on the other side (agx_plain.cu k_flux).
__global__ void k_na_flux(NaArgs a, double* scr) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.E) return;
  const int s = a.b.edge_slot[e];
  const int o = a.b.edge_opp[e];
  if (s < 0 || s >= 3 * a.N || o < -1 || o >= 3 * a.N) {
    atomicOr(na_flag(scr), 1ull);
    return;
  }
  const int k = s / 3, i = s - 3 * k;
  const int4 c = reinterpret_cast<const int4*>(a.b.conn)[k];
  if (!na_cell_ok(c, a.N, a.B)) {
    atomicOr(na_flag(scr), 1ull);
    return;
  }
  const Riverwall RW = {nullptr, nullptr, nullptr, nullptr, 0};
  SlotResult R;
  double hr;
  agx::slot_flux(a.P, k, i, c, a.b.stage_e, a.b.xmom_e, a.b.ymom_e, a.b.elev_e, a.b.height_e, a.b.stage_b,
                 a.b.xmom_b, a.b.ymom_b, a.b.normals, a.b.stage_c, a.b.height_c, a.b.elev_c, RW, R, hr);
  scr[0 * NA_SLOTS + s] = R.f[0];
  scr[1 * NA_SLOTS + s] = R.f[1];
  scr[2 * NA_SLOTS + s] = R.f[2];
  scr[3 * NA_SLOTS + s] = R.speed;
  scr[4 * NA_SLOTS + s] = R.pflux;
  scr[5 * NA_SLOTS + s] = R.hleft;
  na_stamps(scr)[s] = a.call;
  if (o >= 0) {
    scr[0 * NA_SLOTS + o] = -R.f[0];
    scr[1 * NA_SLOTS + o] = -R.f[1];
    scr[2 * NA_SLOTS + o] = -R.f[2];
    scr[3 * NA_SLOTS + o] = R.speed;
    scr[4 * NA_SLOTS + o] = R.pflux;
    scr[5 * NA_SLOTS + o] = hr;
    na_stamps(scr)[o] = a.call;
  }
  atomicAdd(reinterpret_cast<unsigned long long*>(scr + NA_TAIL) + 3, o >= 0 ? 2ull : 1ull);
}

__device__ __forceinline__ double na_warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ unsigned long long na_warp_max(unsigned long long x) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
    x = y > x ? y : x;
  }
  return x;
}

// One thread per cell: the cell's three slot results in the reference's
// accumulation order, the explicit updates, the max speed and the cell's
// timestep as a reduction key (agx_plain.cu k_accum).
__global__ void __launch_bounds__(NA_TPB) k_na_accum(NaArgs a, double* scr, int substep) {
  __shared__ unsigned long long kpart[NA_TPB / 32];
  __shared__ double bpart[NA_TPB / 32];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long key = 0ull;
  double bflux = 0.0;
  if (k < a.N) {
    const int4* conn = reinterpret_cast<const int4*>(a.b.conn);
    const int4 c = conn[k];
    const unsigned* stamp = na_stamps(scr);
    if (!na_cell_ok(c, a.N, a.B)) {
      atomicOr(na_flag(scr), 1ull);
    } else if (stamp[3LL * k] != a.call || stamp[3LL * k + 1] != a.call || stamp[3LL * k + 2] != a.call) {
      atomicOr(na_flag(scr), 2ull);       // a slot of this cell holds an earlier call's value
    } else {
      SlotResult R[3];
      int fn[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const long long s = 3LL * k + i;
        R[i].f[0] = scr[0 * NA_SLOTS + s];
        R[i].f[1] = scr[1 * NA_SLOTS + s];
        R[i].f[2] = scr[2 * NA_SLOTS + s];
        R[i].speed = scr[3 * NA_SLOTS + s];
        R[i].pflux = scr[4 * NA_SLOTS + s];
        R[i].hleft = scr[5 * NA_SLOTS + s];
        const int n = i == 0 ? c.x : i == 1 ? c.y : c.z;
        fn[i] = n >= 0 ? agx::meta_full(conn[n].w) : 1;
      }
      CellFlux F;
      agx::accum_cell(a.P, k, c, R, a.b.height_e, a.b.elev_e, a.b.height_c, a.b.elev_c, a.b.normals,
                      a.b.edgelengths, a.b.inv_area[k], fn, F);
      a.b.stage_x[k] = F.ew;
      a.b.xmom_x[k] = F.euh;
      a.b.ymom_x[k] = F.evh;
      bflux = F.bflux;
      if (substep == 0) {
        a.b.max_speed[k] = F.smax;
        if (F.smax > 0.0) {
          const double dt = agx::ddiv(a.b.radii[k] * 1.0, F.smax);
          key = ~(unsigned long long)__double_as_longlong(dt);
        }
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long* tail = reinterpret_cast<unsigned long long*>(scr + NA_TAIL);
  if (substep == 0) {
    key = na_warp_max(key);
    if (lane == 0) kpart[wid] = key;
    __syncthreads();
    if (wid == 0) {
      unsigned long long r = lane < (int)(blockDim.x >> 5) ? kpart[lane] : 0ull;
      r = na_warp_max(r);
      if (lane == 0 && r != 0ull) atomicMax(&tail[0], r);
    }
  }
  if (__syncthreads_or(bflux != 0.0)) {
    bflux = na_warp_sum(bflux);
    if (lane == 0) bpart[wid] = bflux;
    __syncthreads();
    if (wid == 0) {
      double r = lane < (int)(blockDim.x >> 5) ? bpart[lane] : 0.0;
      r = na_warp_sum(r);
      if (lane == 0) atomicAdd(scr + NA_TAIL + 1, r);
    }
  }
}

}  // namespace

extern "C" agx_status agx_compute_fluxes_noalloc(const agx_params* p, const agx_flux_buffers* b, int32_t substep,
                                                 void* stream, double* flux_timestep, double* boundary_flux_sum,
                                                 char* err, int32_t err_len) {
  if (!p || !b) return na_fail(AGX_E_INVALID, err, err_len, "null params or buffers");
  if (substep < 0 || substep > 2) return na_fail(AGX_E_INVALID, err, err_len, "substep %d is not 0, 1 or 2", substep);
  if (b->N < 1 || b->N > AGX_NOALLOC_MAX_CELLS)
    return na_fail(AGX_E_INVALID, err, err_len,
                   "N = %lld triangles is outside 1..%d, the most the no-allocation flux scratch holds "
                   "(AGX_NOALLOC_MAX_CELLS); use agx_compute_fluxes for larger meshes",
                   (long long)b->N, AGX_NOALLOC_MAX_CELLS);
  if (b->B < 0 || b->B > 3 * b->N) return na_fail(AGX_E_INVALID, err, err_len, "B = %lld out of range", (long long)b->B);
  if (b->E < 1 || b->E > 3 * b->N) return na_fail(AGX_E_INVALID, err, err_len, "E = %lld out of range", (long long)b->E);
  const void* need[] = {b->conn, b->edge_slot, b->edge_opp, b->normals, b->edgelengths, b->radii, b->inv_area,
                        b->stage_e, b->xmom_e, b->ymom_e, b->elev_e, b->height_e, b->stage_c, b->height_c,
                        b->elev_c, b->stage_x, b->xmom_x, b->ymom_x};
  for (const void* q : need)
    if (!q) return na_fail(AGX_E_INVALID, err, err_len, "a required device pointer is null");
  if (substep == 0 && !b->max_speed) return na_fail(AGX_E_INVALID, err, err_len, "max_speed is null at substep 0");
  if (b->B > 0 && (!b->stage_b || !b->xmom_b || !b->ymom_b))
    return na_fail(AGX_E_INVALID, err, err_len, "boundary value pointers are null");
  if (reinterpret_cast<uintptr_t>(b->conn) % 16 != 0)
    return na_fail(AGX_E_INVALID, err, err_len, "conn must be 16-byte aligned (read as int4 rows)");

  double* scr = nullptr;
  unsigned call = 0;
  agx_status st = na_scratch(&scr, &call, err, err_len);
  if (st != AGX_OK) return st;

  NaArgs a;
  a.b = *b;
  a.N = (int)b->N;
  a.B = (int)b->B;
  a.E = (int)b->E;
  a.call = call;
  Params& P = a.P;
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

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_na_reset<<<1, 1, 0, s>>>(scr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_na_flux<<<(a.E + NA_TPB - 1) / NA_TPB, NA_TPB, 0, s>>>(a, scr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_na_accum<<<(a.N + NA_TPB - 1) / NA_TPB, NA_TPB, 0, s>>>(a, scr, substep);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return na_fail(AGX_E_CUDA, err, err_len, "kernel launch failed: %s", cudaGetErrorString(e));
  agx::count_launch(3);
  unsigned long long tail[4] = {0ull, 0ull, 0ull, 0ull};
  e = cudaMemcpyAsync(tail, scr + NA_TAIL, sizeof(tail), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return na_fail(AGX_E_CUDA, err, err_len, "flux kernels failed: %s", cudaGetErrorString(e));
  if (tail[2] & 1ull) return na_fail(AGX_E_INVALID, err, err_len, "an edge-list or neighbour index is out of range");
  if ((tail[2] & 2ull) || tail[3] != 3ull * (unsigned long long)b->N)
    return na_fail(AGX_E_INVALID, err, err_len,
                   "the edge list writes %llu slot results, not one for each of the 3N = %lld slots",
                   tail[3], 3LL * (long long)b->N);
  double dt = p->evolve_max_timestep;
  if (substep == 0) {
    dt = 1.0e100;
    if (tail[0]) {
      const unsigned long long bits = ~tail[0];
      memcpy(&dt, &bits, 8);
    }
  }
  if (flux_timestep) *flux_timestep = dt;
  if (boundary_flux_sum) memcpy(boundary_flux_sum, &tail[1], 8);
  return AGX_OK;
}
