// agx_plain.cu -- FP64 kernels of the DE timestep (plain form, bit-exact).
//
// Compiled with --fmad=false: every floating-point operation is rounded on its
// own, as in the reference built without contraction, so results match the
// reference's FP64 path bit for bit (Manning's pow excepted: CUDA's and the C
// library's pow may differ in the last place).
//
// One timestep is a fixed sequence of kernels (DE1 = RK2 shown):
//   prep(backup) -> extrap -> bc -> flux -> accum(dt) -> timestep -> update
//   -> prep -> extrap -> bc -> flux -> accum -> update(saxpy) -> rates -> clock
// (DE2 = RK3 adds a third stage: generic_domain.py:2053-2172).
// All state stays in device memory; the clock kernel decides on the device
// whether another step is needed and sets the graph's while condition.
#include "agx_internal.cuh"
#include "inlet.cuh"
#include <cuda_runtime.h>

namespace agx {

constexpr int TPB = 256;
// resident blocks of TPB threads per SM asked of the compiler for the
// extrapolation, flux and accumulation kernels (register budgets): four
// blocks (64 registers) for the extrapolation and the flux, measured faster
// on the 4.0M-triangle DE1 step (extrapolation in class order 2.49 -> 2.39 ms,
// flux 1.757 -> 1.714 ms); the accumulation keeps its own budget
#ifndef AGX_MINB_EXTRAP
#define AGX_MINB_EXTRAP 4
#endif
#ifndef AGX_MINB_FLUX
#define AGX_MINB_FLUX 4
#endif
#ifndef AGX_MINB_ACCUM
#define AGX_MINB_ACCUM 1
#endif
// 1: the step's extrapolations visit the cells grouped by the branches each
// took in the previous extrapolation (per-cell results do not depend on the
// order in which cells are visited).  Measured on the 4.0M-triangle DE1 step:
// extrapolation 2.76 -> 2.31 ms, step 6.53 -> 6.12 ms with the sort once per
// step on the dry and wet/dry-factor classes.
#ifndef AGX_EXTRAP_ORDER
#define AGX_EXTRAP_ORDER 1
#endif
// the class bits the sort distinguishes (see k_extrap): 2 = dry cell and
// wet/dry factor below 1
#ifndef AGX_CLASS_BITS
#define AGX_CLASS_BITS 2
#endif
// 1: the cells are sorted after every extrapolation of a step; 2: only after
// its last (the step's stages visit the cells in one order)
#ifndef AGX_SORT_CADENCE
#define AGX_SORT_CADENCE 2
#endif
static const double kNaN = __builtin_nan("");

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long x) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
    x = y > x ? y : x;
  }
  return x;
}

// Block-wide sum, result valid in thread 0.
__device__ double block_sum(double x) {
  __shared__ double part[TPB / 32];
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = x;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

__device__ unsigned long long block_max_u64(unsigned long long x) {
  __shared__ unsigned long long part[TPB / 32];
  x = warp_max_u64(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = x;
  __syncthreads();
  unsigned long long r = 0;
  if (wid == 0) {
    r = lane < (int)(blockDim.x >> 5) ? part[lane] : 0ull;
    r = warp_max_u64(r);
  }
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// mode bit 0: backup, bit 1: skip protect, bit 2: protect only
__global__ void k_prep(Dev d, int mode) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double added = 0.0;
  if (k < d.N) {
    if (mode & 1) {
      d.w0[k] = d.w[k];
      d.uh0[k] = d.uh[k];
      d.vh0[k] = d.vh[k];
    }
    added = prep_cell(d.P, k, d.w, d.uh, d.vh, d.z, d.areas, d.h, d.u, d.v, (mode & 2) == 0,
                      (mode & 4) == 0);
  }
  const int any = __syncthreads_or(added != 0.0);
  if (any) {
    const double s = block_sum(added);
    if (threadIdx.x == 0) atomicAdd(&d.clock->mass_added, s);
  }
}

// ORD: thread i takes cell order[i] and records the cell's branch class
template <bool VERT, bool ORD = false>
__global__ void __launch_bounds__(TPB, AGX_MINB_EXTRAP) k_extrap(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.N) return;
  const int k = ORD ? d.order[i] : i;
  EdgeOut E;
  int cls = 0;
  const bool sdry = extrap_cell(d.P, k, d.conn, d.surr, d.geo, d.w, d.h, d.u, d.v, E, ORD ? &cls : nullptr);
  if (ORD) {
    // the classes the sort distinguishes: all eight bits, or the four
    // limiter bits merged into one (5), or none of them (4), or only the
    // dry and wet/dry-factor bits (2), or only the dry bit (1).  Measured
    // extrapolation per 4.0M-triangle DE1 step: 2.38, 2.39, 2.31, 2.31,
    // 2.73 ms (2.76 unsorted): what pays is keeping the cells of the wet/dry
    // fronts (factor below 1: the divided-out factor, mixed betas, limiter
    // products) out of the warps of the rest; finer classes only cut the
    // cells' runs shorter.
    if (AGX_CLASS_BITS == 5) cls = (cls & 15) | ((cls & 240) ? 16 : 0);
    if (AGX_CLASS_BITS == 4) cls &= 15;
    if (AGX_CLASS_BITS == 2) cls &= 12;
    if (AGX_CLASS_BITS == 1) cls &= 4;
    d.cls[k] = (unsigned char)cls;
  }
  const size_t b = 3 * (size_t)k;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    d.we[b + i] = E.w[i];
    d.he[b + i] = E.h[i];
    d.uhe[b + i] = E.uh[i];
    d.vhe[b + i] = E.vh[i];
    d.ze[b + i] = E.z[i];
  }
  if (sdry) {
    d.uh[k] = 0.0;
    d.vh[k] = 0.0;
  }
  if (!VERT && d.P.sloped_mannings) {
    double vx[3];
    vertex_from_edges(E.z, vx);   // sloped friction reads the bed vertex values
    for (int i = 0; i < 3; i++) d.zv[b + i] = vx[i];
  }
  if (VERT) {
    double vx[3];
    vertex_from_edges(E.w, vx);
    for (int i = 0; i < 3; i++) d.wv[b + i] = vx[i];
    vertex_from_edges(E.h, vx);
    for (int i = 0; i < 3; i++) d.hv[b + i] = vx[i];
    vertex_from_edges(E.uh, vx);
    for (int i = 0; i < 3; i++) d.uhv[b + i] = vx[i];
    vertex_from_edges(E.vh, vx);
    for (int i = 0; i < 3; i++) d.vhv[b + i] = vx[i];
    vertex_from_edges(E.z, vx);
    for (int i = 0; i < 3; i++) d.zv[b + i] = vx[i];
  }
}

__global__ void k_order_init(Dev d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < d.N) d.order[k] = k;
}

// Counting sort of the cells by branch class: counts, exclusive offsets,
// scatter.  Each block takes SORT_SPAN consecutive cells and tallies them in
// shared memory (lanes of a warp with the same class with one shared
// atomic), so the global counters see one atomic per class and block; within
// a warp cells of one class keep their order.
constexpr int SORT_SPAN = 16 * TPB;
static_assert(TPB == 256, "the class sort keeps one shared counter per thread and class");

// The lanes of `active` with the same class as this lane (most warps hold
// one class: checked with a vote before the general match).
__device__ __forceinline__ unsigned class_peers(unsigned active, int c) {
  const int c0 = __shfl_sync(active, c, __ffs(active) - 1);
  if (__all_sync(active, c == c0)) return active;
  return __match_any_sync(active, c);
}

// every lane of a warp runs the same iterations (warp collectives inside)
__device__ __forceinline__ void cls_tally(const Dev& d, int k0, unsigned* hist) {
  for (int j = 0; j < SORT_SPAN; j += TPB) {
    const int k = k0 + j + threadIdx.x;
    const bool in = k < d.N;
    const unsigned active = __ballot_sync(0xffffffffu, in);
    if (in) {
      const int c = d.cls[k];
      const unsigned peers = class_peers(active, c);
      if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[c], (unsigned)__popc(peers));
    }
  }
}

__global__ void __launch_bounds__(TPB) k_cls_count(Dev d) {
  __shared__ unsigned hist[256];
  hist[threadIdx.x] = 0u;
  __syncthreads();
  cls_tally(d, blockIdx.x * SORT_SPAN, hist);
  __syncthreads();
  const unsigned n = hist[threadIdx.x];
  if (n) atomicAdd(&d.cls_count[threadIdx.x], n);
}

__global__ void k_cls_offsets(Dev d) {      // one block of 256 threads
  __shared__ unsigned s[256];
  const int t = threadIdx.x;
  const unsigned v = d.cls_count[t];
  s[t] = v;
  __syncthreads();
  for (int off = 1; off < 256; off <<= 1) {
    const unsigned x = t >= off ? s[t - off] : 0u;
    __syncthreads();
    s[t] += x;
    __syncthreads();
  }
  d.cls_count[256 + t] = s[t] - v;     // first position of class t
  d.cls_count[t] = 0u;                 // counts start from zero next time
}

__global__ void __launch_bounds__(TPB) k_cls_scatter(Dev d) {
  __shared__ unsigned hist[256];
  const int k0 = blockIdx.x * SORT_SPAN;
  hist[threadIdx.x] = 0u;
  __syncthreads();
  cls_tally(d, k0, hist);
  __syncthreads();
  // this block's run of each class, then positions inside the runs
  const unsigned n = hist[threadIdx.x];
  hist[threadIdx.x] = n ? atomicAdd(&d.cls_count[256 + threadIdx.x], n) : 0u;
  __syncthreads();
  for (int j = 0; j < SORT_SPAN; j += TPB) {
    const int k = k0 + j + threadIdx.x;
    const bool in = k < d.N;
    const unsigned active = __ballot_sync(0xffffffffu, in);
    if (in) {
      const int c = d.cls[k];
      const unsigned peers = class_peers(active, c);
      const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
      unsigned base = 0u;
      if (lane == leader) base = atomicAdd(&hist[c], (unsigned)__popc(peers));
      base = __shfl_sync(peers, base, leader);
      const unsigned pos = base + (unsigned)__popc(peers & ((1u << lane) - 1u));
      if (pos < (unsigned)d.N) d.order[pos] = k;
    }
  }
}

__device__ void series_value(const double* rows, int n, double t, double out[3]) {
  if (n <= 0) { out[0] = out[1] = out[2] = 0.0; return; }
  if (t <= rows[0]) { out[0] = rows[1]; out[1] = rows[2]; out[2] = rows[3]; return; }
  if (t >= rows[4 * (n - 1)]) {
    const double* r = rows + 4 * (n - 1);
    out[0] = r[1]; out[1] = r[2]; out[2] = r[3];
    return;
  }
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (rows[4 * mid] <= t) lo = mid; else hi = mid;
  }
  const double* a = rows + 4 * lo;
  const double* c = rows + 4 * hi;
  const double ratio = (t - a[0]) / (c[0] - a[0]);
  for (int q = 0; q < 3; q++) out[q] = a[1 + q] + ratio * (c[1 + q] - a[1 + q]);
}

// Boundary values; a time series is read at t_override, or (NaN) at the
// clock's time + frac * timestep (the stage's time: frac 0, 1 or 0.5).
__global__ void k_bc(Dev d, double t_override, double frac) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= d.B) return;
  const int kind = d.bkind[m];
  if (kind == BK_NONE) return;
  const int s = d.bslot[m];
  const int k = s / 3;
  double tv[3];
  const double* val = d.bval + 3 * (size_t)m;
  if (kind == BK_TIME_SERIES) {
    double t = t_override;
    if (t != t) t = d.clock->time + frac * d.clock->timestep;  // NaN: use the clock
    series_value(d.bseries, d.nseries, t, tv);
    val = tv;
  }
  double wb, uhb, vhb;
  boundary_value(kind, d.normals[2 * s], d.normals[2 * s + 1], d.we[s], d.uhe[s], d.vhe[s], d.ze[s], d.w[k],
                 d.uh[k], d.vh[k], d.z[k], d.P.g, val, wb, uhb, vhb);
  d.wb[m] = wb;
  d.uhb[m] = uhb;
  d.vhb[m] = vhb;
}

__global__ void __launch_bounds__(TPB, AGX_MINB_FLUX) k_flux(Dev d) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.E) return;
  const int s = d.edge_slot[e];
  const int k = s / 3, i = s - 3 * k;
  const Riverwall RW = {d.rw_counter, d.rw_elev, d.rw_row, d.rw_hyd, d.rw_ncol};
  SlotResult R;
  double hr;
  slot_flux(d.P, k, i, d.conn[k], d.we, d.uhe, d.vhe, d.ze, d.he, d.wb, d.uhb, d.vhb, d.normals, d.w,
            d.h, d.z, RW, R, hr);
  d.sl0[s] = R.f[0];
  d.sl1[s] = R.f[1];
  d.sl2[s] = R.f[2];
  d.slsp[s] = R.speed;
  d.slpf[s] = R.pflux;
  d.slhl[s] = R.hleft;
  const int o = d.edge_opp[e];
  if (o >= 0) {
    d.sl0[o] = -R.f[0];
    d.sl1[o] = -R.f[1];
    d.sl2[o] = -R.f[2];
    d.slsp[o] = R.speed;
    d.slpf[o] = R.pflux;
    d.slhl[o] = hr;
  }
}

__global__ void __launch_bounds__(TPB, AGX_MINB_ACCUM) k_accum(Dev d, int substep) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long key = 0ull;
  double bflux = 0.0;
  if (k < d.N) {
    const int4 c = d.conn[k];
    SlotResult R[3];
    int fn[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const size_t s = 3 * (size_t)k + i;
      R[i].f[0] = d.sl0[s];
      R[i].f[1] = d.sl1[s];
      R[i].f[2] = d.sl2[s];
      R[i].speed = d.slsp[s];
      R[i].pflux = d.slpf[s];
      R[i].hleft = d.slhl[s];
      const int n = i == 0 ? c.x : i == 1 ? c.y : c.z;
      fn[i] = n >= 0 ? meta_full(d.conn[n].w) : 1;
    }
    // A dry cell whose three slots carry a zero flux, no speed, a +0 pressure
    // flux and zero depths on both sides: every term of accum_cell is then
    // a zero, its sums and the pressure terms come out +0 (the pressure
    // bracket is +0 - +0 - (+0 * dz) = +0 whatever the sign of dz), so the
    // FP64 arithmetic is skipped with the same bits.
    bool dry = !dnz(d.h[k]);
#pragma unroll
    for (int i = 0; i < 3; i++)
      dry = dry && !dnz(R[i].f[0]) && !dnz(R[i].f[1]) && !dnz(R[i].f[2]) && dbits(R[i].pflux) == 0 &&
            !dnz(R[i].hleft) && !dnz(d.he[3 * (size_t)k + i]) && !dgt(R[i].speed, d.P.epsilon);
    CellFlux F;
    if (dry) {
      F.ew = F.euh = F.evh = 0.0 * d.inv_area[k];     // +0 * (1/area), as the sums' scaling
      F.smax = 0.0;
      F.bflux = 0.0;
    } else {
      accum_cell(d.P, k, c, R, d.he, d.ze, d.h, d.z, d.normals, d.lengths, d.inv_area[k], fn, F);
    }
    d.xw[k] = F.ew;
    d.xuh[k] = F.euh;
    d.xvh[k] = F.evh;
    bflux = F.bflux;
    if (substep == 0) {
      d.max_speed[k] = F.smax;
      if (F.smax > 0.0) {
        const double dt = ddiv(d.radii[k] * 1.0, F.smax);
        key = ~(unsigned long long)__double_as_longlong(dt);
      }
    }
  }
  if (substep == 0) {
    const unsigned long long bk = block_max_u64(key);
    if (threadIdx.x == 0 && bk != 0ull) atomicMax(&d.clock->dt_key, bk);
  }
  const int any = __syncthreads_or(bflux != 0.0);
  if (any) {
    const double bs = block_sum(bflux);
    if (threadIdx.x == 0) atomicAdd(&d.clock->bfs_acc, bs);
  }
}

__global__ void k_timestep(Dev d, int substep_count) {
  (void)substep_count;
  d.clock->bfs[0] = d.clock->bfs_acc;
  timestep_logic(d.clock);
}

// saxpy: 0 none; 1 RK2 combine 0.5 Q + 0.5 Q0; 2 RK3 second stage
// 0.25 Q + 0.75 Q0; 3 RK3 last stage (2 Q + Q0) / 3 (generic_domain.py:2126, 2160-2166).
__global__ void k_update(Dev d, int stage, int use_clock_dt, double dt_arg, int saxpy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int bad = 0, neg = 0, nf = 0;
  if (k < d.N) {
    const double dt = use_clock_dt ? d.clock->timestep : dt_arg;
    double w = d.w[k], uh = d.uh[k], vh = d.vh[k];
    const double z = d.z[k];
    double sw = d.sw[k], suh = d.suh[k], svh = d.svh[k];
    if (stage >= 0) {   // forcing terms: manning_friction_implicit
      double S;
      if (d.P.sloped_mannings) S = manning_S_sloped(d.P, w, d.zv + 3 * (size_t)k, d.vcoord + 6 * (size_t)k, uh, vh, d.eta[k]);
      else S = manning_S(d.P, w, z, uh, vh, d.eta[k]);
      suh += S * uh;
      svh += S * vh;
    }
    if (!update_quantity(w, d.xw[k], sw, dt)) bad = 1;
    if (!update_quantity(uh, d.xuh[k], suh, dt)) bad = 1;
    if (!update_quantity(vh, d.xvh[k], svh, dt)) bad = 1;
    if ((dkey(w - z) < -1) & (meta_full(d.conn[k].w) > 0)) {     // w - z < 0
      neg = 1;
      w = z;
      uh = 0.0;
      vh = 0.0;
    }
    if (saxpy) {
      const double a = saxpy == 2 ? 0.25 : (saxpy == 3 ? 2.0 : 0.5);
      const double b = saxpy == 2 ? 0.75 : (saxpy == 3 ? 1.0 : 0.5);
      w = a * w + b * d.w0[k];
      uh = a * uh + b * d.uh0[k];
      vh = a * vh + b * d.vh0[k];
      if (saxpy == 3) {
        w = ddiv(w, 3.0);
        uh = ddiv(uh, 3.0);
        vh = ddiv(vh, 3.0);
      }
    }
    d.w[k] = w;
    d.uh[k] = uh;
    d.vh[k] = vh;
    d.sw[k] = sw;
    d.suh[k] = suh;
    d.svh[k] = svh;
    // a NaN or an infinity in the conserved state stops the step loop (the
    // CFL minimum would otherwise skip the cell and let it spread)
    nf = nonfinite64(w) | nonfinite64(uh) | nonfinite64(vh);
  }
  const int anyneg = __syncthreads_count(neg);
  const int anybad = __syncthreads_or(bad);
  const int nnf = __syncthreads_count(nf);
  if (threadIdx.x == 0) {
    if (anyneg) atomicAdd((unsigned long long*)&d.clock->negative_cells, (unsigned long long)anyneg);
    if (anybad) atomicOr(&d.clock->error, (int)ERR_NUMERIC);
    if (nnf) {
      atomicAdd((unsigned long long*)&d.clock->nonfinite_cells, (unsigned long long)nnf);
      atomicOr(&d.clock->error, (int)ERR_NONFINITE);
    }
  }
}

// Forcing only (per-phase API): accumulate Manning into semi_implicit_update.
__global__ void k_forcing(Dev d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  const double w = d.w[k], uh = d.uh[k], vh = d.vh[k];
  double S;
  if (d.P.sloped_mannings) S = manning_S_sloped(d.P, w, d.zv + 3 * (size_t)k, d.vcoord + 6 * (size_t)k, uh, vh, d.eta[k]);
  else S = manning_S(d.P, w, d.z[k], uh, vh, d.eta[k]);
  d.suh[k] += S * uh;
  d.svh[k] += S * vh;
}

__global__ void k_backup(Dev d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  d.w0[k] = d.w[k];
  d.uh0[k] = d.uh[k];
  d.vh0[k] = d.vh[k];
}

// Conserved centroid values divided by `divisor` (the last RK3 stage's
// Q / 3.0, generic_domain.py:2163-2166).
__global__ void k_divide(Dev d, double divisor) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  d.w[k] = ddiv(d.w[k], divisor);
  d.uh[k] = ddiv(d.uh[k], divisor);
  d.vh[k] = ddiv(d.vh[k], divisor);
}

__global__ void k_saxpy(Dev d, double a, double b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  d.w[k] = a * d.w[k] + b * d.w0[k];
  d.uh[k] = a * d.uh[k] + b * d.uh0[k];
  d.vh[k] = a * d.vh[k] + b * d.vh0[k];
}

// Rate_operator with a constant non-negative or negative rate.
// dt_arg < 0: the step's timestep from the device clock (the step loop);
// otherwise the timestep the host gives (operators applied from the host).
__global__ void k_rate(Dev d, const int* idx, int n, double rate, double factor, int op, double dt_arg) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double influx = 0.0;
  if (j < n) {
    const int k = idx ? idx[j] : j;
    const double dt = dt_arg >= 0.0 ? dt_arg : d.clock->timestep;
    if (rate >= 0.0) {
      const double local = factor * dt * rate;
      d.w[k] = d.w[k] + local;
      influx = local * d.areas[k];
    } else {
      const double height = d.w[k] - d.z[k];
      const double local = fmax(factor * dt * rate, -height);
      const double f = local < 0.0 ? (local + height) / (height + 1.0e-10) : 1.0;
      d.w[k] = d.w[k] + local;
      d.uh[k] = d.uh[k] * f;
      d.vh[k] = d.vh[k] * f;
      influx = local * d.areas[k];
    }
  }
  const int any = __syncthreads_or(influx != 0.0);
  if (any) {
    const double s = block_sum(influx);
    if (threadIdx.x == 0 && op < MAX_OPS) atomicAdd(&d.clock->op_influx[op], s);
  }
}

// Inlet_operator (structures/inlet_operator.py:75-165, inlet.py:107-226) on
// the scenario's stage-stored state; the steps are in inlet.cuh.  The
// discharge is Q = 0.5 (q1 + q2) over the timestep (dt_arg < 0: the step's
// timestep from the clock).
struct PlainInletCells {
  Dev d;
  __device__ int cell(int a) const { return d_idx[a]; }
  __device__ double stage(int k) const { return d.w[k]; }
  __device__ double height(int k) const { return d.w[k] - d.z[k]; }
  __device__ double area(int k) const { return d.areas[k]; }
  __device__ double uh(int k) const { return d.uh[k]; }
  __device__ double vh(int k) const { return d.vh[k]; }
  __device__ void set_level(int k, double level) { d.w[k] = level; }
  __device__ void set_depth(int k, double depth) { d.w[k] = d.z[k] + depth; }
  __device__ void empty(int k) {
    d.w[k] = d.z[k];
    d.uh[k] = 0.0;
    d.vh[k] = 0.0;
  }
  __device__ void set_momenta(int k, double mx, double my) {
    d.uh[k] = mx;
    d.vh[k] = my;
  }
  const int* d_idx;
};

__global__ void __launch_bounds__(INLET_TPB) k_inlet(Dev d, RateOp op, int slot, double q1, double q2, double dt_arg) {
  const double dt = dt_arg >= 0.0 ? dt_arg : d.clock->timestep;
  const double volume = 0.5 * (q1 + q2) * dt;
  PlainInletCells c{d, op.idx};
  const double applied = inlet_apply(c, op.n, op.flags, op.vu, op.vv, op.area, volume);
  if (threadIdx.x == 0 && slot < MAX_OPS) d.clock->op_influx[slot] += applied;
}

// One sww frame (file/sww.py:352-410 store_timestep, smoothed node values):
// per node the mean over its vertex slots in the order the caller gives (the
// reference's vertex_value_indices, summed and divided as quantity.c:823-915
// do, total / k) of the centroid values of the slots' triangles
// (centroid_avg: the DE algorithms' centroid averaging,
// shallow_water_domain.py:596) or of the slots' vertex values; a node is
// storable when its mean stage minus its mean bed is at least
// minimum_storable_height: otherwise the stage stored is the bed and the
// momenta are zero.  Centroid values are stored as they are.  All as float.
__global__ void k_sww_nodes(Dev d, int P, const int* off, const int* slot, double msh, int centroid_avg, float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double aw = 0.0, az = 0.0, au = 0.0, av = 0.0;
  const int a = off[p], b = off[p + 1];
  for (int q = a; q < b; q++) {
    const int s = slot[q];
    if (centroid_avg) {
      const int k = s / 3;
      aw += d.w[k];
      az += d.z[k];
      au += d.uh[k];
      av += d.vh[k];
    } else {
      aw += d.wv[s];
      az += d.zv[s];
      au += d.uhv[s];
      av += d.vhv[s];
    }
  }
  if (b > a) {
    const double k = (double)(b - a);
    aw = aw / k;
    az = az / k;
    au = au / k;
    av = av / k;
  }
  const bool storable = aw - az >= msh;
  out[p] = (float)(storable ? aw : az);
  out[P + p] = storable ? (float)au : 0.0f;
  out[2 * P + p] = storable ? (float)av : 0.0f;
}

__global__ void k_sww_cells(Dev d, float* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.N) return;
  out[k] = (float)d.w[k];
  out[d.N + k] = (float)d.uh[k];
  out[2 * d.N + k] = (float)d.vh[k];
}


__global__ void k_clock(Dev d, double t0_unused, cudaGraphConditionalHandle handle, int set_cond) {
  (void)t0_unused;
  const int reason = clock_logic(d.clock);
  if (set_cond) cudaGraphSetConditional(handle, reason == 0 ? 1u : 0u);
}

// Stage bookkeeping inside an RK2 step: time at stage 2 (set_relative_time).
__global__ void k_reset_accum(Dev d) {
  d.clock->dt_key = 0ull;
  d.clock->bfs_acc = 0.0;
}

__global__ void k_store_bfs(Dev d, int substep) {
  d.clock->bfs[substep] = d.clock->bfs_acc;
  d.clock->bfs_acc = 0.0;
}

// ---------------------------------------------------------------------------
static inline int nblk(int n) { return (n + TPB - 1) / TPB; }

#define LAUNCHK(cat, ...)                  \
  do {                                     \
    __VA_ARGS__;                           \
    count_launch();                        \
    cudaError_t _e = cudaGetLastError();   \
    if (_e != cudaSuccess) return _e;      \
    phase_mark(st, cat);                   \
  } while (0)
#define LAUNCH(...) LAUNCHK(PH_SMALL, __VA_ARGS__)

cudaError_t enqueue_reset_accum(Scenario* s, cudaStream_t st) {
  LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(s->d));
  return cudaSuccess;
}

cudaError_t enqueue_distribute(Scenario* s, cudaStream_t st, bool with_protect, bool vertices) {
  const Dev& d = s->d;
  if (d.N == 0) return cudaSuccess;
  LAUNCHK(PH_PREP, k_prep<<<nblk(d.N), TPB, 0, st>>>(d, with_protect ? 0 : 2));
  if (vertices) LAUNCHK(PH_EXTRAP, k_extrap<true><<<nblk(d.N), TPB, 0, st>>>(d));
  else LAUNCHK(PH_EXTRAP, k_extrap<false><<<nblk(d.N), TPB, 0, st>>>(d));
  return cudaSuccess;
}

cudaError_t enqueue_protect(Scenario* s, cudaStream_t st) {
  if (s->d.N == 0) return cudaSuccess;
  LAUNCHK(PH_PREP, k_prep<<<nblk(s->d.N), TPB, 0, st>>>(s->d, 4));
  return cudaSuccess;
}

cudaError_t enqueue_boundary(Scenario* s, cudaStream_t st, double t_override, bool stage2) {
  const Dev& d = s->d;
  if (d.B == 0) return cudaSuccess;
  LAUNCHK(PH_BC, k_bc<<<nblk(d.B), TPB, 0, st>>>(d, t_override, stage2 ? 1.0 : 0.0));
  return cudaSuccess;
}

cudaError_t enqueue_fluxes(Scenario* s, cudaStream_t st, int substep) {
  const Dev& d = s->d;
  if (d.N == 0) return cudaSuccess;
  LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(d));
  LAUNCHK(PH_FLUX, k_flux<<<nblk(d.E), TPB, 0, st>>>(d));
  LAUNCHK(PH_ACCUM, k_accum<<<nblk(d.N), TPB, 0, st>>>(d, substep));
  LAUNCH(k_store_bfs<<<1, 1, 0, st>>>(d, substep));
  return cudaSuccess;
}

cudaError_t enqueue_forcing(Scenario* s, cudaStream_t st) {
  const Dev& d = s->d;
  if (d.N == 0) return cudaSuccess;
  LAUNCHK(PH_UPDATE, k_forcing<<<nblk(d.N), TPB, 0, st>>>(d));
  return cudaSuccess;
}

cudaError_t enqueue_update(Scenario* s, cudaStream_t st, int stage, bool use_clock_dt, double dt) {
  const Dev& d = s->d;
  if (d.N == 0) return cudaSuccess;
  // stage < 0: forcing already accumulated (per-phase API)
  LAUNCHK(PH_UPDATE, k_update<<<nblk(d.N), TPB, 0, st>>>(d, stage, use_clock_dt ? 1 : 0, dt, 0));
  return cudaSuccess;
}

cudaError_t enqueue_backup(Scenario* s, cudaStream_t st) {
  if (s->d.N == 0) return cudaSuccess;
  LAUNCH(k_backup<<<nblk(s->d.N), TPB, 0, st>>>(s->d));
  return cudaSuccess;
}

cudaError_t enqueue_divide(Scenario* s, cudaStream_t st, double divisor) {
  if (s->d.N == 0) return cudaSuccess;
  LAUNCH(k_divide<<<nblk(s->d.N), TPB, 0, st>>>(s->d, divisor));
  return cudaSuccess;
}

cudaError_t enqueue_saxpy(Scenario* s, cudaStream_t st, double a, double b) {
  if (s->d.N == 0) return cudaSuccess;
  LAUNCH(k_saxpy<<<nblk(s->d.N), TPB, 0, st>>>(s->d, a, b));
  return cudaSuccess;
}

// One full timestep (Euler, RK2 or RK3), ending with the clock kernel.
cudaError_t enqueue_order_init(Scenario* s, cudaStream_t st) {
  if (s->d.N == 0) return cudaSuccess;
  LAUNCH(k_order_init<<<nblk(s->d.N), TPB, 0, st>>>(s->d));
  return cudaSuccess;
}

// The step's extrapolation; with AGX_EXTRAP_ORDER it visits the cells in the
// order of the previous one's classes and sorts them by this one's.
static cudaError_t enqueue_step_extrap(const Dev& d, cudaStream_t st, bool last) {
  const int nb = nblk(d.N);
  if (AGX_EXTRAP_ORDER) {
    const int sb = (d.N + SORT_SPAN - 1) / SORT_SPAN;
    LAUNCHK(PH_EXTRAP, k_extrap<false, true><<<nb, TPB, 0, st>>>(d));
    if (last || AGX_SORT_CADENCE == 1) {
      LAUNCH(k_cls_count<<<sb, TPB, 0, st>>>(d));
      LAUNCH(k_cls_offsets<<<1, 256, 0, st>>>(d));
      LAUNCH(k_cls_scatter<<<sb, TPB, 0, st>>>(d));
    }
  } else {
    LAUNCHK(PH_EXTRAP, k_extrap<false><<<nb, TPB, 0, st>>>(d));
  }
  return cudaSuccess;
}

cudaError_t enqueue_step(Scenario* s, cudaStream_t st, unsigned long long cond_handle, bool set_cond) {
  const Dev& d = s->d;
  const int nb = nblk(d.N), eb = nblk(d.E), bb = nblk(d.B);
  const bool rk2 = s->prm.timestepping_method == 2;
  const bool rk3 = s->prm.timestepping_method == 3;
  // stage 1
  LAUNCHK(PH_PREP, k_prep<<<nb, TPB, 0, st>>>(d, (rk2 || rk3) ? 1 : 0));
  if (cudaError_t e = enqueue_step_extrap(d, st, !(rk2 || rk3))) return e;
  if (d.B) LAUNCHK(PH_BC, k_bc<<<bb, TPB, 0, st>>>(d, kNaN, 0.0));
  LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(d));
  LAUNCHK(PH_FLUX, k_flux<<<eb, TPB, 0, st>>>(d));
  LAUNCHK(PH_ACCUM, k_accum<<<nb, TPB, 0, st>>>(d, 0));
  LAUNCH(k_timestep<<<1, 1, 0, st>>>(d, 0));
  LAUNCHK(PH_UPDATE, k_update<<<nb, TPB, 0, st>>>(d, 1, 1, 0.0, 0));
  if (rk2) {
    LAUNCHK(PH_PREP, k_prep<<<nb, TPB, 0, st>>>(d, 0));
    if (cudaError_t e = enqueue_step_extrap(d, st, true)) return e;
    if (d.B) LAUNCHK(PH_BC, k_bc<<<bb, TPB, 0, st>>>(d, kNaN, 1.0));
    LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(d));
    LAUNCHK(PH_FLUX, k_flux<<<eb, TPB, 0, st>>>(d));
    LAUNCHK(PH_ACCUM, k_accum<<<nb, TPB, 0, st>>>(d, 1));
    LAUNCH(k_store_bfs<<<1, 1, 0, st>>>(d, 1));
    LAUNCHK(PH_UPDATE, k_update<<<nb, TPB, 0, st>>>(d, 2, 1, 0.0, 1));
  }
  if (rk3) {
    // second stage at t + dt, combined to 0.25 Q + 0.75 Q0
    LAUNCHK(PH_PREP, k_prep<<<nb, TPB, 0, st>>>(d, 0));
    if (cudaError_t e = enqueue_step_extrap(d, st, false)) return e;
    if (d.B) LAUNCHK(PH_BC, k_bc<<<bb, TPB, 0, st>>>(d, kNaN, 1.0));
    LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(d));
    LAUNCHK(PH_FLUX, k_flux<<<eb, TPB, 0, st>>>(d));
    LAUNCHK(PH_ACCUM, k_accum<<<nb, TPB, 0, st>>>(d, 1));
    LAUNCH(k_store_bfs<<<1, 1, 0, st>>>(d, 1));
    LAUNCHK(PH_UPDATE, k_update<<<nb, TPB, 0, st>>>(d, 2, 1, 0.0, 2));
    // third stage at t + dt/2, combined to (2 Q + Q0) / 3
    LAUNCHK(PH_PREP, k_prep<<<nb, TPB, 0, st>>>(d, 0));
    if (cudaError_t e = enqueue_step_extrap(d, st, true)) return e;
    if (d.B) LAUNCHK(PH_BC, k_bc<<<bb, TPB, 0, st>>>(d, kNaN, 0.5));
    LAUNCH(k_reset_accum<<<1, 1, 0, st>>>(d));
    LAUNCHK(PH_FLUX, k_flux<<<eb, TPB, 0, st>>>(d));
    LAUNCHK(PH_ACCUM, k_accum<<<nb, TPB, 0, st>>>(d, 2));
    LAUNCH(k_store_bfs<<<1, 1, 0, st>>>(d, 2));
    LAUNCHK(PH_UPDATE, k_update<<<nb, TPB, 0, st>>>(d, 3, 1, 0.0, 3));
  }
  for (size_t i = 0; i < s->ops.size(); i++) {
    const RateOp& op = s->ops[i];
    if (op.kind == 1) {
      LAUNCHK(PH_RATE, k_inlet<<<1, INLET_TPB, 0, st>>>(d, op, (int)i, op.rate, op.rate, -1.0));
    } else {
      LAUNCHK(PH_RATE, k_rate<<<nblk(op.n), TPB, 0, st>>>(d, op.idx, op.n, op.rate, op.factor, (int)i, -1.0));
    }
  }
  LAUNCH(k_clock<<<1, 1, 0, st>>>(d, 0.0, (cudaGraphConditionalHandle)cond_handle, set_cond ? 1 : 0));
  return cudaSuccess;
}

cudaError_t enqueue_rate_once(Scenario* s, cudaStream_t st, int i, double rate, double factor, double dt) {
  const Dev& d = s->d;
  const RateOp& op = s->ops[i];
  if (op.n == 0) return cudaSuccess;
  if (op.kind == 1) {
    LAUNCHK(PH_RATE, k_inlet<<<1, INLET_TPB, 0, st>>>(d, op, i, rate, factor, dt));
  } else {
    LAUNCHK(PH_RATE, k_rate<<<nblk(op.n), TPB, 0, st>>>(d, op.idx, op.n, rate, factor, i, dt));
  }
  return cudaSuccess;
}

cudaError_t enqueue_sww_frame(Scenario* s, cudaStream_t st, double msh, int centroid_avg) {
  const Dev& d = s->d;
  if (s->P > 0)
    LAUNCH(k_sww_nodes<<<nblk(s->P), TPB, 0, st>>>(d, s->P, s->node_off, s->node_slot, msh, centroid_avg, s->frame));
  if (d.N > 0) LAUNCH(k_sww_cells<<<nblk(d.N), TPB, 0, st>>>(d, s->frame + 3 * (size_t)s->P));
  return cudaSuccess;
}

}  // namespace agx
