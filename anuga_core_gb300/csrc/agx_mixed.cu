// agx_mixed.cu -- mixed-precision DE step over a pool of scenarios.
//
// A pool is one device arena holding many scenarios (meshes of any size).
// Cells are stored scenario by scenario in space-filling-curve order and
// grouped into tiles of TILE cells; a tile belongs to one scenario.  Every
// kernel is persistent (a grid sized to the GPU) and walks the tile table,
// so one launch advances every active scenario, each with its own timestep,
// clock and boundary conditions.  A single mixed-precision domain is a pool
// with one scenario; the batched and serving forms use the same kernels.
//
// Per DE1 (RK2) step:
//   flux1  : FP32 reconstruction + edge fluxes + accumulation, per-scenario
//            CFL minimum (reduced as FP64 keys)
//   dt     : update_timestep per scenario (FP64)
//   update1: FP64 accumulation q1 = protect(q0) + dt E, Manning, fix_negative,
//            and the FP32 work record for stage 2
//   flux2  : stage-2 fluxes fused with the update, fix_negative, the RK2
//            combine 0.5 q0 + 0.5 q2 and the work record of the next step
//   rates  : Rate_operator stage changes
//   clock  : per-scenario time bookkeeping; sets the graph's while condition
// The conserved state is kept as (depth h = w - z, uh, vh) in FP64, so the
// depth at wet/dry fronts needs no subtraction in the step; the stage w
// exists only at the interface (set/get).  Fluxes and reconstruction are FP32.
#include "agx_internal.cuh"
#include "de_mixed.cuh"
#include "inlet.cuh"
#include "bits.cuh"
#include "../../include/agx_pool.h"
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <cstdio>
#include <map>
#include "free_runs.h"

namespace agx {

constexpr int TILE = 128;

struct PoolScn {             // device-resident per-scenario record
  Clock clock;
  MParams P;
  int cell0, ncell, tile0, ntile;
  int bnd0, nbnd;
  int active, alive;
  const double* series;      // time series rows (t, w, uh, vh) or null
  int nseries;
  int pad[3];
};

constexpr int HALO_MAX = 128;   // halo cells a tile stages in shared memory
constexpr int LNK_INLINE = 1023;

struct PoolDev {
  int ntiles;
  const int* tile_scn;       // [ntiles] scenario of each tile, -1 = free
  const int2* tile_halo;     // [ntiles] (offset, count) into halo_cells
  const int* halo_cells;     // pool cells staged by each tile besides its own
  const int* lnk;            // per cell: staging index of each slot's neighbour (10 bits each)
  float2* tile_red1;         // [tiles] stage-1 partials: (min radius/speed, boundary flux)
  float* tile_red2;          // [tiles] stage-2 boundary flux partials
  unsigned int* ctl;         // [16] grid barrier of the one-kernel step: [0] arrivals, [1] generation, [2] timed out
  PoolScn* scn;
  const int4* conn;          // neighbours (pool-global; boundary -(m+1)) + meta
  const float4* g0;          // M00 M01 M02 M10
  const float4* g1;          // M11 M12 M20 M21
  const float4* g2;          // M22 ex0 ey0 ex1
  float4* g3;                // ey1 ex2 ey2 radius
  float4* g4;                // dz0 dz1 dz2 inv_area
  double *wA, *uhA, *vhA, *wB, *uhB, *vhB, *z;
  const double* area;
  const double* radius;      // FP64 radius of each cell (the CFL quotient of the selected cell)
  float* eta;
  float4 *W0, *W1;           // work records (h, u, v, -) of stage 1 / stage 2
  float4* W2;                // of the third RK3 stage (allocated with the first rk3 scenario)
  float4* E;                 // explicit update (ew, euh, evh, flags)
  float* maxs;
  const int* bkind;
  const double* bval;
  const int* bcell;
  // riverwalls (only read where conn.w bit 20 + i marks slot i a wall edge):
  // crest elevation and hydraulic-table row per slot, the table [row][5]
  const double* rw_crest;
  const int* rw_row;
  const float* rw_hyd;
};

__device__ __forceinline__ int nb_of(int meta) { return (meta >> 16) & 3; }
__device__ __forceinline__ int nedge_of(int meta, int i) { return (meta >> (2 * i)) & 3; }

__device__ __forceinline__ float warp_min_f(float x) {
  for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_down_sync(0xffffffffu, x, o));
  return x;
}
// minimum over the warp, held by every lane
__device__ __forceinline__ float warp_allmin_f(float x) {
  for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ double warp_sum_d(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// Block reductions (TILE threads); results valid in thread 0.
__device__ float block_min_f(float x, float* sh) {
  x = warp_min_f(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  float r = 3.0e38f;
  if (wid == 0) {
    r = lane < TILE / 32 ? sh[lane] : 3.0e38f;
    r = warp_min_f(r);
  }
  __syncthreads();
  return r;
}
__device__ double block_sum_d(double x, double* sh) {
  x = warp_sum_d(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < TILE / 32 ? sh[lane] : 0.0;
    r = warp_sum_d(r);
  }
  __syncthreads();
  return r;
}

// ---- work record: protect + depth + velocity (FP64 depth, FP32 result) ----
// protect: sw_domain_openmp.c:1096-1171; preparation: :1373-1402.  Applies
// the state changes to (w, uh, vh) and returns the work record and the mass
// added.
__device__ __forceinline__ float4 protect_prep(const MParams& P, double& h, double& uh, double& vh,
                                               double area, double& added) {
  added = 0.0;
  if (h < P.hmin64) {
    uh = 0.0;
    if (h < 0.0) {             // stage below the bed
      added = -h * area;
      h = 0.0;
    }
  }
  const double dk = fmax(h, 0.0);
  float4 r;
  r.x = (float)dk;
  r.w = 0.0f;
  if (dk <= P.hmin64) {
    uh = 0.0;
    vh = 0.0;
    r.y = 0.0f;
    r.z = 0.0f;
  } else if (P.velocity_extrapolation) {
    const float inv = 1.0f / r.x;
    r.y = (float)uh * inv;
    r.z = (float)vh * inv;
  } else {
    r.y = (float)uh;
    r.z = (float)vh;
  }
  return r;
}

// ---- reconstruction of one cell's three edges (FP32, relative form) -------
// Core of the reconstruction: the cell's own work record rc and those of its
// three surrogate neighbours r0..r2 (self where a slot is a boundary edge:
// b0..b2 true).
__device__ __forceinline__ void reconstruct_core(const PoolDev& d, const MParams& P, int c, int meta,
                                                 const float4 rc, const float4 r0, const float4 r1,
                                                 const float4 r2, bool b0, bool b1, bool b2,
                                                 EdgeState out[3], bool& sdry) {
  const int nb = nb_of(meta);
  const float hk = rc.x;
  sdry = ((r0.x < P.hmin) | b0) & ((r1.x < P.hmin) | b1) & ((r2.x < P.hmin) | b2);
  float uk = rc.y, vk = rc.z;
  if (sdry) { uk = 0.0f; vk = 0.0f; }
  const float4 a = d.g0[c], b = d.g1[c], e = d.g2[c], f4 = d.g4[c];
  const float M[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, e.x};
  float Dh[3] = {r0.x - hk, r1.x - hk, r2.x - hk};
  float Dw[3] = {f4.x + Dh[0], f4.y + Dh[1], f4.z + Dh[2]};
  float Du[3] = {!b0 ? r0.y - uk : 0.0f, !b1 ? r1.y - uk : 0.0f, !b2 ? r2.y - uk : 0.0f};
  float Dv[3] = {!b0 ? r0.z - vk : 0.0f, !b1 ? r1.z - vk : 0.0f, !b2 ? r2.z - vk : 0.0f};
  if (b0) { Dh[0] = 0.0f; Dw[0] = 0.0f; }
  if (b1) { Dh[1] = 0.0f; Dw[1] = 0.0f; }
  if (b2) { Dh[2] = 0.0f; Dw[2] = 0.0f; }
  float bw, bu, bv;
  if (nb <= 1) {
    const float hlo = fminf(fminf(r0.x, fminf(r1.x, r2.x)), hk);
    const float hhi = fmaxf(fmaxf(r0.x, fmaxf(r1.x, r2.x)), hk);
    const float hf = wet_dry_factor32(P, hk, hlo, hhi);
    bw = P.beta_w_dry + (P.beta_w - P.beta_w_dry) * hf;
    bu = P.beta_uh_dry + (P.beta_uh - P.beta_uh_dry) * hf;
    bv = P.beta_vh_dry + (P.beta_vh - P.beta_vh_dry) * hf;
  } else {
    bw = bu = bv = (nb == 2) ? P.beta_w : 0.0f;
  }
  float Jw[3], Jh[3], Ju[3], Jv[3];
  limited_jumps(M, Dw, bw, Jw);
  limited_jumps(M, Dh, bw, Jh);
  limited_jumps(M, Du, bu, Ju);
  limited_jumps(M, Dv, bv, Jv);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float he = hk + Jh[i];
    const float ue = uk + Ju[i];
    const float ve = vk + Jv[i];
    out[i].h = he;
    if (P.velocity_extrapolation) {
      out[i].uh = ue * he;
      out[i].vh = ve * he;
    } else {
      out[i].uh = ue;
      out[i].vh = ve;
    }
    out[i].dz = Jw[i] - Jh[i];
  }
}

// Reconstruction of cell c gathering the work records from global memory.
__device__ __forceinline__ void reconstruct(const PoolDev& d, const MParams& P, int c, const float4* W,
                                            EdgeState out[3], bool& sdry, float4& rc) {
  const int4 cn = d.conn[c];
  rc = W[c];
  const bool b0 = cn.x < 0, b1 = cn.y < 0, b2 = cn.z < 0;
  const float4 r0 = b0 ? rc : W[cn.x];
  const float4 r1 = b1 ? rc : W[cn.y];
  const float4 r2 = b2 ? rc : W[cn.z];
  reconstruct_core(d, P, c, cn.w, rc, r0, r1, r2, b0, b1, b2, out, sdry);
}

__device__ void series_at(const double* rows, int n, double t, double out[3]) {
  if (n <= 0 || !rows) { out[0] = out[1] = out[2] = 0.0; return; }
  if (t <= rows[0]) { out[0] = rows[1]; out[1] = rows[2]; out[2] = rows[3]; return; }
  if (t >= rows[4 * (n - 1)]) { const double* r = rows + 4 * (n - 1); out[0] = r[1]; out[1] = r[2]; out[2] = r[3]; return; }
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (rows[4 * mid] <= t) lo = mid; else hi = mid;
  }
  const double* A = rows + 4 * lo;
  const double* C = rows + 4 * hi;
  const double ratio = (t - A[0]) / (C[0] - A[0]);
  for (int q = 0; q < 3; q++) out[q] = A[1 + q] + ratio * (C[1 + q] - A[1 + q]);
}

// Manning friction as the factor x with q_new = q_tmp * (1 - x):
// q_new = q_tmp / (1 - dt S), S = -g eta^2 |q| / h^(7/3)  (sw_domain_openmp.c:1954-1986,
// quantity.c:772-818).  x = a / (1 + a), a = -dt S >= 0.
__device__ __forceinline__ float manning_x(const MParams& P, float h, float uh, float vh, float eta, float dt32) {
  if (!(eta > P.hmin) || !(h >= P.hmin)) return 0.0f;
  const float mom = sqrtf(uh * uh + vh * vh);
  const float h73 = h * h * cbrtf(h);
  const float S = P.g * eta * eta * mom / h73;     // -S
  const float a = dt32 * S;
  if (!(a < 1.0e30f)) return 1.0f;
  return a / (1.0f + a);
}

// Work record (depth, velocity) of a state whose depth w - z is `depth`
// (protect and the preparation of the extrapolation, in FP32 on the depth
// formed in FP64).
__device__ __forceinline__ float4 record_of(const MParams& P, double depth, double uh, double vh) {
  const float h = fmaxf(d2f_bits(depth), 0.0f);
  float4 r = make_float4(h, 0.0f, 0.0f, 0.0f);
  if (h > P.hmin) {
    if (P.velocity_extrapolation) {
      const float inv = 1.0f / h;
      r.y = d2f_bits(uh) * inv;
      r.z = d2f_bits(vh) * inv;
    } else {
      r.y = d2f_bits(uh);
      r.z = d2f_bits(vh);
    }
  }
  return r;
}


// FP64 update of one cell from the stage-start state (w, uh, vh):
// protect + preparation zeroing (distribute_to_vertices_and_edges), the
// surrounded-by-dry zeroing, Manning friction with its semi-implicit factor
// (sw_domain_openmp.c:1954-1986, quantity.c:772-818) and fix_negative_cells.
// The depth takes dt*E with the FP64 timestep of the clock (one FP64 fused
// multiply-add, so the volume applied is the one the clock's time advance
// implies); the momentum increments, friction included, are formed in FP32
// from the same timestep rounded once and added in FP64.
// Returns 1 if the cell was fixed as negative; depth1 = w - z afterwards.
__device__ __forceinline__ int update_lean(const MParams& P, double& depth, double& uh, double& vh,
                                           const double* area, float eta, float4 Ek, double dt, float dt32,
                                           double& added) {
  const float h = d2f_bits(depth);
  added = 0.0;
  if (h <= P.hmin) {
    uh = 0.0;
    vh = 0.0;
    if (negative_bits(depth)) {
      added = -depth * (*area);
      depth = 0.0;
    }
  }
  if (Ek.w != 0.0f) { uh = 0.0; vh = 0.0; }
  const float uh32 = d2f_bits(uh), vh32 = d2f_bits(vh);
  const float x = manning_x(P, fmaxf(h, 0.0f), uh32, vh32, eta, dt32);
  depth = fma(dt, f2d_bits(Ek.x), depth);
  float du = dt32 * Ek.y;
  float dv = dt32 * Ek.z;
  du = du - x * (uh32 + du);
  dv = dv - x * (vh32 + dv);
  uh = uh + f2d_bits(du);
  vh = vh + f2d_bits(dv);
  if (negative_bits(depth)) {
    depth = 0.0;
    uh = 0.0;
    vh = 0.0;
    return 1;
  }
  return 0;
}

// A NaN or an infinity in a scenario's conserved state: counted, and the
// scenario's clock stops its step loop with an error (the CFL minimum would
// otherwise pass over the cell and let the NaN spread).
__device__ __noinline__ void report_nonfinite(PoolScn* S, int n) {
  atomicAdd((unsigned long long*)&S->clock.nonfinite_cells, (unsigned long long)n);
  atomicOr(&S->clock.error, (int)ERR_NONFINITE);
}

__device__ __forceinline__ float warp_sum_f(float x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}
__device__ float block_sum_f(float x, float* sh) {
  x = warp_sum_f(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  float r = 0.0f;
  if (wid == 0) {
    r = lane < TILE / 32 ? sh[lane] : 0.0f;
    r = warp_sum_f(r);
  }
  __syncthreads();
  return r;
}

// Boundary kinds 7-10 (shallow_water/boundaries.py: stage given with the
// edge's momenta, the edge's stage with zero momenta, Flather, the
// characteristic stage boundary), out of line so that they take no
// registers in the flux kernel where no edge has them.  Returns the outside
// depth above the edge bed and the momenta; heights relative to the cell's
// centroid bed zc (bv0: the boundary value of the stage).
__device__ __noinline__ float3 boundary_state_rare(int kind, const double* bv, double zc, EdgeState L, float n1,
                                                   float n2, float g) {
  float hre = 0.0f, uhr = 0.0f, vhr = 0.0f;
  const double bv0 = bv[0];
  switch (kind) {
    case BK_INFLOW:                   // boundaries.py:902-992: a depth above the edge bed
      hre = fmaxf((float)bv0, 0.0f);
      uhr = (float)bv[1];
      vhr = (float)bv[2];
      break;
    case BK_TRANSMISSIVE_SET_STAGE:
      hre = fmaxf((float)(bv0 - zc) - L.dz, 0.0f);
      uhr = L.uh;
      vhr = L.vh;
      break;
    case BK_TRANSMISSIVE_ZERO_MOM:
      hre = fmaxf(L.h, 0.0f);
      uhr = 0.0f;
      vhr = 0.0f;
      break;
    case BK_FLATHER: {
      // heights relative to the cell's centroid bed (boundaries.py:1242-1330)
      const float so = (float)(bv0 - zc);
      const float win = L.h + L.dz;               // edge stage - centroid bed
      const float depth = fmaxf(win, 0.0f);
      float q0;
      if (depth == 0.0f || so > 0.0f) {
        q0 = so >= 0.0f ? so : L.dz;
        uhr = 0.0f;
        vhr = 0.0f;
      } else {
        const float sg = sqrtf(g / depth);
        const float ndotq = n1 * L.uh + n2 * L.vh;
        const float w1 = -sg * so;
        const float w2 = ndotq > 0.0f ? (n2 * L.uh - n1 * L.vh) / depth : 0.0f;
        const float w3 = ndotq / depth + sg * win;
        q0 = (w3 - w1) / (2.0f * sg);
        const float qperp = 0.5f * (w3 + w1) * depth;
        const float qpar = w2 * depth;
        uhr = qperp * n1 + qpar * n2;
        vhr = qperp * n2 - qpar * n1;
      }
      hre = fmaxf(q0 - L.dz, 0.0f);
      break;
    }
    case BK_CHARACTERISTIC: {
      // heights relative to the edge bed (boundaries.py:757-848)
      const float ho = fmaxf((float)(bv0 - zc) - L.dz, 0.0f);
      const float hi = fmaxf(L.h, 0.0f);
      if (hi == 0.0f || ho == 0.0f) {
        hre = ho;
        uhr = 0.0f;
        vhr = 0.0f;
      } else {
        const float sqrt_g = sqrtf(g);
        const float uh_in = n1 * L.uh + n2 * L.vh;
        const float vh_in = n2 * L.uh - n1 * L.vh;
        const float u_in = uh_in / hi;
        const float si = sqrtf(hi), so = sqrtf(ho);
        float h_m = 0.5f * (si + so) + 0.25f * u_in / sqrt_g;
        h_m = h_m * h_m;
        const float uh_m = h_m * (0.5f * u_in + sqrt_g * (si - so));
        const float vh_m = uh_in > 0.0f ? vh_in : 0.0f;
        hre = h_m;
        uhr = uh_m * n1 + vh_m * n2;
        vhr = uh_m * n2 - vh_m * n1;
      }
      break;
    }
    default:
      break;
  }
  return make_float3(hre, uhr, vhr);
}

// ---------------------------------------------------------------------------
// Fused flux kernel.  Phase 1 reconstructs the tile's own cells and its halo
// cells (the outside neighbours its edges need) into shared memory; phase 2
// evaluates the three edge fluxes of every own cell from shared memory and
// accumulates them.  STG 1: first stage (explicit update and CFL minimum);
// STG 2: second stage of the two-stage (RK2) scenarios with the update and
// the combine 0.5 Q + 0.5 Q0 into A fused in; STG 4: second stage of the
// three-stage (RK3) scenarios, 0.25 Q + 0.75 Q0 into B; STG 3: their third
// stage, (2 Q + Q0) / 3 into A (generic_domain.py:1974-2172).
// EXT: the extended form, launched only for pools with a riverwall or a
// boundary of kinds 7-10 (riverwall weir branch, the rarer boundaries), so
// that the common form carries none of their registers.
// Flux timestep of a scenario's step from its reduction key: the FP64
// quotient radius / speed of the cell the key selects.
__device__ __forceinline__ double pool_flux_dt(const PoolDev& d, const Clock& c) {
  const unsigned long long key = c.dt_key;
  if (!key) return 1.0e100;
  const int cell = (int)(key & 0xffffffffull);
  return d.radius[cell] / (double)d.maxs[cell];
}

// The timestep of the scenario's current step.  LOCALDT false: the value the
// timestep kernel has written into the clock; true (the one-kernel step):
// formed here from the reduction key, as the clock phase will form it.
template <bool LOCALDT>
__device__ __forceinline__ double step_timestep(const PoolDev& d, const PoolScn* S) {
  if (!LOCALDT) return S->clock.timestep;
  return timestep_value(&S->clock, pool_flux_dt(d, S->clock));
}
// The same for a whole warp (all lanes active): formed by lane 0 and shared,
// so that the one-kernel step pays one FP64 division per warp and tile.
template <bool LOCALDT>
__device__ __forceinline__ double warp_timestep(const PoolDev& d, const PoolScn* S) {
  if (!LOCALDT) return S->clock.timestep;
  double v = 0.0;
  if ((threadIdx.x & 31) == 0) v = timestep_value(&S->clock, pool_flux_dt(d, S->clock));
  return __shfl_sync(0xffffffffu, v, 0);
}
// the same in FP32 (the friction factor's timestep)
template <bool LOCALDT>
__device__ __forceinline__ float step_timestep32(const PoolScn* S, double ts) {
  if (!LOCALDT) return S->clock.timestep32;
  return (float)ts;
}

// 1: the stage-2 flux blocks ask L2, 2: L1, for the FP64 state their update
// reads after the flux loop, when the tile starts (a prefetch holds no
// register); 0: no prefetch.  Measured on the 4.0M-triangle DE1 pool step:
// 0.4985 ms without, 0.4807 with L2, 0.4808 with L1 prefetches.
#ifndef AGX_STATE_PREFETCH
#define AGX_STATE_PREFETCH 1
#endif
// 1: also the cell's area and friction (stage 2) and the geometry block only
// the flux loop reads (both stages): 0.4849 -> 0.4721 ms on the 4.0M-triangle
// step, 0.0702 -> 0.0716 ms on a 0.45M-cell pool of 32 small scenarios
#ifndef AGX_GEO_PREFETCH
#define AGX_GEO_PREFETCH 1
#endif
__device__ __forceinline__ void prefetch_line(const void* p) {
#if AGX_STATE_PREFETCH == 1
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
#elif AGX_STATE_PREFETCH == 2
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
#else
  (void)p;
#endif
}

template <int STG, bool EXT, bool LOCALDT>
__device__ __forceinline__ void flux_phase(const PoolDev& d, EdgeState* es) {
  constexpr bool FUSED2 = STG >= 2;
  const float4* W = STG == 1 ? d.W0 : (STG == 3 ? d.W2 : d.W1);
  for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
    const int base = tile * TILE;
    const int k = base + threadIdx.x;
    // the own cell's tables are loaded before the tile's scenario is known
    const int4 cn_s = d.conn[k];
    const int lk_s = d.lnk[k];
    const float4 rk_s = W[k];
    const int2 ht = d.tile_halo[tile];
    const int sid = d.tile_scn[tile];
    if (sid < 0) continue;
    PoolScn* S = d.scn + sid;
    if (!S->active) continue;
    if (FUSED2 && !S->P.rk2) continue;        // Euler scenarios have one stage
    if (STG == 2 && S->P.rk3) continue;       // RK3 scenarios take STG 4 and 3
    if (STG >= 3 && !S->P.rk3) continue;
    // prefetches only for the tiles of running scenarios (free tiles and
    // finished scenarios' tiles skip the work and need no data)
    if (FUSED2 && AGX_STATE_PREFETCH) {        // k lies inside every per-cell array of the pool
      prefetch_line(d.wB + k);
      prefetch_line(d.uhB + k);
      prefetch_line(d.vhB + k);
      prefetch_line(d.wA + k);
      prefetch_line(d.uhA + k);
      prefetch_line(d.vhA + k);
      if (AGX_GEO_PREFETCH) {
        prefetch_line(d.area + k);
        prefetch_line(d.eta + k);
      }
    }
    if (AGX_GEO_PREFETCH) prefetch_line(d.g3 + k);   // read only by the flux loop
    const MParams P = S->P;
    const double ts_w = FUSED2 ? warp_timestep<LOCALDT>(d, S) : 0.0;     // the step's timestep
    const bool valid = k < S->cell0 + S->ncell;
    bool sdry = false;
    float4 rk = make_float4(0.f, 0.f, 0.f, 0.f);
    EdgeState own[3];
    int4 cn = make_int4(-1, -1, -1, 0);
    int lk = 0;
    if (valid) {
      cn = cn_s;
      lk = lk_s;
      rk = rk_s;
      const bool b0 = cn.x < 0, b1 = cn.y < 0, b2 = cn.z < 0;
      const float4 r0 = b0 ? rk : W[cn.x];
      const float4 r1 = b1 ? rk : W[cn.y];
      const float4 r2 = b2 ? rk : W[cn.z];
      reconstruct_core(d, P, k, cn.w, rk, r0, r1, r2, b0, b1, b2, own, sdry);
    } else {
#pragma unroll
      for (int i = 0; i < 3; i++) own[i] = EdgeState{0.f, 0.f, 0.f, 0.f};
    }
#pragma unroll
    for (int i = 0; i < 3; i++) es[threadIdx.x * 3 + i] = own[i];
    for (int h = threadIdx.x; h < ht.y; h += TILE) {
      EdgeState hs[3];
      bool sd;
      float4 rn;
      reconstruct(d, P, d.halo_cells[ht.x + h], W, hs, sd, rn);
#pragma unroll
      for (int i = 0; i < 3; i++) es[(TILE + h) * 3 + i] = hs[i];
    }
    __syncthreads();
    float ew = 0.f, ex = 0.f, ey = 0.f, smax = 0.f, bfl = 0.f;
    float4 g3 = make_float4(0.f, 0.f, 0.f, 0.f), g4 = g3;
    double sw = 0.0, suh = 0.0, svh = 0.0;
    // A cell whose three edges are dry on both sides (edge depths exactly
    // zero; no boundary, riverwall or unstaged neighbour) has a zero flux:
    // every term the loop below would add is +0 (both Audusse depths are
    // zero, so the flux, the speed and the pressure terms vanish), so the
    // loop and its geometry loads are skipped with the same result.
    bool dry = valid && cn.x >= 0 && cn.y >= 0 && cn.z >= 0 && !(EXT && ((cn.w >> 20) & 7));
    if (dry) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const int li = (lk >> (10 * i)) & 1023;
        const float lh = es[threadIdx.x * 3 + i].h;
        const float rh = li != LNK_INLINE ? es[li * 3 + nedge_of(cn.w, i)].h : 1.0f;
        dry = dry && lh == 0.0f && rh == 0.0f;
      }
    }
    if (valid && !dry) {
      const float4 g2 = d.g2[k];
      g3 = d.g3[k];
      g4 = d.g4[k];
      const float evx[3] = {g2.y, g2.w, g3.y};
      const float evy[3] = {g2.z, g3.x, g3.z};
      const float dzn[3] = {g4.x, g4.y, g4.z};
      const int nbr[3] = {cn.x, cn.y, cn.z};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const EdgeState L = es[threadIdx.x * 3 + i];   // own edge from the staging (fewer live registers)
        const int n = nbr[i];
        float hre, uhr, vhr, dd = 0.0f;
        const float len = sqrtf(evx[i] * evx[i] + evy[i] * evy[i]);
        const float il = 1.0f / len;
        const float n1 = evy[i] * il, n2 = -evx[i] * il;
        if (n >= 0) {
          const int m = nedge_of(cn.w, i);
          const int li = (lk >> (10 * i)) & 1023;
          EdgeState R;
          if (li != LNK_INLINE) {
            R = es[li * 3 + m];
          } else {      // halo overflow: reconstruct inline
            EdgeState tmp[3];
            bool sd;
            float4 rn;
            reconstruct(d, P, n, W, tmp, sd, rn);
            R = m == 0 ? tmp[0] : (m == 1 ? tmp[1] : tmp[2]);
          }
          hre = R.h;
          uhr = R.uh;
          vhr = R.vh;
          dd = dzn[i] + R.dz - L.dz;        // zr - zl
        } else {
          const int mb = -n - 1;
          const int kind = d.bkind[mb];
          const double* bv = d.bval + 3 * (size_t)mb;
          switch (kind) {
            case BK_REFLECTIVE: {
              hre = fmaxf(L.h, 0.0f);
              const float q1 = L.uh, q2 = L.vh;
              const float r1 = -q1 * n1 - q2 * n2;
              const float r2 = -q1 * n2 + q2 * n1;
              uhr = n1 * r1 - n2 * r2;
              vhr = n2 * r1 + n1 * r2;
              break;
            }
            case BK_TRANSMISSIVE:
              hre = fmaxf(L.h, 0.0f);
              uhr = L.uh;
              vhr = L.vh;
              break;
            case BK_TRANSMISSIVE_C:
              hre = fmaxf(rk.x - L.dz, 0.0f);
              uhr = P.velocity_extrapolation ? rk.y * rk.x : rk.y;
              vhr = P.velocity_extrapolation ? rk.z * rk.x : rk.z;
              break;
            case BK_TRANSMISSIVE_SET_STAGE:
            case BK_TRANSMISSIVE_ZERO_MOM:
            case BK_FLATHER:
            case BK_CHARACTERISTIC:
            case BK_INFLOW: {
              if (EXT) {
                const float3 q = boundary_state_rare(kind, bv, d.z[k], L, n1, n2, P.g);
                hre = q.x;
                uhr = q.y;
                vhr = q.z;
              } else {     // not reached: such pools run the extended form
                hre = fmaxf(L.h, 0.0f);
                uhr = 0.0f;
                vhr = 0.0f;
              }
              break;
            }
            case BK_TRANSMISSIVE_N0: {
              hre = fmaxf((float)(bv[0] - d.z[k]) - L.dz, 0.0f);
              const float nq = n1 * L.uh + n2 * L.vh;
              uhr = nq * n1;
              vhr = nq * n2;
              break;
            }
            case BK_TIME_SERIES: {
              double v3[3];
              const double tnow = STG == 1 ? S->clock.time : S->clock.time + (STG == 3 ? 0.5 : 1.0) * ts_w;
              series_at(S->series, S->nseries, tnow, v3);
              hre = fmaxf((float)(v3[0] - d.z[k]) - L.dz, 0.0f);
              uhr = (float)v3[1];
              vhr = (float)v3[2];
              break;
            }
            default: {   // Dirichlet, or no boundary object (values stay zero)
              hre = fmaxf((float)(bv[0] - d.z[k]) - L.dz, 0.0f);
              uhr = (float)bv[1];
              vhr = (float)bv[2];
              break;
            }
          }
        }
        Flux32 F;
        if (EXT && ((cn.w >> (20 + i)) & 1)) {
          // riverwall edge (sw_domain_openmp.c:581-650), all heights relative
          // to this edge's bed zl: crest c, Audusse bed zh = max(0, zr - zl, c)
          const size_t q = 3 * (size_t)k + i;
          const float c = (float)(d.rw_crest[q] - d.z[k]) - L.dz;
          central_flux32<true>(L.h, L.uh, L.vh, hre, uhr, vhr, dd, n1, n2, P, F, c);
          const float zh = fmaxf(fmaxf(dd, 0.0f), c);
          // neighbour centroid bed - zl; on a boundary edge the reference
          // takes the cell's own centroid and zr = zl for the far head
          const float zn = n >= 0 ? dzn[i] - L.dz : -L.dz;
          const float hl_c = fmaxf(rk.x - L.dz - zh, 0.0f);      // own centroid stage - z_half
          const float hr_c = n >= 0 ? fmaxf(W[n].x + zn - zh, 0.0f) : fmaxf(rk.x + dd - zh, 0.0f);
          const float weir_height = fmaxf(c - fminf(dd, 0.0f), 0.0f);
          if (c > fmaxf(-L.dz, zn)) weir_adjust32(F, hl_c, hr_c, P.g, weir_height, d.rw_hyd + 5 * d.rw_row[q]);
        } else {
          central_flux32(L.h, L.uh, L.vh, hre, uhr, vhr, dd, n1, n2, P, F);
        }
        const float e0 = -F.f0 * len;
        const float e1 = -F.f1 * len;
        const float e2 = -F.f2 * len;
        const float pg = len * (-P.g * 0.5f * (F.hl * F.hl - L.h * L.h - (L.h + rk.x) * L.dz) + F.pflux);
        ew += e0;
        ex += e1;
        ey += e2;
        ex -= n1 * pg;
        ey -= n2 * pg;
        if (F.speed > P.eps) smax = fmaxf(smax, F.speed);
        if (n < 0) bfl += e0;
      }
      const float ia = g4.w;
      ew *= ia;
      ex *= ia;
      ey *= ia;
    }
    if (!FUSED2) {
      float dtk = 3.0e38f;
      if (valid) {
        d.E[k] = make_float4(ew, ex, ey, sdry ? 1.0f : 0.0f);
        d.maxs[k] = smax;
        if (smax > 0.0f) dtk = g3.w / smax;
      }
      // per-warp reductions, no block barrier.  The CFL key selects the
      // cell of the smallest FP32 radius/speed (ties: the higher index) and
      // is order independent whatever the grouping; the timestep kernel
      // forms that cell's quotient in FP64.  The boundary flux sum is
      // accumulated by atomics in no fixed order either way.
      const float wm = warp_allmin_f(dtk);
      const float ws = warp_sum_f(bfl);
      const unsigned win = __ballot_sync(0xffffffffu, dtk == wm);
      if ((threadIdx.x & 31) == 0) {      // fire-and-forget reductions (no return value)
        if (wm < 3.0e38f) {
          const int cell = k + 31 - __clz(win);
          const unsigned long long key = ((unsigned long long)(~__float_as_uint(wm)) << 32) | (unsigned)cell;
          if (key > __ldcg(&S->clock.dt_key)) atomicMax(&S->clock.dt_key, key);   // only a new maximum
        }
        if (ws != 0.0f) atomicAdd(&S->clock.bfs_acc, (double)ws);
      }
    } else {
      int neg = 0, nf = 0;
      double added = 0.0;
      if (valid) {
        sw = d.wB[k];
        suh = d.uhB[k];
        svh = d.vhB[k];
        double h = sw, uh = suh, vh = svh;
        neg = update_lean(P, h, uh, vh, d.area + k, d.eta[k], make_float4(ew, ex, ey, sdry ? 1.f : 0.f),
                          ts_w, step_timestep32<LOCALDT>(S, ts_w), added);
        if (STG == 2) {
          h = half_sum(h, d.wA[k]);
          uh = half_sum(uh, d.uhA[k]);
          vh = half_sum(vh, d.vhA[k]);
          d.wA[k] = h;
          d.uhA[k] = uh;
          d.vhA[k] = vh;
          d.W0[k] = record_of(P, h, uh, vh);     // work record of the next step
        } else if (STG == 4) {                    // RK3: Q2 = 0.25 Q + 0.75 Q0 (depth-linear)
          h = 0.25 * h + 0.75 * d.wA[k];
          uh = 0.25 * uh + 0.75 * d.uhA[k];
          vh = 0.25 * vh + 0.75 * d.vhA[k];
          d.wB[k] = h;
          d.uhB[k] = uh;
          d.vhB[k] = vh;
          d.W2[k] = record_of(P, h, uh, vh);     // work record of the third stage
        } else {                                  // RK3: Q = (2 Q + Q0) / 3
          h = ddiv(2.0 * h + d.wA[k], 3.0);       // correctly rounded, off the FP64 pipe
          uh = ddiv(2.0 * uh + d.uhA[k], 3.0);
          vh = ddiv(2.0 * vh + d.vhA[k], 3.0);
          d.wA[k] = h;
          d.uhA[k] = uh;
          d.vhA[k] = vh;
          d.W0[k] = record_of(P, h, uh, vh);
        }
        nf = nonfinite64(h) | nonfinite64(uh) | nonfinite64(vh);
      }
      // per-warp reductions, no block barrier (the sums go to atomics in no
      // fixed order either way)
      const float ws = warp_sum_f(bfl);
      const unsigned anym = __ballot_sync(0xffffffffu, __double_as_longlong(added) != 0);
      const double wa = anym ? warp_sum_d(added) : 0.0;
      const int wneg = __popc(__ballot_sync(0xffffffffu, neg));
      const int wnf = __popc(__ballot_sync(0xffffffffu, nf));
      if ((threadIdx.x & 31) == 0) {
        if (ws != 0.0f) atomicAdd(&S->clock.bfs[STG == 3 ? 2 : 1], (double)ws);
        if (wa != 0.0) atomicAdd(&S->clock.mass_added, wa);
        if (wneg) atomicAdd((unsigned long long*)&S->clock.negative_cells, (unsigned long long)wneg);
        if (wnf) report_nonfinite(S, wnf);
      }
    }
    __syncthreads();
  }
}

template <int STG, int MINB, bool EXT = false>
__global__ void __launch_bounds__(TILE, MINB) k_pool_flux(PoolDev d) {
  __shared__ EdgeState es[(TILE + HALO_MAX) * 3];
  flux_phase<STG, EXT, false>(d, es);
}

// Stage-1 update (RK2: q1 into B; Euler: in place into A) and the next
// stage's work record.  One block per tile; warp-level bookkeeping only.
template <bool LOCALDT>
__device__ __forceinline__ void update_phase(const PoolDev& d) {
  for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
    const int k = tile * TILE + threadIdx.x;
    // the cell's data are loaded before the tile's scenario is known (every
    // index of a used tile lies inside the pool's arrays)
    double h = d.wA[k], uh = d.uhA[k], vh = d.vhA[k];
    const float etak = d.eta[k];
    const float4 Ek = d.E[k];
    const int sid = d.tile_scn[tile];
    if (sid < 0) continue;
    PoolScn* S = d.scn + sid;
    if (!S->active) continue;
    const MParams P = S->P;
    const int euler = !P.rk2;
    const double ts = warp_timestep<LOCALDT>(d, S);
    const bool valid = k < S->cell0 + S->ncell;
    int neg = 0, nf = 0;
    double added = 0.0;
    if (valid) {
      neg = update_lean(P, h, uh, vh, d.area + k, etak, Ek, ts, step_timestep32<LOCALDT>(S, ts), added);
      if (euler) nf = nonfinite64(h) | nonfinite64(uh) | nonfinite64(vh);   // the step's result (RK2: checked after stage 2)
      const float4 r = record_of(P, h, uh, vh);
      if (euler) {
        d.wA[k] = h; d.uhA[k] = uh; d.vhA[k] = vh;
        d.W0[k] = r;
      } else {
        d.wB[k] = h; d.uhB[k] = uh; d.vhB[k] = vh;
        d.W1[k] = r;
      }
    }
    const unsigned full = 0xffffffffu;
    const unsigned nb = __ballot_sync(full, neg);
    if (__any_sync(full, __double_as_longlong(added) != 0)) {
      const double ws = warp_sum_d(added);
      if ((threadIdx.x & 31) == 0 && ws != 0.0) atomicAdd(&S->clock.mass_added, ws);
    }
    if (nb && (threadIdx.x & 31) == 0)
      atomicAdd((unsigned long long*)&S->clock.negative_cells, (unsigned long long)__popc(nb));
    if (euler) {                          // uniform over the tile (one scenario)
      const unsigned nfb = __ballot_sync(full, nf);
      if (nfb && (threadIdx.x & 31) == 0) report_nonfinite(S, __popc(nfb));
    }
  }
}

__global__ void __launch_bounds__(TILE) k_pool_update(PoolDev d, int unused) {
  (void)unused;
  update_phase<false>(d);
}

// Work record from the state A (after set_field or an operator), optionally
// applying protect to A in place (distribute_to_vertices_and_edges).
__global__ void k_pool_prep(PoolDev d, int inplace, int only_scn) {
  __shared__ double shd[TILE / 32];
  for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
    const int sid = d.tile_scn[tile];
    if (sid < 0 || (only_scn >= 0 && sid != only_scn)) continue;
    PoolScn* S = d.scn + sid;
    const int k = tile * TILE + threadIdx.x;
    const bool valid = k < S->cell0 + S->ncell;
    double added = 0.0;
    if (valid) {
      double h = d.wA[k], uh = d.uhA[k], vh = d.vhA[k];
      d.W0[k] = protect_prep(S->P, h, uh, vh, d.area[k], added);
      if (inplace) { d.wA[k] = h; d.uhA[k] = uh; d.vhA[k] = vh; }
    }
    const double ma = block_sum_d(added, shd);
    if (threadIdx.x == 0 && inplace && ma != 0.0) atomicAdd(&S->clock.mass_added, ma);
  }
}

// Surrounded-by-dry momentum zeroing of the extrapolation (persistent part).
__global__ void k_pool_sdry(PoolDev d, int only_scn) {
  for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
    const int sid = d.tile_scn[tile];
    if (sid < 0 || (only_scn >= 0 && sid != only_scn)) continue;
    PoolScn* S = d.scn + sid;
    const int k = tile * TILE + threadIdx.x;
    if (k >= S->cell0 + S->ncell) continue;
    const int4 cn = d.conn[k];
    const float hm = S->P.hmin;
    const int s0 = cn.x >= 0 ? cn.x : k, s1 = cn.y >= 0 ? cn.y : k, s2 = cn.z >= 0 ? cn.z : k;
    const bool sd = ((d.W0[s0].x < hm) | (s0 == k)) & ((d.W0[s1].x < hm) | (s1 == k)) & ((d.W0[s2].x < hm) | (s2 == k));
    if (sd) { d.uhA[k] = 0.0; d.vhA[k] = 0.0; }
  }
}

// Bed differences to the surrogate neighbours (after the elevation changes).
__global__ void k_pool_dz(PoolDev d, int only_scn) {
  for (int tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
    const int sid = d.tile_scn[tile];
    if (sid < 0 || (only_scn >= 0 && sid != only_scn)) continue;
    PoolScn* S = d.scn + sid;
    const int k = tile * TILE + threadIdx.x;
    if (k >= S->cell0 + S->ncell) continue;
    const int4 cn = d.conn[k];
    const double zk = d.z[k];
    float4 g = d.g4[k];
    g.x = cn.x >= 0 ? (float)(d.z[cn.x] - zk) : 0.0f;
    g.y = cn.y >= 0 ? (float)(d.z[cn.y] - zk) : 0.0f;
    g.z = cn.z >= 0 ? (float)(d.z[cn.z] - zk) : 0.0f;
    d.g4[k] = g;
  }
}

// Edge and vertex values in FP64 (for output and the Quantity API).
__global__ void k_pool_edges(PoolDev d, int sid, double* we, double* he, double* uhe, double* vhe, double* ze,
                             const int* order) {
  PoolScn* S = d.scn + sid;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= S->ncell) return;
  const int k = S->cell0 + j;
  EdgeState es[3];
  bool sd;
  float4 rk;
  reconstruct(d, S->P, k, d.W0, es, sd, rk);
  const int o = order[j];
  const double z = d.z[k];
  for (int i = 0; i < 3; i++) {
    const double zz = z + (double)es[i].dz;
    ze[3 * (size_t)o + i] = zz;
    he[3 * (size_t)o + i] = es[i].h;
    we[3 * (size_t)o + i] = zz + (double)es[i].h;
    uhe[3 * (size_t)o + i] = es[i].uh;
    vhe[3 * (size_t)o + i] = es[i].vh;
  }
}

// One vertex slot's stage, bed and momenta in FP64 from the reconstruction of
// its cell, formed as k_pool_edges forms the edge values and the vertex value
// from them as the host export does (vertex i = e(i+1) + e(i+2) - e(i)).
__device__ __forceinline__ void pool_vertex(const PoolDev& d, const MParams& P, int k, int i, double& w, double& z,
                                            double& uh, double& vh) {
  EdgeState es[3];
  bool sd;
  float4 rk;
  reconstruct(d, P, k, d.W0, es, sd, rk);
  const double zc = d.z[k];
  double we[3], ze[3], ue[3], ve[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    ze[j] = zc + (double)es[j].dz;
    we[j] = ze[j] + (double)es[j].h;
    ue[j] = es[j].uh;
    ve[j] = es[j].vh;
  }
  const int a = i == 0 ? 1 : 0, b = i == 2 ? 1 : 2;      // the two other edges, in increasing order
  w = we[a] + we[b] - we[i];
  z = ze[a] + ze[b] - ze[i];
  uh = ue[a] + ue[b] - ue[i];
  vh = ve[a] + ve[b] - ve[i];
}

// sww frame of one scenario (see agx_sww_frame): node means of the centroid
// values of the slots' triangles (centroid_avg) or of the slots' vertex
// values, the storable-height mask at the nodes, centroid values as stored.
__global__ void k_pool_sww_nodes(PoolDev d, int sid, int P, const int* off, const int* slot, const int* inv,
                                 double msh, int centroid_avg, float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const PoolScn* S = d.scn + sid;
  double aw = 0.0, az = 0.0, au = 0.0, av = 0.0;
  const int a = off[p], b = off[p + 1];
  for (int q = a; q < b; q++) {
    const int s = slot[q];
    const int ko = s / 3;
    const int k = S->cell0 + inv[ko];
    double w, z, uh, vh;
    if (centroid_avg) {
      z = d.z[k];
      w = d.wA[k] + z;
      uh = d.uhA[k];
      vh = d.vhA[k];
    } else {
      pool_vertex(d, S->P, k, s - 3 * ko, w, z, uh, vh);
    }
    aw += w;
    az += z;
    au += uh;
    av += vh;
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

__global__ void k_pool_sww_cells(PoolDev d, int sid, const int* order, float* out) {
  const PoolScn* S = d.scn + sid;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = S->ncell;
  if (j >= n) return;
  const int k = S->cell0 + j, o = order[j];
  out[o] = (float)(d.wA[k] + d.z[k]);
  out[n + o] = (float)d.uhA[k];
  out[2 * n + o] = (float)d.vhA[k];
}

// update_timestep per scenario (one thread each).
__global__ void k_pool_timestep(PoolDev d, int nscn) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nscn) return;
  PoolScn* S = d.scn + s;
  if (!S->alive || !S->active) return;
  const unsigned long long key = S->clock.dt_key;
  if (key) {                 // radius / speed of the selected cell in FP64
    const int c = (int)(key & 0xffffffffull);
    const double dt = d.radius[c] / (double)d.maxs[c];
    S->clock.dt_key = ~(unsigned long long)__double_as_longlong(dt);
  }
  S->clock.bfs[0] = S->clock.bfs_acc;
  timestep_logic(&S->clock);
}

__global__ void k_pool_reset(PoolDev d, int nscn) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nscn) return;
  PoolScn* S = d.scn + s;
  S->clock.dt_key = 0ull;
  S->clock.bfs_acc = 0.0;
  S->clock.bfs[1] = 0.0;
  S->clock.bfs[2] = 0.0;       // third (RK3) stage's sum
}

// A fractional-step operator of one scenario: Rate_operator (kind 0) or
// Inlet_operator (kind 1: rate = the discharge Q, vu/vv the imposed velocity
// when flags & 1, zero velocity when flags & 2, area = the inlet's area).
struct PoolOp {
  int sid;
  const int* idx;    // pool cells
  int n;
  double rate, factor;
  int kind = 0;
  int flags = 0;
  double vu = 0.0, vv = 0.0, area = 0.0;
  double dt = -1.0;  // < 0: the step's timestep from the scenario's clock
};

// Rate_operator change of one cell of op's index set; returns the influx.
__device__ __forceinline__ double rate_cell(const PoolDev& d, const PoolOp& op, PoolScn* S) {
  const int k = op.idx[threadIdx.x + blockIdx.x * blockDim.x];
  const double dt = op.dt >= 0.0 ? op.dt : S->clock.timestep;
  double infl;
  if (op.rate >= 0.0) {
    const double local = op.factor * dt * op.rate;
    d.wA[k] = d.wA[k] + local;
    infl = local * d.area[k];
  } else {
    const double height = d.wA[k];
    const double local = fmax(op.factor * dt * op.rate, -height);
    const double f = local < 0.0 ? (local + height) / (height + 1.0e-10) : 1.0;
    d.wA[k] = d.wA[k] + local;
    d.uhA[k] = d.uhA[k] * f;
    d.vhA[k] = d.vhA[k] * f;
    infl = local * d.area[k];
  }
  double h = d.wA[k], uh = d.uhA[k], vh = d.vhA[k], added;
  d.W0[k] = protect_prep(S->P, h, uh, vh, d.area[k], added);
  return infl;
}

// One application of a Rate_operator: inside the step loop (from_host 0)
// only while the scenario is running; from the host after a step always.
__global__ void __launch_bounds__(256) k_pool_rate(PoolDev d, PoolOp op, int slot, int from_host) {
  __shared__ double part[256 / 32];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  PoolScn* S = d.scn + op.sid;
  if (!from_host && !S->active) return;
  double infl = 0.0;
  if (j < op.n) infl = rate_cell(d, op, S);
  // influx: one atomic per block (a single address receives every block's sum)
  infl = warp_sum_d(infl);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = infl;
  __syncthreads();
  if (wid == 0) {
    double r = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    r = warp_sum_d(r);
    if (lane == 0 && slot < MAX_OPS && r != 0.0) atomicAdd(&S->clock.op_influx[slot], r);
  }
}

// Inlet_operator on the pool's depth-stored state (steps in inlet.cuh).
struct PoolInletCells {
  PoolDev d;
  const int* idx;
  __device__ int cell(int a) const { return idx[a]; }
  __device__ double stage(int k) const { return d.wA[k] + d.z[k]; }
  __device__ double height(int k) const { return d.wA[k]; }
  __device__ double area(int k) const { return d.area[k]; }
  __device__ double uh(int k) const { return d.uhA[k]; }
  __device__ double vh(int k) const { return d.vhA[k]; }
  __device__ void set_level(int k, double level) { d.wA[k] = level - d.z[k]; }
  __device__ void set_depth(int k, double depth) { d.wA[k] = depth; }
  __device__ void empty(int k) {
    d.wA[k] = 0.0;
    d.uhA[k] = 0.0;
    d.vhA[k] = 0.0;
  }
  __device__ void set_momenta(int k, double mx, double my) {
    d.uhA[k] = mx;
    d.vhA[k] = my;
  }
};

// Discharge Q = 0.5 (q1 + q2) over the timestep (op.dt, or the clock's);
// the changed cells' work records are formed again for the next step.
__global__ void __launch_bounds__(INLET_TPB) k_pool_inlet(PoolDev d, PoolOp op, int slot, double q1, double q2,
                                                          int from_host) {
  PoolScn* S = d.scn + op.sid;
  if (!from_host && !S->active) return;
  const double dt = op.dt >= 0.0 ? op.dt : S->clock.timestep;
  PoolInletCells c{d, op.idx};
  const double applied = inlet_apply(c, op.n, op.flags, op.vu, op.vv, op.area, 0.5 * (q1 + q2) * dt);
  for (int a = threadIdx.x; a < op.n; a += INLET_TPB) {
    const int k = op.idx[a];
    double h = d.wA[k], uh = d.uhA[k], vh = d.vhA[k], added;
    d.W0[k] = protect_prep(S->P, h, uh, vh, d.area[k], added);
  }
  if (threadIdx.x == 0 && slot < MAX_OPS) S->clock.op_influx[slot] += applied;
}

// ---------------------------------------------------------------------------
// The whole DE step of every scenario in one cooperative launch (two-stage
// and one-stage scenarios without riverwalls, the rarer boundary kinds or
// inlets in the step loop): stage-1 fluxes, the first update, the stage-2
// fluxes with the RK2 combine, the rates, and the clocks, separated by grid
// barriers.  Every block computes each scenario's timestep from the reduced
// key as the clock phase does (timestep_value), so no barrier is spent on
// the timestep itself.

// One rate operator of the one-kernel step and its influx slot.
struct StepOp {
  PoolOp op;
  int slot;
  int pad;
};

constexpr unsigned long long BARRIER_SPINS = 1ull << 26;   // with the sleeps below: tens of seconds

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier over the cooperative launch's blocks (all resident).  A
// block whose wait runs out of spins records it in ctl[2] and returns false;
// a block that enters with ok false does not arrive (its later barriers then
// run out too, and the step ends with an error instead of a hang).
__device__ bool grid_barrier(unsigned* ctl, unsigned& gen, bool ok) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = ok ? 1 : 0;
    if (good) {
      __threadfence();
      const unsigned g = gen;
      if (atomicAdd(&ctl[0], 1u) == gridDim.x - 1) {
        atomicExch(&ctl[0], 0u);
        __threadfence();
        atomicAdd(&ctl[1], 1u);
      } else {
        unsigned long long n = 0;
        while (ld_acquire_u32(&ctl[1]) == g) {
          if (++n > BARRIER_SPINS) {
            good = 0;
            atomicOr(&ctl[2], 1u);
            break;
          }
          __nanosleep(256);
        }
      }
      gen = g + 1;
      __threadfence();
    }
    s_ok = good;
  }
  __syncthreads();
  return s_ok != 0;
}

// Rate_operator changes of the step (k_pool_rate over the whole grid).
__device__ void rate_phase(const PoolDev& d, const StepOp* ops, int nops) {
  const int nthreads = gridDim.x * blockDim.x;
  for (int o = 0; o < nops; o++) {
    const PoolOp op = ops[o].op;
    PoolScn* S = d.scn + op.sid;
    if (!S->active) continue;
    double infl = 0.0;
    const double ts = warp_timestep<true>(d, S);         // the step's timestep, as the clock phase forms it
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < op.n; j += nthreads) {
      const int k = op.idx[j];
      if (op.rate >= 0.0) {
        const double local = op.factor * ts * op.rate;
        d.wA[k] = d.wA[k] + local;
        infl += local * d.area[k];
      } else {
        const double height = d.wA[k];
        const double local = fmax(op.factor * ts * op.rate, -height);
        const double f = local < 0.0 ? (local + height) / (height + 1.0e-10) : 1.0;
        d.wA[k] = d.wA[k] + local;
        d.uhA[k] = d.uhA[k] * f;
        d.vhA[k] = d.vhA[k] * f;
        infl += local * d.area[k];
      }
      double h = d.wA[k], uh = d.uhA[k], vh = d.vhA[k], added;
      d.W0[k] = protect_prep(S->P, h, uh, vh, d.area[k], added);
    }
    infl = warp_sum_d(infl);
    if ((threadIdx.x & 31) == 0 && infl != 0.0 && ops[o].slot < MAX_OPS)
      atomicAdd(&S->clock.op_influx[ops[o].slot], infl);
  }
}

// The clocks (block 0): the timestep bookkeeping of k_pool_timestep, the end
// of the step of k_pool_clock, then the accumulators of the next step are
// cleared.  Always sets the while condition (0 after a barrier that ran out).
__device__ void clock_phase(const PoolDev& d, int nscn, bool ok, cudaGraphConditionalHandle handle, int set_cond) {
  int running = 0;
  for (int s = threadIdx.x; s < nscn; s += blockDim.x) {
    PoolScn* S = d.scn + s;
    if (!S->alive || !S->active) continue;
    Clock* c = &S->clock;
    if (c->dt_key) c->dt_key = ~(unsigned long long)__double_as_longlong(pool_flux_dt(d, *c));
    c->bfs[0] = c->bfs_acc;
    timestep_logic(c);
    if (!ok) c->error |= ERR_BARRIER;
    const int reason = clock_logic(c);
    if (reason) S->active = 0;
    else running = 1;
    c->dt_key = 0ull;
    c->bfs_acc = 0.0;
    c->bfs[1] = 0.0;
    c->bfs[2] = 0.0;
  }
  const int any = __syncthreads_or(running);
  if (threadIdx.x == 0 && set_cond) cudaGraphSetConditional(handle, (any && ok) ? 1u : 0u);
}

template <int MINB>
__global__ void __launch_bounds__(TILE, MINB) k_pool_step(PoolDev d, const StepOp* ops, int nops, int nscn,
                                                         cudaGraphConditionalHandle handle, int set_cond) {
  __shared__ EdgeState es[(TILE + HALO_MAX) * 3];
  __shared__ unsigned s_gen;
  if (threadIdx.x == 0) s_gen = ld_acquire_u32(&d.ctl[1]);
  __syncthreads();
  unsigned gen = s_gen;
  flux_phase<1, false, true>(d, es);
  bool ok = grid_barrier(d.ctl, gen, true);
  if (ok) update_phase<true>(d);
  ok = grid_barrier(d.ctl, gen, ok);
  if (ok) flux_phase<2, false, true>(d, es);
  ok = grid_barrier(d.ctl, gen, ok);
  if (nops > 0) {
    if (ok) rate_phase(d, ops, nops);
    ok = grid_barrier(d.ctl, gen, ok);
  }
  if (blockIdx.x == 0) clock_phase(d, nscn, ok, handle, set_cond);
}

// Before the step loop of the one-kernel step: the accumulators of the first
// step cleared, the grid barrier's arrival count and timeout flag reset.
__global__ void k_pool_step_prepare(PoolDev d, int nscn) {
  for (int s = threadIdx.x; s < nscn; s += blockDim.x) {
    Clock* c = &d.scn[s].clock;
    c->dt_key = 0ull;
    c->bfs_acc = 0.0;
    c->bfs[1] = 0.0;
    c->bfs[2] = 0.0;
  }
  if (threadIdx.x == 0) {
    d.ctl[0] = 0u;
    d.ctl[2] = 0u;
  }
}

// Per-scenario clocks (one thread each, one block); sets the graph's while
// condition when any scenario is still running.
__global__ void k_pool_clock(PoolDev d, int nscn, cudaGraphConditionalHandle handle, int set_cond) {
  int running = 0;
  for (int s = threadIdx.x; s < nscn; s += blockDim.x) {
    PoolScn* S = d.scn + s;
    if (!S->alive || !S->active) continue;
    const int reason = clock_logic(&S->clock);
    if (reason) S->active = 0;
    else running = 1;
  }
  const int any = __syncthreads_or(running);
  if (threadIdx.x == 0 && set_cond) cudaGraphSetConditional(handle, any ? 1u : 0u);
}

__global__ void k_gather(double* dst, const double* src, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[j] = src[order[j]];
}
__global__ void k_gather_f(float* dst, const double* src, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[j] = (float)src[order[j]];
}
__global__ void k_scatter(double* dst, const double* src, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[order[j]] = src[j];
}
__global__ void k_scatter_f(double* dst, const float* src, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[order[j]] = (double)src[j];
}
__global__ void k_scatter_height(double* dst, const double* h, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[order[j]] = fmax(h[j], 0.0);
}
// The pool's conserved state is (depth h = stage - bed, uh, vh) in FP64; the
// stage exists only at the interface.
__global__ void k_gather_depth(double* h, const double* z, const double* stage, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) h[j] = stage[order[j]] - z[j];
}
__global__ void k_gather_bed(double* h, double* z, const double* bed, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const double zn = bed[order[j]];
    h[j] = (h[j] + z[j]) - zn;
    z[j] = zn;
  }
}
__global__ void k_scatter_stage(double* dst, const double* h, const double* z, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[order[j]] = h[j] + z[j];
}
__global__ void k_scatter_E(double* dst, const float4* E, int comp, const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const float4 e = E[j];
    dst[order[j]] = comp == 0 ? e.x : comp == 1 ? e.y : e.z;
  }
}

// ---------------------------------------------------------------------------
// host side
struct ScnHost {
  int alive = 0;
  // sww output: node -> vertex-slot map (original order), device frame and its page-locked copy
  int sww_P = 0;
  int* sww_off = nullptr;
  int* sww_slot = nullptr;
  float* frame = nullptr;
  float* frame_host = nullptr;
  cudaEvent_t frame_done = nullptr;
  cudaEvent_t frame_ready = nullptr;      // after the frame kernels
  cudaStream_t copy_stream = nullptr;     // the frame copy's own stream
  int N = 0, B = 0, tile0 = 0, ntile = 0, bnd0 = 0, halo0 = 0, nhalo = 0;
  agx_params prm{};
  int* order = nullptr;          // device [N]: original index of each stored cell
  int* inv = nullptr;            // device [N]: stored index of each original cell
  double* series = nullptr;
  std::vector<PoolOp> ops;
  bool host_ops = false;         // operators applied from the host after each step, not in the loop
  bool work_dirty = true;
  bool running = false;          // serving: still has steps to take towards its final time
};

struct Pool {
  int device = 0;
  int cap_cells = 0, cap_tiles = 0, cap_bnd = 0, cap_scn = 0, cap_halo = 0;
  std::vector<int> halo_owner;   // host: halo slot owner (-1 free)
  FreeRuns free_tiles, free_bnd, free_halo;
  PoolDev d{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  int* tile_scn_dev = nullptr;
  std::vector<int> tile_scn;     // host mirror
  std::vector<int> bnd_owner;    // host: boundary slot owner (-1 free)
  std::vector<ScnHost> scn;
  PoolScn* scn_host = nullptr;   // pinned mirror of d.scn
  // scn_host equals d.scn: set by every pull and push, cleared by every
  // launch of a kernel that writes the headers (the step kernels, operators
  // and protect-in-place); a pull that may be skipped then costs nothing.
  bool scn_fresh = false;
  double* staging = nullptr;     // device [cap_cells * 3] for permuted copies
  double* staging_host = nullptr;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_valid = false;
  int grid = 0;
  int grid_v[2] = {0, 0};        // persistent grid per flux variant
  int variant = 1;               // flux kernel variant: 0 = at most 6 blocks of 128 per SM (80 registers),
                                 // 1 = at most 8 (64 registers; the faster one on every large pool measured)
  int grid_mode = 0;             // 0 = persistent grid, 1 = one block per tile, 2 = one-kernel step
  int step_grid[2] = {0, 0};     // resident blocks of the one-kernel step per variant
  StepOp* step_ops = nullptr;    // device table of the step loop's rate operators
  int step_nops = 0;
  int l2_window = 0;             // 1: the work records a kernel gathers are kept in L2 (access policy window)
  size_t l2_persist_max = 0;     // the device's persisting L2 size and window limit
  size_t l2_window_max = 0;
  void* snap = nullptr;          // snapshot of the dynamic state (autotuning, checkpoints)
  size_t snap_bytes = 0;
  int kernels_per_iter = 0;
  int mode_rk2_any = 1;
  bool rw_any = false;           // some scenario has riverwalls: the flux kernels take the wall branch
  bool rare_bc_any = false;      // some boundary has kind 7-10: the extended flux kernels run
  bool rk3_any = false;          // some scenario has three stages: the third-stage flux kernel runs
  int stages_done = 0;           // stages run by agx_pool_step_begin / _stage in the current split step
  void* w2_mem = nullptr;        // third-stage work records
  void* rw_mem = nullptr;        // per-slot riverwall crest and row (3 x cap_cells)
  float* rw_hyd_dev = nullptr;   // hydraulic table, rows of 5
  std::vector<float> rw_hyd;     // host copy of the table
};

static thread_local char g_perr[512] = "";
static agx_status pfail(agx_status c, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_perr, sizeof(g_perr), fmt, ap);
  va_end(ap);
  return c;
}
const char* pool_last_error() { return g_perr; }

#define PCK(call)                                                                                     \
  do {                                                                                                \
    cudaError_t _e = (call);                                                                          \
    if (_e != cudaSuccess) return pfail(AGX_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                                        __FILE__, __LINE__);                                          \
  } while (0)

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t pool_layout(Pool* p, char* base) {
  const size_t C = p->cap_cells, Bt = p->cap_bnd, T = p->cap_tiles, S = p->cap_scn;
  size_t off = 0;
  auto take = [&](size_t b) -> char* { char* r = base ? base + off : nullptr; off += al(b ? b : 8); return r; };
  PoolDev& d = p->d;
  d.conn = (const int4*)take(C * 16);
  d.g0 = (const float4*)take(C * 16);
  d.g1 = (const float4*)take(C * 16);
  d.g2 = (const float4*)take(C * 16);
  d.g3 = (float4*)take(C * 16);
  d.g4 = (float4*)take(C * 16);
  double** dd[] = {&d.wA, &d.uhA, &d.vhA, &d.wB, &d.uhB, &d.vhB, &d.z};
  for (auto q : dd) *q = (double*)take(C * 8);
  d.area = (const double*)take(C * 8);
  d.radius = (const double*)take(C * 8);
  d.eta = (float*)take(C * 4);
  d.W0 = (float4*)take(C * 16);
  d.W1 = (float4*)take(C * 16);
  d.E = (float4*)take(C * 16);
  d.maxs = (float*)take(C * 4);
  d.bkind = (const int*)take(Bt * 4);
  d.bval = (const double*)take(Bt * 24);
  d.bcell = (const int*)take(Bt * 4);
  d.lnk = (const int*)take(C * 4);
  d.tile_halo = (const int2*)take(T * 8);
  d.tile_red1 = (float2*)take(T * 8);
  d.tile_red2 = (float*)take(T * 4);
  d.ctl = (unsigned int*)take(64);
  d.halo_cells = (const int*)take((size_t)p->cap_halo * 4);
  p->tile_scn_dev = (int*)take(T * 4);
  d.scn = (PoolScn*)take(S * sizeof(PoolScn));
  p->staging = (double*)take(C * 8 * 5);
  return off;
}

}  // namespace agx

using namespace agx;

struct agx_pool_s : public agx::Pool {};

static void free_sww(ScnHost& s) {
  if (s.copy_stream) {
    cudaStreamSynchronize(s.copy_stream);
    cudaStreamDestroy(s.copy_stream);
  }
  if (s.sww_off) cudaFree(s.sww_off);
  if (s.sww_slot) cudaFree(s.sww_slot);
  if (s.frame) cudaFree(s.frame);
  if (s.frame_host) cudaFreeHost(s.frame_host);
  if (s.frame_done) cudaEventDestroy(s.frame_done);
  if (s.frame_ready) cudaEventDestroy(s.frame_ready);
  s.sww_off = s.sww_slot = nullptr;
  s.frame = s.frame_host = nullptr;
  s.frame_done = s.frame_ready = nullptr;
  s.copy_stream = nullptr;
  s.sww_P = 0;
}

static agx_status psync(Pool* p) {
  PCK(cudaStreamSynchronize(p->stream));
  return AGX_OK;
}
// Header exchange.  `may_skip`: callers that only read the headers, or
// change them and push them straight back, take the host mirror when no
// header-writing kernel has run since the last exchange.
static agx_status pull_scn(Pool* p, bool may_skip = false) {
  if (may_skip && p->scn_fresh) return AGX_OK;
  p->scn_fresh = false;
  PCK(cudaMemcpyAsync(p->scn_host, p->d.scn, sizeof(PoolScn) * p->cap_scn, cudaMemcpyDeviceToHost, p->stream));
  agx_status st = psync(p);
  p->scn_fresh = st == AGX_OK;
  return st;
}
static agx_status push_scn(Pool* p) {
  p->scn_fresh = false;
  PCK(cudaMemcpyAsync(p->d.scn, p->scn_host, sizeof(PoolScn) * p->cap_scn, cudaMemcpyHostToDevice, p->stream));
  agx_status st = psync(p);
  p->scn_fresh = st == AGX_OK;
  return st;
}

static MParams make_mparams(const agx_params& a) {
  MParams P;
  P.g = (float)a.g;
  P.eps = (float)a.epsilon;
  P.hmin = (float)a.minimum_allowed_height;
  P.hmin64 = a.minimum_allowed_height;
  P.beta_w = (float)a.beta_w;
  P.beta_w_dry = (float)a.beta_w_dry;
  P.beta_uh = (float)a.beta_uh;
  P.beta_uh_dry = (float)a.beta_uh_dry;
  P.beta_vh = (float)a.beta_vh;
  P.beta_vh_dry = (float)a.beta_vh_dry;
  const double c = 1.0 / (0.3 - 0.1);
  P.c_tmp = (float)c;
  P.d_tmp = (float)(1.0 - c * 0.3);
  P.velocity_extrapolation = a.extrapolate_velocity_second_order == 1;
  P.rk2 = a.timestepping_method >= 2;
  P.low_froude = a.low_froude;
  P.rk3 = a.timestepping_method == 3;
  return P;
}

static void init_clock_p(Clock* c, const agx_params& p) {
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

static int nblk1(int n) { return (n + 255) / 256; }

// One step of every active scenario in two parts: the first stage (flux,
// timestep, first update; Euler scenarios are complete after it), then the
// second RK2 stage, the operators of the step loop and the clocks.
// With the pool's L2 option on, the kernels launched next on `st` keep the
// work records `rec` of the used cells resident in L2 (persisting accesses
// up to the device's persisting size; the rest stream).  rec null: no window.
// Kernels captured into the step graph take the stream's window with them.
static void set_l2_window(Pool* p, cudaStream_t st, const void* rec) {
  if (!p->l2_window && rec) return;
  cudaStreamAttrValue v = {};
  if (rec && p->l2_window_max > 0) {
    const size_t bytes = std::min((size_t)p->d.ntiles * TILE * 16, p->l2_window_max);
    v.accessPolicyWindow.base_ptr = const_cast<void*>(rec);
    v.accessPolicyWindow.num_bytes = bytes;
    v.accessPolicyWindow.hitRatio = bytes ? (float)std::min(1.0, (double)p->l2_persist_max / (double)bytes) : 0.0f;
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  } else {
    v.accessPolicyWindow.num_bytes = 0;
  }
  cudaStreamSetAttribute(st, cudaStreamAttributeAccessPolicyWindow, &v);
}

static cudaError_t enqueue_first_stage(Pool* p, cudaStream_t st) {
  const PoolDev& d = p->d;
  p->scn_fresh = false;
  const int S = p->cap_scn;
  k_pool_reset<<<nblk1(S), 256, 0, st>>>(d, S);
  count_launch();
  const int Gf = p->grid_mode == 1 ? std::max(d.ntiles, 1) : p->grid_v[p->variant];
  set_l2_window(p, st, d.W0);
  if (p->rw_any || p->rare_bc_any) k_pool_flux<1, 6, true><<<Gf, TILE, 0, st>>>(d);
  else if (p->variant == 0) k_pool_flux<1, 6><<<Gf, TILE, 0, st>>>(d);
  else k_pool_flux<1, 8><<<Gf, TILE, 0, st>>>(d);
  count_launch();
  phase_mark(st, PH_FLUX);
  set_l2_window(p, st, d.W1);        // the update writes the records stage 2 gathers
  k_pool_timestep<<<nblk1(S), 256, 0, st>>>(d, S);
  count_launch();
  phase_mark(st, PH_SMALL);
  // RK2 scenarios: update1 into B + flux2 fused; Euler scenarios only update.
  // Both forms are handled by the same kernels with the per-scenario flag:
  // the update kernel is launched once per form.
  k_pool_update<<<std::max(d.ntiles, 1), TILE, 0, st>>>(d, 0);
  count_launch();
  phase_mark(st, PH_UPDATE);
  if (p->l2_window) set_l2_window(p, st, nullptr);
  return cudaGetLastError();
}

// Flux kernel of stage 2 or 3 (stage 3 only when some scenario has three).
static cudaError_t enqueue_later_stage(Pool* p, cudaStream_t st, int stage) {
  const PoolDev& d = p->d;
  p->scn_fresh = false;
  const int Gf = p->grid_mode == 1 ? std::max(d.ntiles, 1) : p->grid_v[p->variant];
  if (stage == 3 && !p->rk3_any) return cudaSuccess;
  set_l2_window(p, st, stage == 3 ? (const void*)d.W2 : (const void*)d.W1);
  if (stage == 2) {
    if (p->rw_any || p->rare_bc_any) k_pool_flux<2, 6, true><<<Gf, TILE, 0, st>>>(d);
    else if (p->variant == 0) k_pool_flux<2, 6><<<Gf, TILE, 0, st>>>(d);
    else k_pool_flux<2, 8><<<Gf, TILE, 0, st>>>(d);
    if (p->rk3_any) {
      count_launch();
      if (p->rw_any || p->rare_bc_any) k_pool_flux<4, 6, true><<<Gf, TILE, 0, st>>>(d);
      else if (p->variant == 0) k_pool_flux<4, 6><<<Gf, TILE, 0, st>>>(d);
      else k_pool_flux<4, 8><<<Gf, TILE, 0, st>>>(d);
    }
  } else {
    if (p->rw_any || p->rare_bc_any) k_pool_flux<3, 6, true><<<Gf, TILE, 0, st>>>(d);
    else if (p->variant == 0) k_pool_flux<3, 6><<<Gf, TILE, 0, st>>>(d);
    else k_pool_flux<3, 8><<<Gf, TILE, 0, st>>>(d);
  }
  count_launch();
  phase_mark(st, PH_FLUX);
  if (p->l2_window) set_l2_window(p, st, nullptr);
  return cudaGetLastError();
}

// The operators of the step loop and the clocks.
static cudaError_t enqueue_step_end(Pool* p, cudaStream_t st, unsigned long long h, bool set_cond) {
  const PoolDev& d = p->d;
  p->scn_fresh = false;
  const int S = p->cap_scn;
  for (size_t s = 0; s < p->scn.size(); s++) {
    const ScnHost& sh = p->scn[s];
    if (!sh.alive || sh.host_ops) continue;
    for (size_t i = 0; i < sh.ops.size(); i++) {
      const PoolOp& op = sh.ops[i];
      if (op.kind == 1) k_pool_inlet<<<1, INLET_TPB, 0, st>>>(d, op, (int)i, op.rate, op.rate, 0);
      else k_pool_rate<<<nblk1(op.n), 256, 0, st>>>(d, op, (int)i, 0);
      count_launch();
      phase_mark(st, PH_RATE);
    }
  }
  k_pool_clock<<<1, 1024, 0, st>>>(d, S, (cudaGraphConditionalHandle)h, set_cond ? 1 : 0);
  count_launch();
  phase_mark(st, PH_SMALL);
  return cudaGetLastError();
}

// The one-kernel step serves pools whose scenarios take one or two stages,
// without riverwalls, boundary kinds 7-10 or inlets in the step loop.
static bool step_kernel_ok(const Pool* p) {
  if (p->rk3_any || p->rw_any || p->rare_bc_any) return false;
  for (const ScnHost& sh : p->scn) {
    if (!sh.alive || sh.host_ops) continue;
    for (const PoolOp& op : sh.ops) if (op.kind != 0) return false;
  }
  return true;
}

// Device table of the step loop's rate operators (rebuilt with the graph).
static agx_status build_step_ops(Pool* p) {
  std::vector<StepOp> v;
  for (size_t s = 0; s < p->scn.size(); s++) {
    const ScnHost& sh = p->scn[s];
    if (!sh.alive || sh.host_ops) continue;
    for (size_t i = 0; i < sh.ops.size(); i++) v.push_back(StepOp{sh.ops[i], (int)i, 0});
  }
  if (p->step_ops) cudaFree(p->step_ops);
  p->step_ops = nullptr;
  p->step_nops = (int)v.size();
  if (v.empty()) return AGX_OK;
  PCK(cudaMalloc(&p->step_ops, v.size() * sizeof(StepOp)));
  PCK(cudaMemcpyAsync(p->step_ops, v.data(), v.size() * sizeof(StepOp), cudaMemcpyHostToDevice, p->stream));
  return psync(p);
}

static cudaError_t enqueue_step_kernel(Pool* p, cudaStream_t st, unsigned long long h, bool set_cond) {
  p->scn_fresh = false;
  const int G = std::max(1, std::min(p->step_grid[p->variant], std::max(p->d.ntiles, 1)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(TILE);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const StepOp* ops = p->step_ops;
  const int nops = p->step_nops, nscn = p->cap_scn, sc = set_cond ? 1 : 0;
  const cudaGraphConditionalHandle hh = (cudaGraphConditionalHandle)h;
  cudaError_t e = p->variant == 0 ? cudaLaunchKernelEx(&cfg, k_pool_step<6>, p->d, ops, nops, nscn, hh, sc)
                                  : cudaLaunchKernelEx(&cfg, k_pool_step<8>, p->d, ops, nops, nscn, hh, sc);
  count_launch();
  phase_mark(st, PH_FLUX);
  return e;
}

static cudaError_t enqueue_pool_iter(Pool* p, cudaStream_t st, unsigned long long h, bool set_cond) {
  if (p->grid_mode == 2 && step_kernel_ok(p) && set_cond) return enqueue_step_kernel(p, st, h, set_cond);
  cudaError_t e = enqueue_first_stage(p, st);
  if (e == cudaSuccess) e = enqueue_later_stage(p, st, 2);
  if (e == cudaSuccess) e = enqueue_later_stage(p, st, 3);
  if (e != cudaSuccess) return e;
  return enqueue_step_end(p, st, h, set_cond);
}

static agx_status pool_build_graph(Pool* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  PCK(cudaGraphCreate(&p->graph, 0));
  cudaGraphConditionalHandle handle;
  PCK(cudaGraphConditionalHandleCreate(&handle, p->graph, 1, cudaGraphCondAssignDefault));
  const bool one_kernel = p->grid_mode == 2 && step_kernel_ok(p);
  cudaGraphNode_t prep = nullptr;
  if (one_kernel) {
    agx_status so = build_step_ops(p);
    if (so) return so;
    // accumulators and barrier words cleared once before the loop
    PoolDev dev = p->d;
    int nscn = p->cap_scn;
    void* args[] = {&dev, &nscn};
    cudaKernelNodeParams kp = {};
    kp.func = (void*)k_pool_step_prepare;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(256);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    PCK(cudaGraphAddKernelNode(&prep, p->graph, nullptr, 0, &kp));
  }
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = handle;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  PCK(cudaGraphAddNode(&node, p->graph, prep ? &prep : nullptr, nullptr, prep ? 1 : 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  PCK(cudaStreamSynchronize(p->stream));
  PCK(cudaStreamBeginCaptureToGraph(p->own_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  set_capturing(true);
  cudaError_t e = enqueue_pool_iter(p, p->own_stream, (unsigned long long)handle, true);
  set_capturing(false);
  cudaGraph_t cap = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(p->own_stream, &cap);
  if (e != cudaSuccess || e2 != cudaSuccess)
    return pfail(AGX_E_CUDA, "pool capture failed: %s / %s", cudaGetErrorString(e), cudaGetErrorString(e2));
  PCK(cudaGraphInstantiate(&p->exec, p->graph, 0));
  size_t nn = 0;
  PCK(cudaGraphGetNodes(body, nullptr, &nn));
  p->kernels_per_iter = (int)nn;
  p->graph_valid = true;
  return AGX_OK;
}

extern "C" {

agx_status agx_pool_create(int64_t cap_cells, int64_t cap_boundary, int32_t cap_scenarios, agx_pool* out) {
  if (!out || cap_cells <= 0 || cap_scenarios <= 0 || cap_boundary < 0)
    return pfail(AGX_E_INVALID, "bad pool capacity");
  *out = nullptr;
  if (cap_cells > (1ll << 30)) return pfail(AGX_E_INVALID, "pool capacity above 2^30 cells");
  agx_pool p = new agx_pool_s();
  PCK(cudaGetDevice(&p->device));
  p->cap_tiles = (int)((cap_cells + TILE - 1) / TILE) + cap_scenarios;
  p->cap_cells = p->cap_tiles * TILE;
  p->cap_bnd = (int)std::max<int64_t>(cap_boundary, 1);
  p->cap_scn = cap_scenarios;
  p->cap_halo = p->cap_cells / 2 + 1024;
  const size_t bytes = pool_layout(p, nullptr);
  cudaError_t e = cudaMalloc(&p->arena, bytes);
  if (e != cudaSuccess) {
    delete p;
    return pfail(AGX_E_NOMEM, "pool allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  p->arena_bytes = bytes;
  pool_layout(p, (char*)p->arena);
  p->d.tile_scn = p->tile_scn_dev;
  p->d.ntiles = 0;
  p->tile_scn.assign(p->cap_tiles, -1);
  p->bnd_owner.assign(p->cap_bnd, -1);
  p->halo_owner.assign(p->cap_halo, -1);
  p->free_tiles.init(p->cap_tiles);
  p->free_bnd.init(p->cap_bnd);
  p->free_halo.init(p->cap_halo);
  p->scn.resize(p->cap_scn);
  PCK(cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking));
  p->stream = p->own_stream;
  PCK(cudaMallocHost(&p->scn_host, sizeof(PoolScn) * p->cap_scn));
  memset(p->scn_host, 0, sizeof(PoolScn) * p->cap_scn);
  PCK(cudaMemsetAsync(p->arena, 0, bytes, p->stream));
  PCK(cudaMemcpyAsync(p->tile_scn_dev, p->tile_scn.data(), p->cap_tiles * 4, cudaMemcpyHostToDevice, p->stream));
  agx_status st = push_scn(p);
  if (st) return st;
  int sms = 0, per = 0, per4 = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pool_flux<1, 6>, TILE, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per4, k_pool_flux<1, 8>, TILE, 0);
  p->grid = std::max(1, sms * std::max(per, 1));
  p->grid_v[0] = p->grid;
  p->grid_v[1] = std::max(1, sms * std::max(per4, 1));
  int ps6 = 0, ps8 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps6, k_pool_step<6>, TILE, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps8, k_pool_step<8>, TILE, 0);
  p->step_grid[0] = sms * std::max(ps6, 0);
  p->step_grid[1] = sms * std::max(ps8, 0);
  *out = p;
  return AGX_OK;
}

int64_t agx_pool_footprint(int64_t cap_cells, int64_t cap_boundary, int32_t cap_scenarios) {
  Pool tmp;
  tmp.cap_tiles = (int)((cap_cells + TILE - 1) / TILE) + cap_scenarios;
  tmp.cap_cells = tmp.cap_tiles * TILE;
  tmp.cap_bnd = (int)std::max<int64_t>(cap_boundary, 1);
  tmp.cap_scn = cap_scenarios;
  tmp.cap_halo = tmp.cap_cells / 2 + 1024;
  return (int64_t)pool_layout(&tmp, nullptr);
}

int64_t agx_pool_bytes_per_cell(void) {
  // static tables + FP64 state (2 buffers) + work records + explicit update
  return 16 * 6 + 8 * 9 + 4 + 16 * 3 + 4 + 8 * 5;
}

agx_status agx_pool_destroy(agx_pool p) {
  if (!p) return AGX_OK;
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (auto& s : p->scn) {
    if (s.order) cudaFree(s.order);
    if (s.inv) cudaFree(s.inv);
    if (s.series) cudaFree(s.series);
    free_sww(s);
    for (auto& op : s.ops) if (op.idx) cudaFree((void*)op.idx);
  }
  if (p->arena) cudaFree(p->arena);
  if (p->snap) cudaFree(p->snap);
  if (p->rw_mem) cudaFree(p->rw_mem);
  if (p->w2_mem) cudaFree(p->w2_mem);
  if (p->step_ops) cudaFree(p->step_ops);
  if (p->rw_hyd_dev) cudaFree(p->rw_hyd_dev);
  if (p->scn_host) cudaFreeHost(p->scn_host);
  if (p->own_stream) cudaStreamDestroy(p->own_stream);
  delete p;
  return AGX_OK;
}

agx_status agx_pool_set_stream(agx_pool p, void* stream) {
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  agx_status st = psync(p);
  if (st) return st;
  p->stream = stream ? (cudaStream_t)stream : p->own_stream;
  return AGX_OK;
}

// Add a scenario.  conn [N*4] (neighbours in the stored order, boundary
// -(m+1), meta word), geo [N*16] floats (g0 g1 g2 g3 blocks: jump matrix,
// edge vectors, radius; dz and inv_area are filled here), area [N], the
// FP64 radius [N] (the timestep quotient of the cell the CFL minimum selects),
// order [N], boundary_cell [B] (stored order), lnk [N] (staging index of
// each slot's neighbour), per tile halo_off/halo_cnt [ceil(N/TILE)] into
// halo_cells [n_halo] (stored cell indices).
agx_status agx_pool_add(agx_pool p, int64_t N, int64_t B, const int32_t* conn, const float* geo,
                        const double* area, const double* radius, const int32_t* order, const int32_t* bcell, const int32_t* lnk,
                        const int32_t* halo_off, const int32_t* halo_cnt, int64_t n_halo,
                        const int32_t* halo_cells, const agx_params* prm, int32_t* sid_out) {
  AGX_TRACE("agx_pool_add");
  if (!p || !conn || !geo || !area || !radius || !order || !prm || !sid_out || !lnk || !halo_off || !halo_cnt || N <= 0 ||
      B < 0 || n_halo < 0)
    return pfail(AGX_E_INVALID, "bad arguments");
  if (prm->timestepping_method < 1 || prm->timestepping_method > 3)
    return pfail(AGX_E_INVALID, "timestepping_method must be 1, 2 or 3");
  int sid = -1;
  for (int s = 0; s < p->cap_scn; s++) if (!p->scn[s].alive) { sid = s; break; }
  if (sid < 0) return pfail(AGX_E_NOMEM, "pool has no free scenario slot");
  if (prm->timestepping_method == 3 && !p->w2_mem) {      // third-stage work records
    PCK(cudaMalloc(&p->w2_mem, (size_t)p->cap_cells * 16));
    p->d.W2 = (float4*)p->w2_mem;
  }
  if (prm->timestepping_method == 3) {
    p->rk3_any = true;
    p->graph_valid = false;
  }
  const int nt = (int)((N + TILE - 1) / TILE);
  const int t0 = (int)p->free_tiles.find(nt);            // first fit: the lowest free run
  if (t0 < 0) return pfail(AGX_E_NOMEM, "pool has no %d free contiguous tiles", nt);
  int b0 = 0;
  if (B > 0) {
    b0 = (int)p->free_bnd.find(B);
    if (b0 < 0) return pfail(AGX_E_NOMEM, "pool has no %lld free boundary slots", (long long)B);
  }
  int h0 = 0;
  if (n_halo > 0) {
    h0 = (int)p->free_halo.find(n_halo);
    if (h0 < 0) return pfail(AGX_E_NOMEM, "pool has no %lld free halo slots", (long long)n_halo);
  }
  for (int t = 0; t < nt; t++) {
    if (halo_cnt[t] < 0 || halo_cnt[t] > HALO_MAX || halo_off[t] < 0 || halo_off[t] + halo_cnt[t] > n_halo)
      return pfail(AGX_E_INVALID, "bad halo table at tile %d", t);
  }
  for (int64_t k = 0; k < N; k++) {
    for (int i = 0; i < 3; i++) {
      const int li = (lnk[k] >> (10 * i)) & 1023;
      if (li != LNK_INLINE && li >= TILE + halo_cnt[k / TILE])
        return pfail(AGX_E_INVALID, "bad staging index at cell %lld", (long long)k);
    }
  }
  const int c0 = t0 * TILE;
  // relocate indices to the pool
  std::vector<int32_t> cc((size_t)N * 4);
  for (int64_t k = 0; k < N; k++) {
    for (int i = 0; i < 3; i++) {
      const int32_t n = conn[4 * k + i];
      if (n >= 0) {
        if (n >= N) return pfail(AGX_E_INVALID, "neighbour index out of range");
        cc[4 * k + i] = n + c0;
      } else {
        const int32_t m = -n - 1;
        if (m >= B) return pfail(AGX_E_INVALID, "boundary index out of range");
        cc[4 * k + i] = -(m + b0) - 1;
      }
    }
    cc[4 * k + 3] = conn[4 * k + 3];
  }
  std::vector<float> G[5];
  for (int g = 0; g < 5; g++) G[g].assign((size_t)N * 4, 0.f);
  for (int64_t k = 0; k < N; k++)
    for (int g = 0; g < 4; g++)
      for (int c = 0; c < 4; c++) G[g][4 * k + c] = geo[16 * k + 4 * g + c];
  for (int64_t k = 0; k < N; k++) G[4][4 * k + 3] = (float)(1.0 / area[k]);
  cudaStream_t st = p->stream;
  PCK(cudaMemcpyAsync((void*)(p->d.conn + c0), cc.data(), N * 16, cudaMemcpyHostToDevice, st));
  const float4* gd[5] = {p->d.g0, p->d.g1, p->d.g2, p->d.g3, p->d.g4};
  for (int g = 0; g < 5; g++) PCK(cudaMemcpyAsync((void*)(gd[g] + c0), G[g].data(), N * 16, cudaMemcpyHostToDevice, st));
  PCK(cudaMemcpyAsync((void*)(p->d.area + c0), area, N * 8, cudaMemcpyHostToDevice, st));
  PCK(cudaMemcpyAsync((void*)(p->d.radius + c0), radius, N * 8, cudaMemcpyHostToDevice, st));
  PCK(cudaMemcpyAsync((void*)(p->d.lnk + c0), lnk, N * 4, cudaMemcpyHostToDevice, st));
  {
    std::vector<int2> th(nt);
    for (int t = 0; t < nt; t++) th[t] = make_int2(halo_off[t] + h0, halo_cnt[t]);
    PCK(cudaMemcpyAsync((void*)(p->d.tile_halo + t0), th.data(), nt * 8, cudaMemcpyHostToDevice, st));
    if (n_halo > 0) {
      std::vector<int32_t> hc(n_halo);
      for (int64_t h = 0; h < n_halo; h++) {
        if (halo_cells[h] < 0 || halo_cells[h] >= N) return pfail(AGX_E_INVALID, "halo cell out of range");
        hc[h] = halo_cells[h] + c0;
      }
      PCK(cudaMemcpyAsync((void*)(p->d.halo_cells + h0), hc.data(), n_halo * 4, cudaMemcpyHostToDevice, st));
      PCK(cudaStreamSynchronize(st));
    }
  }
  ScnHost& sh = p->scn[sid];
  sh = ScnHost();
  PCK(cudaMalloc(&sh.order, N * 4));
  PCK(cudaMemcpyAsync(sh.order, order, N * 4, cudaMemcpyHostToDevice, st));
  {
    std::vector<int32_t> iv((size_t)N, -1);
    for (int64_t j = 0; j < N; j++) {
      if (order[j] < 0 || order[j] >= N || iv[order[j]] >= 0) return pfail(AGX_E_INVALID, "order is not a permutation");
      iv[order[j]] = (int32_t)j;
    }
    PCK(cudaMalloc(&sh.inv, N * 4));
    PCK(cudaMemcpyAsync(sh.inv, iv.data(), N * 4, cudaMemcpyHostToDevice, st));
    PCK(cudaStreamSynchronize(st));
  }
  if (B > 0) {
    std::vector<int32_t> bc(B);
    for (int64_t m = 0; m < B; m++) bc[m] = bcell[m] + c0;
    PCK(cudaMemcpyAsync((void*)(p->d.bcell + b0), bc.data(), B * 4, cudaMemcpyHostToDevice, st));
    PCK(cudaMemsetAsync((void*)(p->d.bkind + b0), 0, B * 4, st));
    PCK(cudaMemsetAsync((void*)(p->d.bval + 3 * (size_t)b0), 0, B * 24, st));
  }
  // zero the scenario's dynamic arrays
  double* zd[] = {p->d.wA, p->d.uhA, p->d.vhA, p->d.wB, p->d.uhB, p->d.vhB, p->d.z};
  for (double* a : zd) PCK(cudaMemsetAsync(a + c0, 0, (size_t)nt * TILE * 8, st));
  PCK(cudaMemsetAsync(p->d.eta + c0, 0, (size_t)nt * TILE * 4, st));
  PCK(cudaMemsetAsync(p->d.W0 + c0, 0, (size_t)nt * TILE * 16, st));
  PCK(cudaMemsetAsync(p->d.W1 + c0, 0, (size_t)nt * TILE * 16, st));
  PCK(cudaMemsetAsync(p->d.E + c0, 0, (size_t)nt * TILE * 16, st));
  PCK(cudaMemsetAsync(p->d.maxs + c0, 0, (size_t)nt * TILE * 4, st));
  for (int t = t0; t < t0 + nt; t++) p->tile_scn[t] = sid;
  for (int b = b0; b < b0 + B; b++) p->bnd_owner[b] = sid;
  for (int h = h0; h < h0 + n_halo; h++) p->halo_owner[h] = sid;
  p->free_tiles.take(t0, nt);
  if (B > 0) p->free_bnd.take(b0, B);
  if (n_halo > 0) p->free_halo.take(h0, n_halo);
  const int ntiles = (int)p->free_tiles.used_end();
  PCK(cudaMemcpyAsync(p->tile_scn_dev + t0, p->tile_scn.data() + t0, (size_t)nt * 4, cudaMemcpyHostToDevice, st));
  agx_status s2 = pull_scn(p);
  if (s2) return s2;
  PoolScn& S = p->scn_host[sid];
  memset(&S, 0, sizeof(S));
  init_clock_p(&S.clock, *prm);
  S.P = make_mparams(*prm);
  S.cell0 = c0;
  S.ncell = (int)N;
  S.tile0 = t0;
  S.ntile = nt;
  S.bnd0 = b0;
  S.nbnd = (int)B;
  S.alive = 1;
  S.active = 0;
  if ((s2 = push_scn(p))) return s2;
  sh.alive = 1;
  sh.N = (int)N;
  sh.B = (int)B;
  sh.tile0 = t0;
  sh.ntile = nt;
  sh.bnd0 = b0;
  sh.halo0 = h0;
  sh.nhalo = (int)n_halo;
  sh.prm = *prm;
  sh.work_dirty = true;
  if (ntiles != p->d.ntiles) {
    p->d.ntiles = ntiles;
    p->graph_valid = false;
  }
  *sid_out = sid;
  return AGX_OK;
}

agx_status agx_pool_remove(agx_pool p, int32_t sid) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  agx_status st = pull_scn(p);
  if (st) return st;
  ScnHost& sh = p->scn[sid];
  for (int t = sh.tile0; t < sh.tile0 + sh.ntile; t++) p->tile_scn[t] = -1;
  for (int b = sh.bnd0; b < sh.bnd0 + sh.B; b++) p->bnd_owner[b] = -1;
  for (int h = sh.halo0; h < sh.halo0 + sh.nhalo; h++) p->halo_owner[h] = -1;
  p->free_tiles.give(sh.tile0, sh.ntile);
  p->free_bnd.give(sh.bnd0, sh.B);
  p->free_halo.give(sh.halo0, sh.nhalo);
  PCK(cudaMemcpyAsync(p->tile_scn_dev + sh.tile0, p->tile_scn.data() + sh.tile0, (size_t)sh.ntile * 4,
                      cudaMemcpyHostToDevice, p->stream));
  p->scn_host[sid].alive = 0;
  p->scn_host[sid].active = 0;
  if ((st = push_scn(p))) return st;
  if (sh.order) cudaFree(sh.order);
  if (sh.inv) cudaFree(sh.inv);
  if (sh.series) cudaFree(sh.series);
  free_sww(sh);
  bool had_ops = !sh.ops.empty();
  for (auto& op : sh.ops) if (op.idx) cudaFree((void*)op.idx);
  sh = ScnHost();
  const int ntiles = (int)p->free_tiles.used_end();
  if (ntiles != p->d.ntiles || had_ops) {
    p->d.ntiles = ntiles;
    p->graph_valid = false;
  }
  return AGX_OK;
}

static agx_status ensure_work(Pool* p, int sid) {
  ScnHost& sh = p->scn[sid];
  if (!sh.work_dirty) return AGX_OK;
  k_pool_prep<<<p->grid, TILE, 0, p->stream>>>(p->d, 0, sid);   // writes the work records only
  count_launch();
  PCK(cudaGetLastError());
  sh.work_dirty = false;
  return AGX_OK;
}

// Field access in the caller's (original) cell order.
agx_status agx_pool_set_field(agx_pool p, int32_t sid, int32_t f, const double* host, int64_t n) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  if (n != sh.N) return pfail(AGX_E_INVALID, "field needs %d values", sh.N);
  const int c0 = sh.tile0 * TILE;
  double* dst = nullptr;
  switch (f) {
    case AGX_STAGE_C: dst = p->d.wA; break;
    case AGX_XMOM_C: dst = p->d.uhA; break;
    case AGX_YMOM_C: dst = p->d.vhA; break;
    case AGX_ELEV_C: dst = p->d.z; break;
    case AGX_FRICTION_C: break;
    default: return pfail(AGX_E_STATE, "field %d cannot be set on a mixed-precision scenario", f);
  }
  PCK(cudaMemcpyAsync(p->staging, host, n * 8, cudaMemcpyHostToDevice, p->stream));
  if (f == AGX_FRICTION_C) {
    k_gather_f<<<nblk1((int)n), 256, 0, p->stream>>>(p->d.eta + c0, p->staging, sh.order, (int)n);
  } else if (f == AGX_STAGE_C) {       // the pool keeps the depth stage - bed
    k_gather_depth<<<nblk1((int)n), 256, 0, p->stream>>>(p->d.wA + c0, p->d.z + c0, p->staging, sh.order, (int)n);
  } else if (f == AGX_ELEV_C) {        // a new bed keeps the stage
    k_gather_bed<<<nblk1((int)n), 256, 0, p->stream>>>(p->d.wA + c0, p->d.z + c0, p->staging, sh.order, (int)n);
  } else {
    k_gather<<<nblk1((int)n), 256, 0, p->stream>>>(dst + c0, p->staging, sh.order, (int)n);
  }
  count_launch();
  if (f == AGX_ELEV_C) {
    k_pool_dz<<<p->grid, TILE, 0, p->stream>>>(p->d, sid);
    count_launch();
  }
  PCK(cudaGetLastError());
  sh.work_dirty = true;
  return psync(p);
}

__global__ void k_gather3(double* w, double* uh, double* vh, const double* z, const double* src, const int* order,
                          int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const int o = order[j];
    w[j] = src[o] - z[j];
    uh[j] = src[(size_t)n + o];
    vh[j] = src[2 * (size_t)n + o];
  }
}
__global__ void k_scatter3(double* dst, const double* w, const double* uh, const double* vh, const double* z,
                           const int* order, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const int o = order[j];
    dst[o] = w[j] + z[j];
    dst[(size_t)n + o] = uh[j];
    dst[2 * (size_t)n + o] = vh[j];
  }
}

// Page-locked host memory the device can address at the same virtual
// address (cudaPointerGetAttributes: host memory with a device pointer equal
// to the host pointer).  Kernels then read or write it directly over the
// host link; other (pageable) buffers go through copies.
static bool host_mapped(const void* ptr) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer == ptr;
}

// Direct exchange with mapped host buffers, walked in the caller's order
// (contiguous on the host side; permuted on the device side).  The read also
// writes each cell's work record (the k_pool_prep pass without in-place
// protection), so the next step needs no separate pass over the state.
__global__ void k_state_from_host(double* w, double* uh, double* vh, const double* z, float4* W0,
                                  const double* area, const PoolScn* S, const double* hw, const double* huh,
                                  const double* hvh, const int* inv, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < n) {
    const int j = inv[o];
    double h = hw[o] - z[j], u = huh[o], v = hvh[o];
    w[j] = h;
    uh[j] = u;
    vh[j] = v;
    double added;
    W0[j] = protect_prep(S->P, h, u, v, area[j], added);
  }
}
__global__ void k_state_to_host(double* hw, double* huh, double* hvh, const double* w, const double* uh,
                                const double* vh, const double* z, const int* inv, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < n) {
    const int j = inv[o];
    hw[o] = w[j] + z[j];
    huh[o] = uh[j];
    hvh[o] = vh[j];
  }
}

// The conserved state (stage, xmomentum, ymomentum) in the caller's cell
// order, in one call with one synchronisation: read by one kernel straight
// from page-locked host buffers, or else three copies through the staging
// buffer and one permutation kernel.
agx_status agx_pool_set_state(agx_pool p, int32_t sid, const double* w, const double* uh, const double* vh, int64_t n) {
  AGX_TRACE("agx_pool_set_state");
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || !w || !uh || !vh)
    return pfail(AGX_E_INVALID, "bad arguments");
  ScnHost& sh = p->scn[sid];
  if (n != sh.N) return pfail(AGX_E_INVALID, "the state has %d cells", sh.N);
  const int c0 = sh.tile0 * TILE;
  cudaStream_t st = p->stream;
  if (host_mapped(w) && host_mapped(uh) && host_mapped(vh)) {
    k_state_from_host<<<nblk1((int)n), 256, 0, st>>>(p->d.wA + c0, p->d.uhA + c0, p->d.vhA + c0, p->d.z + c0,
                                                    p->d.W0 + c0, p->d.area + c0, p->d.scn + sid, w, uh, vh,
                                                    sh.inv, (int)n);
    count_launch();
    PCK(cudaGetLastError());
    sh.work_dirty = false;
    return psync(p);
  }
  PCK(cudaMemcpyAsync(p->staging, w, n * 8, cudaMemcpyHostToDevice, st));
  PCK(cudaMemcpyAsync(p->staging + n, uh, n * 8, cudaMemcpyHostToDevice, st));
  PCK(cudaMemcpyAsync(p->staging + 2 * n, vh, n * 8, cudaMemcpyHostToDevice, st));
  k_gather3<<<nblk1((int)n), 256, 0, st>>>(p->d.wA + c0, p->d.uhA + c0, p->d.vhA + c0, p->d.z + c0, p->staging,
                                           sh.order, (int)n);
  count_launch();
  PCK(cudaGetLastError());
  sh.work_dirty = true;
  return psync(p);
}

agx_status agx_pool_get_state(agx_pool p, int32_t sid, double* w, double* uh, double* vh, int64_t n) {
  AGX_TRACE("agx_pool_get_state");
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || !w || !uh || !vh)
    return pfail(AGX_E_INVALID, "bad arguments");
  ScnHost& sh = p->scn[sid];
  if (n != sh.N) return pfail(AGX_E_INVALID, "the state has %d cells", sh.N);
  const int c0 = sh.tile0 * TILE;
  cudaStream_t st = p->stream;
  if (host_mapped(w) && host_mapped(uh) && host_mapped(vh)) {
    k_state_to_host<<<nblk1((int)n), 256, 0, st>>>(w, uh, vh, p->d.wA + c0, p->d.uhA + c0, p->d.vhA + c0,
                                                  p->d.z + c0, sh.inv, (int)n);
    count_launch();
    PCK(cudaGetLastError());
    return psync(p);
  }
  k_scatter3<<<nblk1((int)n), 256, 0, st>>>(p->staging, p->d.wA + c0, p->d.uhA + c0, p->d.vhA + c0, p->d.z + c0,
                                            sh.order, (int)n);
  count_launch();
  PCK(cudaGetLastError());
  PCK(cudaMemcpyAsync(w, p->staging, n * 8, cudaMemcpyDeviceToHost, st));
  PCK(cudaMemcpyAsync(uh, p->staging + n, n * 8, cudaMemcpyDeviceToHost, st));
  PCK(cudaMemcpyAsync(vh, p->staging + 2 * n, n * 8, cudaMemcpyDeviceToHost, st));
  return psync(p);
}

agx_status agx_pool_get_field(agx_pool p, int32_t sid, int32_t f, double* host, int64_t n) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  const int N = sh.N;
  const int c0 = sh.tile0 * TILE;
  const bool edge = f >= AGX_STAGE_E && f <= AGX_HEIGHT_V;
  if (n != (edge ? 3 * (int64_t)N : N)) return pfail(AGX_E_INVALID, "field size mismatch");
  double* out = p->staging;
  cudaStream_t st = p->stream;
  switch (f) {
    case AGX_STAGE_C: k_scatter_stage<<<nblk1(N), 256, 0, st>>>(out, p->d.wA + c0, p->d.z + c0, sh.order, N); break;
    case AGX_XMOM_C: k_scatter<<<nblk1(N), 256, 0, st>>>(out, p->d.uhA + c0, sh.order, N); break;
    case AGX_YMOM_C: k_scatter<<<nblk1(N), 256, 0, st>>>(out, p->d.vhA + c0, sh.order, N); break;
    case AGX_ELEV_C: k_scatter<<<nblk1(N), 256, 0, st>>>(out, p->d.z + c0, sh.order, N); break;
    case AGX_FRICTION_C: k_scatter_f<<<nblk1(N), 256, 0, st>>>(out, p->d.eta + c0, sh.order, N); break;
    case AGX_HEIGHT_C: k_scatter_height<<<nblk1(N), 256, 0, st>>>(out, p->d.wA + c0, sh.order, N); break;
    case AGX_MAX_SPEED: k_scatter_f<<<nblk1(N), 256, 0, st>>>(out, p->d.maxs + c0, sh.order, N); break;
    case AGX_STAGE_X: case AGX_XMOM_X: case AGX_YMOM_X:
      k_scatter_E<<<nblk1(N), 256, 0, st>>>(out, p->d.E + c0, f - AGX_STAGE_X, sh.order, N); break;
    default:
      if (edge) {
        agx_status s2 = ensure_work(p, sid);
        if (s2) return s2;
        double* tmp = nullptr;
        PCK(cudaMalloc(&tmp, (size_t)15 * N * 8));
        double* we = tmp;
        double* he = we + 3 * (size_t)N;
        double* uhe = he + 3 * (size_t)N;
        double* vhe = uhe + 3 * (size_t)N;
        double* ze = vhe + 3 * (size_t)N;
        k_pool_edges<<<nblk1(N), 256, 0, st>>>(p->d, sid, we, he, uhe, vhe, ze, sh.order);
        count_launch();
        const int idx = (f - AGX_STAGE_E) % 5;     // stage, xmom, ymom, elev, height
        double* src[5] = {we, uhe, vhe, ze, he};
        cudaError_t ce = cudaMemcpyAsync(host, src[idx], 3 * (size_t)N * 8, cudaMemcpyDeviceToHost, st);
        agx_status s3 = psync(p);
        cudaFree(tmp);
        if (ce != cudaSuccess) return pfail(AGX_E_CUDA, "edge export copy failed: %s", cudaGetErrorString(ce));
        if (s3) return s3;
        if (f >= AGX_STAGE_V) {
          // vertex values from edge values on the host
          for (int64_t k = 0; k < N; k++) {
            const double e0 = host[3 * k], e1 = host[3 * k + 1], e2 = host[3 * k + 2];
            host[3 * k] = e1 + e2 - e0;
            host[3 * k + 1] = e0 + e2 - e1;
            host[3 * k + 2] = e0 + e1 - e2;
          }
        }
        return AGX_OK;
      }
      return pfail(AGX_E_STATE, "field %d is not kept by the mixed-precision scenario", f);
  }
  count_launch();
  PCK(cudaGetLastError());
  PCK(cudaMemcpyAsync(host, out, n * 8, cudaMemcpyDeviceToHost, st));
  return psync(p);
}

agx_status agx_pool_set_boundary(agx_pool p, int32_t sid, const int32_t* kind, const double* values, int64_t B) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  if (B != sh.B) return pfail(AGX_E_INVALID, "boundary arrays need %d entries", sh.B);
  if (B == 0) return AGX_OK;
  bool rare = false;
  for (int64_t i = 0; i < B; i++) {
    if (kind[i] < AGX_BC_NONE || kind[i] > AGX_BC_INFLOW)
      return pfail(AGX_E_INVALID, "bad boundary kind %d at %lld", kind[i], (long long)i);
    rare |= kind[i] >= AGX_BC_TRANSMISSIVE_SET_STAGE;
  }
  if (rare && !p->rare_bc_any) {
    p->rare_bc_any = true;
    p->graph_valid = false;
  }
  PCK(cudaMemcpyAsync((void*)(p->d.bkind + sh.bnd0), kind, B * 4, cudaMemcpyHostToDevice, p->stream));
  if (values) PCK(cudaMemcpyAsync((void*)(p->d.bval + 3 * (size_t)sh.bnd0), values, B * 24, cudaMemcpyHostToDevice, p->stream));
  return psync(p);
}

agx_status agx_pool_set_boundary_series(agx_pool p, int32_t sid, const double* rows, int64_t n) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || n < 0) return pfail(AGX_E_INVALID, "bad arguments");
  ScnHost& sh = p->scn[sid];
  agx_status st = psync(p);
  if (st) return st;
  if (sh.series) cudaFree(sh.series);
  sh.series = nullptr;
  if (n > 0) {
    PCK(cudaMalloc(&sh.series, n * 32));
    PCK(cudaMemcpyAsync(sh.series, rows, n * 32, cudaMemcpyHostToDevice, p->stream));
  }
  if ((st = pull_scn(p))) return st;
  p->scn_host[sid].series = sh.series;
  p->scn_host[sid].nseries = (int)n;
  return push_scn(p);
}

// Registers an operator over the caller's cell indices idx[n] (NULL: every
// cell), mapped to pool cells on the host.
static agx_status pool_add_op(Pool* p, int sid, const int32_t* idx, int64_t n, PoolOp op) {
  ScnHost& sh = p->scn[sid];
  if (sh.ops.size() >= (size_t)MAX_OPS) return pfail(AGX_E_INVALID, "at most %d operators", MAX_OPS);
  std::vector<int32_t> ord(sh.N);
  PCK(cudaMemcpyAsync(ord.data(), sh.order, sh.N * 4, cudaMemcpyDeviceToHost, p->stream));
  agx_status st = psync(p);
  if (st) return st;
  std::vector<int32_t> inv(sh.N);
  for (int j = 0; j < sh.N; j++) inv[ord[j]] = j;
  std::vector<int32_t> cells;
  const int c0 = sh.tile0 * TILE;
  if (idx) {
    for (int64_t i = 0; i < n; i++) {
      if (idx[i] < 0 || idx[i] >= sh.N) return pfail(AGX_E_INVALID, "operator index %d out of range", idx[i]);
      cells.push_back(inv[idx[i]] + c0);
    }
  } else {
    for (int j = 0; j < sh.N; j++) cells.push_back(c0 + j);
  }
  op.sid = sid;
  op.idx = nullptr;
  op.n = (int)cells.size();
  if (!cells.empty()) {
    int* dptr = nullptr;
    PCK(cudaMalloc(&dptr, cells.size() * 4));
    PCK(cudaMemcpyAsync(dptr, cells.data(), cells.size() * 4, cudaMemcpyHostToDevice, p->stream));
    op.idx = dptr;
  }
  sh.ops.push_back(op);
  p->graph_valid = false;
  return psync(p);
}

agx_status agx_pool_add_rate(agx_pool p, int32_t sid, const int32_t* idx, int64_t n, double rate, double factor) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  PoolOp op{};
  op.rate = rate;
  op.factor = factor;
  return pool_add_op(p, sid, idx, n, op);
}

agx_status agx_pool_add_inlet(agx_pool p, int32_t sid, const int32_t* idx, int64_t n, double Q, double area,
                              int32_t flags, double velocity_u, double velocity_v) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  if (!idx || n <= 0) return pfail(AGX_E_INVALID, "an inlet needs at least one cell");
  if (n > INLET_MAX) return pfail(AGX_E_INVALID, "an inlet region holds at most %d cells, got %lld", INLET_MAX,
                                  (long long)n);
  if (!(area > 0.0)) return pfail(AGX_E_INVALID, "inlet area must be positive");
  PoolOp op{};
  op.rate = Q;
  op.factor = 1.0;
  op.kind = 1;
  op.flags = flags;
  op.vu = velocity_u;
  op.vv = velocity_v;
  op.area = area;
  return pool_add_op(p, sid, idx, n, op);
}

// Sets (or, with n_riverwall_edges = 0, removes) the wall bits 20 + i of
// the scenario's conn meta words.
__global__ void k_pool_rw_bits(int4* conn, const int* bits, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int4 c = conn[j];
  c.w = (c.w & ~(7 << 20)) | (bits[j] << 20);
  conn[j] = c;
}

agx_status agx_pool_set_riverwalls(agx_pool p, int32_t sid, const int32_t* edge_counter, int64_t n_slots,
                                   int64_t n_riverwall_edges, const double* elevation, const int32_t* row_index,
                                   int32_t n_rows, int32_t ncol, const double* hydraulic) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  if (n_slots != 3 * (int64_t)sh.N) return pfail(AGX_E_INVALID, "edge_counter has %lld slots, the mesh %lld",
                                                 (long long)n_slots, 3 * (long long)sh.N);
  if (n_riverwall_edges < 0 || (n_riverwall_edges > 0 && (!edge_counter || !elevation || !row_index || !hydraulic)) ||
      (n_riverwall_edges > 0 && (n_rows <= 0 || ncol < 5)))
    return pfail(AGX_E_INVALID, "bad riverwall tables (need 5 hydraulic columns: Qfactor s1 s2 h1 h2)");
  for (int64_t s = 0; n_riverwall_edges > 0 && s < n_slots; s++)
    if (edge_counter[s] < 0 || edge_counter[s] > n_riverwall_edges)
      return pfail(AGX_E_INVALID, "riverwall counter %d at slot %lld out of range", edge_counter[s], (long long)s);
  for (int64_t r = 0; r < n_riverwall_edges; r++)
    if (row_index[r] < 0 || row_index[r] >= n_rows) return pfail(AGX_E_INVALID, "riverwall row index out of range");
  agx_status st = psync(p);
  if (st) return st;
  const size_t C3 = 3 * (size_t)p->cap_cells;
  const size_t b_crest = (C3 * 8 + 255) & ~(size_t)255;
  if (!p->rw_mem && n_riverwall_edges > 0) {
    PCK(cudaMalloc(&p->rw_mem, b_crest + C3 * 4));
    PCK(cudaMemsetAsync(p->rw_mem, 0, b_crest + C3 * 4, p->stream));
    p->d.rw_crest = (const double*)p->rw_mem;
    p->d.rw_row = (const int*)((char*)p->rw_mem + b_crest);
  }
  // hydraulic rows of this call appended to the pool's table
  const int row0 = (int)(p->rw_hyd.size() / 5);
  for (int r = 0; r < n_rows && n_riverwall_edges > 0; r++)
    for (int c = 0; c < 5; c++) p->rw_hyd.push_back((float)hydraulic[(size_t)r * ncol + c]);
  if (n_riverwall_edges > 0) {
    if (p->rw_hyd_dev) cudaFree(p->rw_hyd_dev);
    p->rw_hyd_dev = nullptr;
    PCK(cudaMalloc(&p->rw_hyd_dev, p->rw_hyd.size() * 4));
    PCK(cudaMemcpyAsync(p->rw_hyd_dev, p->rw_hyd.data(), p->rw_hyd.size() * 4, cudaMemcpyHostToDevice, p->stream));
    p->d.rw_hyd = p->rw_hyd_dev;
  }
  // per stored cell: wall bits, crest and row of each wall slot
  std::vector<int32_t> ord(sh.N);
  PCK(cudaMemcpyAsync(ord.data(), sh.order, sh.N * 4, cudaMemcpyDeviceToHost, p->stream));
  if ((st = psync(p))) return st;
  std::vector<int> bits(sh.N, 0);
  std::vector<double> crest(3 * (size_t)sh.N, 0.0);
  std::vector<int32_t> row(3 * (size_t)sh.N, 0);
  bool any = false;
  for (int j = 0; j < sh.N && n_riverwall_edges > 0; j++)
    for (int i = 0; i < 3; i++) {
      const int r = edge_counter[3 * (size_t)ord[j] + i];
      if (r <= 0) continue;
      bits[j] |= 1 << i;
      crest[3 * (size_t)j + i] = elevation[r - 1];
      row[3 * (size_t)j + i] = row0 + row_index[r - 1];
      any = true;
    }
  const int c0 = sh.tile0 * TILE;
  int* bits_dev = nullptr;
  PCK(cudaMalloc(&bits_dev, sh.N * 4));
  PCK(cudaMemcpyAsync(bits_dev, bits.data(), sh.N * 4, cudaMemcpyHostToDevice, p->stream));
  k_pool_rw_bits<<<nblk1(sh.N), 256, 0, p->stream>>>((int4*)p->d.conn + c0, bits_dev, sh.N);
  count_launch();
  PCK(cudaGetLastError());
  if (p->rw_mem) {
    PCK(cudaMemcpyAsync((void*)(p->d.rw_crest + 3 * (size_t)c0), crest.data(), crest.size() * 8,
                        cudaMemcpyHostToDevice, p->stream));
    PCK(cudaMemcpyAsync((void*)(p->d.rw_row + 3 * (size_t)c0), row.data(), row.size() * 4, cudaMemcpyHostToDevice,
                        p->stream));
  }
  st = psync(p);
  cudaFree(bits_dev);
  if (st) return st;
  if (any) p->rw_any = true;
  p->graph_valid = false;
  return AGX_OK;
}

agx_status agx_pool_operators_from_host(agx_pool p, int32_t sid, int32_t on) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  if (p->scn[sid].host_ops != (on != 0)) p->graph_valid = false;
  p->scn[sid].host_ops = on != 0;
  return AGX_OK;
}

agx_status agx_pool_apply_operator(agx_pool p, int32_t sid, int32_t op, double rate, double factor,
                                   double timestep) {
  AGX_TRACE("agx_pool_apply_operator");
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  if (op < 0 || op >= (int)sh.ops.size() || !(timestep >= 0.0))
    return pfail(AGX_E_INVALID, "bad operator %d or timestep", op);
  agx_status st = ensure_work(p, sid);
  if (st) return st;
  PoolOp o = sh.ops[op];
  o.dt = timestep;
  p->scn_fresh = false;
  if (o.n > 0) {
    if (o.kind == 1) {
      k_pool_inlet<<<1, INLET_TPB, 0, p->stream>>>(p->d, o, op, rate, factor, 1);
    } else {
      o.rate = rate;
      o.factor = factor;
      k_pool_rate<<<nblk1(o.n), 256, 0, p->stream>>>(p->d, o, op, 1);
    }
    count_launch();
    PCK(cudaGetLastError());
  }
  return psync(p);
}

agx_status agx_pool_clear_operators(agx_pool p, int32_t sid) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  agx_status st = psync(p);
  if (st) return st;
  for (auto& op : p->scn[sid].ops) if (op.idx) cudaFree((void*)op.idx);
  p->scn[sid].ops.clear();
  p->graph_valid = false;
  return AGX_OK;
}

// distribute_to_vertices_and_edges for one scenario (protect in place,
// surrounded-dry zeroing, fresh work record).
agx_status agx_pool_distribute(agx_pool p, int32_t sid) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  p->scn_fresh = false;
  k_pool_prep<<<p->grid, TILE, 0, p->stream>>>(p->d, 1, sid);
  k_pool_sdry<<<p->grid, TILE, 0, p->stream>>>(p->d, sid);
  k_pool_prep<<<p->grid, TILE, 0, p->stream>>>(p->d, 0, sid);
  count_launch(3);
  PCK(cudaGetLastError());
  p->scn[sid].work_dirty = false;
  return psync(p);
}

agx_status agx_pool_set_clock(agx_pool p, int32_t sid, double time, double yield_time, double final_time,
                              int64_t max_steps) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  agx_status st = pull_scn(p, true);
  if (st) return st;
  Clock& c = p->scn_host[sid].clock;
  c.time = time;
  c.yield_time = yield_time;
  c.final_time = final_time;
  c.steps_target = max_steps > 0 ? max_steps : 0;
  c.steps_call = 0;
  c.reason = 0;
  c.recorded_min = p->scn[sid].prm.evolve_max_timestep;
  c.recorded_max = p->scn[sid].prm.evolve_min_timestep;
  p->scn_host[sid].active = 1;
  p->scn[sid].running = true;
  return push_scn(p);
}

agx_status agx_pool_deactivate(agx_pool p, int32_t sid) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  agx_status st = pull_scn(p, true);
  if (st) return st;
  p->scn_host[sid].active = 0;
  return push_scn(p);
}

static void fill_stats_p(const Clock* c, agx_step_stats* o) {
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

// Advance every active scenario until each reaches its yield time, final
// time or step target.  One graph launch (device-side while loop).
agx_status agx_pool_advance(agx_pool p, int32_t* n_done) {
  AGX_TRACE("agx_pool_advance");
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn[s].alive) { agx_status st = ensure_work(p, s); if (st) return st; }
  agx_status st = pull_scn(p, true);
  if (st) return st;
  int nact = 0;
  for (int s = 0; s < p->cap_scn; s++) if (p->scn_host[s].alive && p->scn_host[s].active) nact++;
  if (nact == 0) { if (n_done) *n_done = 0; return AGX_OK; }
  if (!p->graph_valid && (st = pool_build_graph(p)) != AGX_OK) return st;
  p->scn_fresh = false;
  PCK(cudaGraphLaunch(p->exec, p->stream));
  if ((st = pull_scn(p))) return st;
  long long iters = 0;
  int done = 0;
  for (int s = 0; s < p->cap_scn; s++) {
    if (!p->scn_host[s].alive) continue;
    iters = std::max(iters, p->scn_host[s].clock.steps_call);
    if (p->scn_host[s].clock.reason) done++;
  }
  count_launch(iters * p->kernels_per_iter);
  if (n_done) *n_done = done;
  return AGX_OK;
}

// One step split at the RK2 stages, without the graph (boundary values the
// host evaluates at the second stage's time go in between).
agx_status agx_pool_step_begin(agx_pool p) {
  AGX_TRACE("agx_pool_step_begin");
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn[s].alive) { agx_status st = ensure_work(p, s); if (st) return st; }
  PCK(enqueue_first_stage(p, p->stream));
  p->stages_done = 1;
  return psync(p);
}

agx_status agx_pool_step_stage(agx_pool p, int32_t stage) {
  AGX_TRACE("agx_pool_step_stage");
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  if (stage != p->stages_done + 1 || stage < 2 || stage > 3)
    return pfail(AGX_E_STATE, "stage %d out of order (stage %d ran last)", stage, p->stages_done);
  PCK(enqueue_later_stage(p, p->stream, stage));
  p->stages_done = stage;
  return psync(p);
}

agx_status agx_pool_step_end(agx_pool p, int32_t* n_done) {
  AGX_TRACE("agx_pool_step_end");
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  if (p->stages_done < 1) return pfail(AGX_E_STATE, "agx_pool_step_begin has not run");
  for (int stage = p->stages_done + 1; stage <= 3; stage++) PCK(enqueue_later_stage(p, p->stream, stage));
  p->stages_done = 0;
  PCK(enqueue_step_end(p, p->stream, 0ull, false));
  agx_status st = pull_scn(p);
  if (st) return st;
  int done = 0;
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn_host[s].alive && p->scn_host[s].clock.reason) done++;
  if (n_done) *n_done = done;
  return AGX_OK;
}

agx_status agx_pool_sww_bind(agx_pool p, int32_t sid, int64_t P, const int32_t* node_offsets,
                             const int32_t* node_slots) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  const int64_t S3 = 3 * (int64_t)sh.N;
  if (P < 0 || (P > 0 && (!node_offsets || !node_slots))) return pfail(AGX_E_INVALID, "bad arguments");
  if (node_offsets[0] != 0 || node_offsets[P] != S3) return pfail(AGX_E_INVALID, "node offsets must run from 0 to 3N");
  for (int64_t q = 0; q < P; q++)
    if (node_offsets[q + 1] < node_offsets[q]) return pfail(AGX_E_INVALID, "node offsets must not decrease");
  for (int64_t q = 0; q < S3; q++)
    if (node_slots[q] < 0 || node_slots[q] >= S3) return pfail(AGX_E_INVALID, "vertex slot out of range");
  agx_status st = psync(p);
  if (st) return st;
  free_sww(sh);
  const size_t fbytes = ((size_t)3 * P + (size_t)S3) * 4 + 4;
  PCK(cudaMalloc(&sh.sww_off, (size_t)(P + 1) * 4));
  PCK(cudaMalloc(&sh.sww_slot, (size_t)S3 * 4 + 4));
  PCK(cudaMalloc(&sh.frame, fbytes));
  PCK(cudaMallocHost(&sh.frame_host, fbytes));
  PCK(cudaEventCreateWithFlags(&sh.frame_done, cudaEventDisableTiming));
  PCK(cudaEventCreateWithFlags(&sh.frame_ready, cudaEventDisableTiming));
  PCK(cudaStreamCreateWithFlags(&sh.copy_stream, cudaStreamNonBlocking));
  sh.sww_P = (int)P;
  PCK(cudaMemcpyAsync(sh.sww_off, node_offsets, (size_t)(P + 1) * 4, cudaMemcpyHostToDevice, p->stream));
  PCK(cudaMemcpyAsync(sh.sww_slot, node_slots, (size_t)S3 * 4, cudaMemcpyHostToDevice, p->stream));
  return psync(p);
}

agx_status agx_pool_sww_frame_async(agx_pool p, int32_t sid, double min_storable_height, int32_t centroid_averaging) {
  AGX_TRACE("agx_pool_sww_frame_async");
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  ScnHost& sh = p->scn[sid];
  if (!sh.frame) return pfail(AGX_E_STATE, "agx_pool_sww_bind first");
  agx_status st = ensure_work(p, sid);
  if (st) return st;
  cudaStream_t s = p->stream;
  // the frame kernels wait for the previous frame's copy to leave the buffer;
  // the copy runs on its own stream, so the steps enqueued next overlap it
  PCK(cudaStreamWaitEvent(s, sh.frame_done, 0));
  if (sh.sww_P > 0) {
    k_pool_sww_nodes<<<nblk1(sh.sww_P), 256, 0, s>>>(p->d, sid, sh.sww_P, sh.sww_off, sh.sww_slot, sh.inv,
                                                    min_storable_height, centroid_averaging ? 1 : 0, sh.frame);
    count_launch();
  }
  k_pool_sww_cells<<<nblk1(sh.N), 256, 0, s>>>(p->d, sid, sh.order, sh.frame + 3 * (size_t)sh.sww_P);
  count_launch();
  PCK(cudaGetLastError());
  PCK(cudaEventRecord(sh.frame_ready, s));
  PCK(cudaStreamWaitEvent(sh.copy_stream, sh.frame_ready, 0));
  PCK(cudaMemcpyAsync(sh.frame_host, sh.frame, ((size_t)3 * sh.sww_P + 3 * (size_t)sh.N) * 4,
                      cudaMemcpyDeviceToHost, sh.copy_stream));
  PCK(cudaEventRecord(sh.frame_done, sh.copy_stream));
  return AGX_OK;
}

agx_status agx_pool_sww_frame_wait(agx_pool p, int32_t sid, const float** vertex, const float** centroid) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || !vertex || !centroid)
    return pfail(AGX_E_INVALID, "bad arguments");
  ScnHost& sh = p->scn[sid];
  if (!sh.frame_host) return pfail(AGX_E_STATE, "agx_pool_sww_bind first");
  PCK(cudaEventSynchronize(sh.frame_done));
  *vertex = sh.frame_host;
  *centroid = sh.frame_host + 3 * (size_t)sh.sww_P;
  return AGX_OK;
}

agx_status agx_pool_set_fixed_flux_timestep(agx_pool p, int32_t sid, double flux_timestep) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive) return pfail(AGX_E_INVALID, "bad scenario");
  if (!(flux_timestep >= 0.0)) return pfail(AGX_E_INVALID, "flux_timestep needs to be greater than 0.0");
  agx_status st = pull_scn(p, true);
  if (st) return st;
  p->scn_host[sid].clock.fixed_flux_dt = flux_timestep;
  return push_scn(p);
}

agx_status agx_pool_get_stats(agx_pool p, int32_t sid, agx_step_stats* out) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || !out) return pfail(AGX_E_INVALID, "bad scenario");
  agx_status st = pull_scn(p, true);
  if (st) return st;
  fill_stats_p(&p->scn_host[sid].clock, out);
  const int e = p->scn_host[sid].clock.error;
  if (e & ERR_BARRIER)
    return pfail(AGX_E_TIMEOUT, "a grid barrier of the one-kernel step ran out of waiting; the step loop of scenario "
                 "%d stopped", sid);
  if (e & ERR_NONFINITE)
    return pfail(AGX_E_NUMERIC, "non-finite conserved quantity (NaN or Inf) in %lld cell updates of scenario %d; "
                 "its step loop stopped", (long long)p->scn_host[sid].clock.nonfinite_cells, sid);
  if (e & ERR_NUMERIC) return pfail(AGX_E_NUMERIC, "non-positive semi-implicit denominator");
  if (e & ERR_TIMESTEP) return pfail(AGX_E_TIMESTEP, "too small timestep at first order");
  if (e & ERR_NAN) return pfail(AGX_E_NUMERIC, "non-finite or non-positive timestep (state diverged)");
  if (e & ERR_OVERSHOOT) return pfail(AGX_E_OVERSHOOT, "time overshot finaltime");
  if (e & ERR_STEPCAP) return pfail(AGX_E_STATE, "device loop hit the per-call step cap");
  return AGX_OK;
}

agx_status agx_pool_operator_influx(agx_pool p, int32_t sid, int32_t op, double* v) {
  if (!p || sid < 0 || sid >= p->cap_scn || !p->scn[sid].alive || op < 0 || op >= MAX_OPS || !v)
    return pfail(AGX_E_INVALID, "bad arguments");
  agx_status st = pull_scn(p, true);
  if (st) return st;
  *v = p->scn_host[sid].clock.op_influx[op];
  return AGX_OK;
}

// Per-kernel event timing of `reps` iterations (direct launches).
agx_status agx_pool_time_phases(agx_pool p, int32_t reps, double* ms, int32_t n_cat) {
  if (!p || !ms || reps <= 0 || n_cat < PH_COUNT) return pfail(AGX_E_INVALID, "bad arguments");
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn[s].alive) { agx_status st = ensure_work(p, s); if (st) return st; }
  agx_status st0 = pull_scn(p);
  if (st0) return st0;
  std::vector<PoolScn> saved(p->scn_host, p->scn_host + p->cap_scn);
  for (int s = 0; s < p->cap_scn; s++) {
    if (!p->scn_host[s].alive) continue;
    p->scn_host[s].active = 1;
    p->scn_host[s].clock.yield_time = 1.0e300;
    p->scn_host[s].clock.final_time = -1.0;
    p->scn_host[s].clock.steps_target = 0;
  }
  if ((st0 = push_scn(p))) return st0;
  for (int i = 0; i < n_cat; i++) ms[i] = 0.0;
  cudaEvent_t start;
  cudaEventCreate(&start);
  for (int r = 0; r < reps; r++) {
    begin_phase_timer();
    cudaEventRecord(start, p->stream);
    cudaError_t e = enqueue_pool_iter(p, p->stream, 0ull, false);
    if (e != cudaSuccess) { end_phase_timer(nullptr, 0, start, 1); return pfail(AGX_E_CUDA, "%s", cudaGetErrorString(e)); }
    PCK(cudaStreamSynchronize(p->stream));
    end_phase_timer(ms, reps, start, 0);
  }
  cudaEventDestroy(start);
  // restore activity and the clock targets (the state itself has advanced)
  if ((st0 = pull_scn(p))) return st0;
  for (int s = 0; s < p->cap_scn; s++) {
    if (!p->scn_host[s].alive) continue;
    p->scn_host[s].active = saved[s].active;
    p->scn_host[s].clock.yield_time = saved[s].clock.yield_time;
    p->scn_host[s].clock.final_time = saved[s].clock.final_time;
    p->scn_host[s].clock.steps_target = saved[s].clock.steps_target;
  }
  return push_scn(p);
}

int32_t agx_pool_grid(agx_pool p) { return p ? p->grid : 0; }

// Keep the work records the flux kernels gather resident in L2 (1) or not
// (0).  The first time it is switched on, the context's persisting L2 size is
// set to the device's maximum (a limit of this process's context only).
agx_status agx_pool_set_l2_window(agx_pool p, int32_t on) {
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  agx_status st = psync(p);
  if (st) return st;
  if (on && p->l2_window_max == 0) {
    int persist = 0, window = 0;
    PCK(cudaDeviceGetAttribute(&persist, cudaDevAttrMaxPersistingL2CacheSize, p->device));
    PCK(cudaDeviceGetAttribute(&window, cudaDevAttrMaxAccessPolicyWindowSize, p->device));
    if (persist <= 0 || window <= 0) return pfail(AGX_E_STATE, "this device has no persisting L2");
    PCK(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)persist));
    p->l2_persist_max = (size_t)persist;
    p->l2_window_max = (size_t)window;
  }
  if ((on != 0) != (p->l2_window != 0)) p->graph_valid = false;
  p->l2_window = on ? 1 : 0;
  if (!on) set_l2_window(p, p->stream, nullptr);
  return AGX_OK;
}

// Continuous batching: give every running scenario up to max_steps more
// steps (stopping early at its final or yield time) and launch the device
// loop without waiting.  agx_pool_wait completes the call.
agx_status agx_pool_launch_chunk(agx_pool p, int64_t max_steps) {
  AGX_TRACE("agx_pool_launch_chunk");
  if (!p || max_steps <= 0) return pfail(AGX_E_INVALID, "bad arguments");
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn[s].alive && p->scn[s].running) { agx_status st = ensure_work(p, s); if (st) return st; }
  agx_status st = pull_scn(p);
  if (st) return st;
  int nact = 0;
  for (int s = 0; s < p->cap_scn; s++) {
    PoolScn& S = p->scn_host[s];
    if (!p->scn[s].alive || !p->scn[s].running) continue;
    S.clock.steps_call = 0;
    S.clock.steps_target = max_steps;
    S.clock.reason = 0;
    S.active = 1;
    nact++;
  }
  if ((st = push_scn(p))) return st;
  if (nact == 0) return AGX_OK;
  if (!p->graph_valid && (st = pool_build_graph(p)) != AGX_OK) return st;
  p->scn_fresh = false;
  PCK(cudaGraphLaunch(p->exec, p->stream));
  return AGX_OK;
}

// Wait for the launched chunk; scenarios that reached their final time (or
// failed) stop running.  Returns how many are still running.
agx_status agx_pool_wait(agx_pool p, int32_t* n_running) {
  AGX_TRACE("agx_pool_wait");
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  agx_status st = pull_scn(p);
  if (st) return st;
  long long iters = 0;
  int run = 0;
  for (int s = 0; s < p->cap_scn; s++) {
    if (!p->scn[s].alive) continue;
    const Clock& c = p->scn_host[s].clock;
    iters = std::max(iters, c.steps_call);
    if (p->scn[s].running && (c.reason == AGX_STOP_FINAL || c.reason == AGX_STOP_ERROR || c.error))
      p->scn[s].running = false;
    if (p->scn[s].running) run++;
  }
  count_launch(iters * p->kernels_per_iter);
  if (n_running) *n_running = run;
  return AGX_OK;
}

// Statistics of n scenarios with one device read.  running[i] is 1 while the
// scenario still has steps to take.
agx_status agx_pool_stats_all(agx_pool p, int32_t n, const int32_t* sids, agx_step_stats* out, int32_t* running) {
  if (!p || n < 0 || (n && (!sids || !out))) return pfail(AGX_E_INVALID, "bad arguments");
  agx_status st = pull_scn(p);
  if (st) return st;
  for (int i = 0; i < n; i++) {
    const int s = sids[i];
    if (s < 0 || s >= p->cap_scn || !p->scn[s].alive) return pfail(AGX_E_INVALID, "bad scenario %d", s);
    fill_stats_p(&p->scn_host[s].clock, out + i);
    if (running) running[i] = p->scn[s].running ? 1 : 0;
  }
  return AGX_OK;
}

// Free capacity: cells (tile granular), boundary slots, halo slots, scenario slots.
agx_status agx_pool_capacity(agx_pool p, int64_t* free_cells, int64_t* free_boundary, int64_t* free_halo,
                             int32_t* free_scenarios) {
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  const int64_t fc = p->free_tiles.largest(), fb = p->free_bnd.largest(), fh = p->free_halo.largest();
  int fs = 0;
  for (int s = 0; s < p->cap_scn; s++) fs += p->scn[s].alive ? 0 : 1;
  if (free_cells) *free_cells = fc * TILE;
  if (free_boundary) *free_boundary = fb;
  if (free_halo) *free_halo = fh;
  if (free_scenarios) *free_scenarios = fs;
  return AGX_OK;
}

// Kernel variant of the fused flux kernels (0: at most 6 blocks of 128 per
// SM, 1: at most 8) and grid mode (0: persistent, 1: one block per tile, 2:
// the whole step in one cooperative kernel where the pool allows it).
// Chosen by the autotuner.
agx_status agx_pool_set_variant(agx_pool p, int32_t variant, int32_t grid_mode) {
  if (!p || variant < 0 || variant > 1 || grid_mode < 0 || grid_mode > 2) return pfail(AGX_E_INVALID, "bad variant");
  if (p->variant != variant || p->grid_mode != grid_mode) p->graph_valid = false;
  p->variant = variant;
  p->grid_mode = grid_mode;
  return AGX_OK;
}

// Snapshot / restore of every scenario's dynamic state and clock (device to
// device copies into a buffer allocated on the first snapshot).
static agx_status ensure_work(Pool* p, int sid);
static size_t snap_layout(Pool* p, char* base, bool save) {
  const size_t C = p->cap_cells;
  struct Part { void* a; size_t n; } parts[] = {
      {p->d.wA, C * 8}, {p->d.uhA, C * 8}, {p->d.vhA, C * 8}, {p->d.wB, C * 8}, {p->d.uhB, C * 8},
      {p->d.vhB, C * 8}, {p->d.W0, C * 16}, {p->d.W1, C * 16}, {p->d.E, C * 16}, {p->d.maxs, C * 4},
      {p->d.scn, sizeof(PoolScn) * p->cap_scn}};
  size_t off = 0;
  for (auto& q : parts) {
    if (base) {
      if (save) cudaMemcpyAsync(base + off, q.a, q.n, cudaMemcpyDeviceToDevice, p->stream);
      else cudaMemcpyAsync(q.a, base + off, q.n, cudaMemcpyDeviceToDevice, p->stream);
    }
    off += al(q.n);
  }
  return off;
}

agx_status agx_pool_snapshot(agx_pool p) {
  if (!p) return pfail(AGX_E_INVALID, "null pool");
  // pending work records belong to the state being saved
  for (int s = 0; s < p->cap_scn; s++)
    if (p->scn[s].alive) { agx_status st = ensure_work(p, s); if (st) return st; }
  const size_t need = snap_layout(p, nullptr, true);
  if (!p->snap) {
    PCK(cudaMalloc(&p->snap, need));
    p->snap_bytes = need;
  }
  snap_layout(p, (char*)p->snap, true);
  PCK(cudaGetLastError());
  return psync(p);
}

agx_status agx_pool_restore(agx_pool p) {
  if (!p || !p->snap) return pfail(AGX_E_STATE, "no snapshot to restore");
  snap_layout(p, (char*)p->snap, false);
  PCK(cudaGetLastError());
  agx_status st = psync(p);
  if (st) return st;
  return pull_scn(p);
}

int32_t agx_pool_last_error(char* buf, int32_t n) {
  if (buf && n > 0) {
    strncpy(buf, g_perr, (size_t)n - 1);
    buf[n - 1] = 0;
  }
  return (int32_t)strlen(g_perr);
}

}  // extern "C"
