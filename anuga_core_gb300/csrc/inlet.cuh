// Inlet_operator on the device (structures/inlet_operator.py:75-165,
// inlet.py:107-226), shared by the plain FP64 scenario and the pool.
//
// One block of INLET_TPB threads handles an inlet of n <= INLET_MAX cells.
// A positive volume fills the lowest cells first to a level surface (stages
// sorted, cumulative areas and volumes); a negative one lowers all cells to
// one depth, or empties them.  Momenta become depth x the cells' previous
// velocity (or the imposed one, or zero).
//
// The state is reached through an accessor class C with
//   cell(a)            cell index of the inlet's a-th cell
//   stage(k), height(k), area(k), uh(k), vh(k)
//   set_level(k, w)    stage := w
//   set_depth(k, h)    stage := bed + h
//   empty(k)           stage := bed, momenta := 0
//   set_momenta(k, mx, my)
// so that the plain scenario (stage stored) and the pool (depth stored) run
// the same steps on their own layouts.
#pragma once

namespace agx {

constexpr int INLET_TPB = 1024;
constexpr int INLET_PER = INLET_MAX / INLET_TPB;

__device__ __forceinline__ double inlet_warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

__device__ inline double inlet_block_sum(double x, double* part) {
  x = inlet_warp_sum(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = x;
  __syncthreads();
  if (wid == 0) {
    double r = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    r = inlet_warp_sum(r);
    if (lane == 0) part[0] = r;
  }
  __syncthreads();
  const double r = part[0];
  __syncthreads();
  return r;
}

// Exclusive prefix sum of v[0..INLET_MAX) in place (INLET_PER consecutive
// values per thread, then a scan of the per-thread totals).
__device__ inline void inlet_exclusive_scan(double* v, double* part) {
  const int t = threadIdx.x;
  double run = 0.0;
  double loc[INLET_PER];
#pragma unroll
  for (int j = 0; j < INLET_PER; j++) {
    loc[j] = run;
    run += v[t * INLET_PER + j];
  }
  // inclusive scan of the thread totals across the block
  double x = run;
  const int lane = t & 31, wid = t >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) part[wid] = x;
  __syncthreads();
  if (wid == 0) {
    double w = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    part[lane] = w;
  }
  __syncthreads();
  const double before = (wid > 0 ? part[wid - 1] : 0.0) + (x - run);
#pragma unroll
  for (int j = 0; j < INLET_PER; j++) v[t * INLET_PER + j] = before + loc[j];
  __syncthreads();
}

// Applies `volume` (m^3) to the inlet's n cells; returns the volume applied
// (equal to `volume` unless the inlet was emptied), the same in every
// thread.  Ends with a barrier, after which every write is visible to the
// block.
template <class C>
__device__ double inlet_apply(C& c, int n, int flags, double vu, double vv, double inlet_area, double volume) {
  __shared__ double key[INLET_MAX];     // stages, sorted
  __shared__ int pos[INLET_MAX];        // inlet position of each sorted stage
  __shared__ double acc[INLET_MAX];     // cumulative areas / volumes
  __shared__ double part[INLET_TPB / 32];
  __shared__ int last;
  const int t = threadIdx.x;
  double u[INLET_PER], v[INLET_PER], cur = 0.0;
#pragma unroll
  for (int j = 0; j < INLET_PER; j++) {
    const int a = t + j * INLET_TPB;
    u[j] = v[j] = 0.0;
    if (a < n) {
      const int k = c.cell(a);
      const double h = c.height(k);
      cur += h * c.area(k);
      u[j] = c.uh(k) * h / (h * h + 1.0e-6);
      v[j] = c.vh(k) * h / (h * h + 1.0e-6);
      key[a] = c.stage(k);
      pos[a] = a;
    } else {
      key[a] = INFINITY;
      pos[a] = a;
    }
  }
  const double current = inlet_block_sum(cur, part);
  double applied = volume;
  if (volume >= 0.0) {
    // bitonic sort of (stage, position) over INLET_MAX slots
    for (int size = 2; size <= INLET_MAX; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        __syncthreads();
        for (int a = t; a < INLET_MAX; a += INLET_TPB) {
          const int b = a ^ stride;
          if (b > a) {
            const bool up = (a & size) == 0;
            const double ka = key[a], kb = key[b];
            if ((ka > kb) == up) {
              key[a] = kb;
              key[b] = ka;
              const int pa = pos[a];
              pos[a] = pos[b];
              pos[b] = pa;
            }
          }
        }
      }
    }
    __syncthreads();
    // cumulative areas of the cells ordered by stage
    for (int a = t; a < INLET_MAX; a += INLET_TPB) acc[a] = a < n ? c.area(c.cell(pos[a])) : 0.0;
    __syncthreads();
    inlet_exclusive_scan(acc, part);
    double sa[INLET_PER];
#pragma unroll
    for (int j = 0; j < INLET_PER; j++) {
      const int a = t * INLET_PER + j;
      sa[j] = acc[a] + (a < n ? c.area(c.cell(pos[a])) : 0.0);     // inclusive
    }
    __syncthreads();
    // volume needed to fill the cells below sorted position a to its stage
#pragma unroll
    for (int j = 0; j < INLET_PER; j++) {
      const int a = t * INLET_PER + j;
      acc[a] = (a + 1 < n) ? sa[j] * (key[a + 1] - key[a]) : 0.0;
    }
    __syncthreads();
    inlet_exclusive_scan(acc, part);
    if (t == 0) last = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < INLET_PER; j++) {
      const int a = t * INLET_PER + j;
      if (a < n && acc[a] <= volume) atomicMax(&last, a);
    }
    __syncthreads();
    const int index = last;
    // inclusive cumulative area at `index`
    if (t == index / INLET_PER) part[0] = sa[index % INLET_PER];
    __syncthreads();
    const double depth = (volume - acc[index]) / part[0];
    const double level = key[index] + depth;
    for (int a = t; a < n; a += INLET_TPB)
      if (a <= index) c.set_level(c.cell(pos[a]), level);
  } else if (current + volume >= 0.0) {
    const double depth = (current + volume) / inlet_area;
    for (int a = t; a < n; a += INLET_TPB) c.set_depth(c.cell(a), depth);
  } else {
    for (int a = t; a < n; a += INLET_TPB) c.empty(c.cell(a));
    applied = -current;
  }
  __syncthreads();
  if (!(volume < 0.0 && current + volume < 0.0)) {
#pragma unroll
    for (int j = 0; j < INLET_PER; j++) {
      const int a = t + j * INLET_TPB;
      if (a < n) {
        const int k = c.cell(a);
        const double h = c.height(k);
        double mx = h * u[j], my = h * v[j];
        if (flags & 1) { mx = h * vu; my = h * vv; }
        if (flags & 2) { mx = 0.0; my = 0.0; }
        c.set_momenta(k, mx, my);
      }
    }
  }
  __syncthreads();
  return applied;
}

}  // namespace agx
