// de_mixed.cuh -- FP32 device math of the mixed-precision DE step.
//
// Same algorithm as the FP64 bodies (de_plain.cuh, which restate
// shallow_water/sw_domain_openmp.c), reformulated on small relative
// quantities so that FP32 keeps its relative precision:
//   * everything is expressed per cell relative to the cell's own bed z_k:
//     the depth h_k = w_k - z_k is formed in FP64 and rounded once, and the
//     stage differences to the neighbours are  dz_kj + (h_j - h_k)  with the
//     static bed differences dz_kj = z_j - z_k (FP64 difference, rounded);
//   * the edge values are jumps from the centroid: stage jump dw, depth h_e,
//     velocity u_e, v_e, and the bed offset z_e - z_k = dw - (h_e - h_k);
//   * the Audusse depths become h_left = max(hle - max(zr - zl, 0), 0) and the
//     stage smoothing term fmax(w_r, z_half) - fmax(w_l, z_half) becomes
//     h_right - h_left;
//   * the linear reconstruction is a 3x3 matrix per cell applied to the
//     differences to the three surrogate neighbours (precomputed from the
//     auxiliary-triangle geometry in FP64).
// The conserved quantities are accumulated in FP64 by the update kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace agx {

struct MParams {            // per-scenario parameters
  float g, eps, hmin;
  float beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
  float c_tmp, d_tmp;
  double hmin64;
  int velocity_extrapolation;
  int rk2;                  // two or more stages (rk2 or rk3)
  int low_froude;
  int rk3;                  // three stages (rk3, DE2)
};

struct EdgeState {          // one edge of one cell, relative to that cell
  float h;                  // depth at the edge (extrapolated)
  float uh, vh;             // momenta at the edge (x/y frame)
  float dz;                 // bed at the edge minus the cell's centroid bed
};

__device__ __forceinline__ float limiter_phi32(const float J[3], float lo, float hi, float beta) {
  const float tiny = 1.0e-30f;
  float r = 1000.0f, cand = 1.0f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if (J[i] < -tiny) cand = lo / J[i];
    if (J[i] > tiny) cand = hi / J[i];
    r = fminf(cand, r);
  }
  return fminf(r * beta, 1.0f);
}

// jumps J = M . D for the three edges and the limiter on [min(0,D), max(0,D)]
__device__ __forceinline__ void limited_jumps(const float M[9], const float D[3], float beta, float out[3]) {
  if (!(beta > 0.0f)) {
    out[0] = out[1] = out[2] = 0.0f;
    return;
  }
  float J[3];
#pragma unroll
  for (int i = 0; i < 3; i++) J[i] = M[3 * i] * D[0] + M[3 * i + 1] * D[1] + M[3 * i + 2] * D[2];
  const float hi = fmaxf(fmaxf(fmaxf(D[0], D[1]), D[2]), 0.0f);
  const float lo = fminf(fminf(fminf(D[0], D[1]), D[2]), 0.0f);
  const float phi = limiter_phi32(J, lo, hi, beta);
#pragma unroll
  for (int i = 0; i < 3; i++) out[i] = J[i] * phi;
}

__device__ __forceinline__ float wet_dry_factor32(const MParams& P, float hc, float hlo, float hhi) {
  float f = fmaxf(0.0f, fminf(P.c_tmp * fmaxf(hlo, 0.0f) / fmaxf(hc, 1.0e-06f) + P.d_tmp,
                              fminf(P.c_tmp * fmaxf(hc, 0.0f) / fmaxf(hhi, 1.0e-06f) + P.d_tmp, 1.0f)));
  f = fminf(1.2f * fmaxf(hlo - P.hmin, 0.0f) / (fmaxf(hlo, 0.0f) + 1.0f * P.hmin), f);
  return f;
}

// Central-upwind flux across one edge (KNP), relative form.  Inputs: left
// and right edge depths (unclamped) and momenta in the x/y frame, d = zr - zl,
// normal (n1, n2); WALL: c = riverwall crest - zl raises the Audusse bed
// z_half to max(zl, zr, crest) (sw_domain_openmp.c:581-588).  Outputs the flux
// in the x/y frame, max speed, pressure flux and the left/right Audusse depths.
struct Flux32 {
  float f0, f1, f2, speed, pflux, hl, hr;
};

template <bool WALL = false>
__device__ __forceinline__ void central_flux32(float hle, float uhl_x, float vhl_x, float hre, float uhr_x,
                                               float vhr_x, float d, float n1, float n2, const MParams& P,
                                               Flux32& F, float c = 0.0f) {
  const float hl = WALL ? fmaxf(hle - fmaxf(fmaxf(d, 0.0f), c), 0.0f) : fmaxf(hle - fmaxf(d, 0.0f), 0.0f);
  const float hr = WALL ? fmaxf(hre - fmaxf(fmaxf(-d, 0.0f), c - d), 0.0f) : fmaxf(hre - fmaxf(-d, 0.0f), 0.0f);
  F.hl = hl;
  F.hr = hr;
  if (hl == 0.0f && hr == 0.0f) {
    F.f0 = F.f1 = F.f2 = 0.0f;
    F.speed = 0.0f;
    F.pflux = 0.0f;
    return;
  }
  float uhl = n1 * uhl_x + n2 * vhl_x;
  float vhl = -n2 * uhl_x + n1 * vhl_x;
  float uhr = n1 * uhr_x + n2 * vhr_x;
  float vhr = -n2 * uhr_x + n1 * vhr_x;
  float ul, vl, ur, vr;
  if (hle > 0.0f) {
    const float inv = 1.0f / hle;
    ul = uhl * inv;
    uhl = hl * ul;
    vl = vhl * inv;
    vhl = hl * inv * vhl;
  } else {
    ul = uhl = vhl = vl = 0.0f;
  }
  if (hre > 0.0f) {
    const float inv = 1.0f / hre;
    ur = uhr * inv;
    uhr = hr * ur;
    vr = vhr * inv;
    vhr = hr * inv * vhr;
  } else {
    ur = uhr = vhr = vr = 0.0f;
  }
  const float cl = sqrtf(P.g * hl);
  const float cr = sqrtf(P.g * hr);
  float fs = 1.0f;
  if (P.low_froude == 1) {
    fs = sqrtf(fmaxf(0.001f, fminf(1.0f, (ur * ur + ul * ul + vr * vr + vl * vl) / (cl * cl + cr * cr + 1.0e-10f))));
  } else if (P.low_froude == 2) {
    fs = sqrtf((ur * ur + ul * ul + vr * vr + vl * vl) / (cl * cl + cr * cr + 1.0e-10f));
    fs = sqrtf(fminf(1.0f, 0.01f + fmaxf(fs - 0.01f, 0.0f)));
  }
  float smax = fmaxf(ul + cl, ur + cr);
  if (smax < 0.0f) smax = 0.0f;
  float smin = fminf(ul - cl, ur - cr);
  if (smin > 0.0f) smin = 0.0f;
  const float span = smax - smin;
  if (span < P.eps) {
    F.f0 = F.f1 = F.f2 = 0.0f;
    F.speed = 0.0f;
    F.pflux = 0.5f * P.g * 0.5f * (hl * hl + hr * hr);
    return;
  }
  F.speed = fmaxf(smax, -smin);
  const float inv_span = 1.0f / fmaxf(span, 1.0e-30f);
  const float ss = smax * smin;
  float f0 = smax * (ul * hl) - smin * (ur * hr);
  f0 += ss * (hr - hl);
  f0 *= inv_span;
  float f1 = smax * (ul * uhl) - smin * (ur * uhr);
  f1 += fs * ss * (uhr - uhl);
  f1 *= inv_span;
  float f2 = smax * (ul * vhl) - smin * (ur * vhr);
  f2 += fs * ss * (vhr - vhl);
  f2 *= inv_span;
  F.pflux = 0.5f * P.g * (smax * hl * hl - smin * hr * hr) * inv_span;
  F.f0 = f0;
  F.f1 = n1 * f1 - n2 * f2;
  F.f2 = n2 * f1 + n1 * f2;
}

// Villemonte weir correction of a riverwall edge's flux (FP32 form of
// __adjust_edgeflux_with_weir, sw_domain_openmp.c:324-426): hl, hr are the
// first-order heads of the two centroids above z_half, hp = Qfactor, s1, s2,
// h1, h2.
__device__ __forceinline__ void weir_adjust32(Flux32& F, float hl, float hr, float g, float weir_height,
                                              const float* hp) {
  const float Qfactor = hp[0], s1 = hp[1], s2 = hp[2], h1 = hp[3], h2 = hp[4];
  const float twothirds = 2.0f / 3.0f;
  if ((hl <= 0.0f) && (hr <= 0.0f)) return;
  const float minhd = fminf(hl, hr);
  const float maxhd = fmaxf(hl, hr);
  float rw = Qfactor * twothirds * maxhd * sqrtf(twothirds * g * maxhd);
  const float rw2 = Qfactor * twothirds * minhd * sqrtf(twothirds * g * minhd);
  const float rwRat = rw2 / fmaxf(rw, 1.0e-30f);
  const float hdRat = minhd / fmaxf(maxhd, 1.0e-30f);
  const float hdWrRat = minhd / fmaxf(weir_height, 1.0e-30f);
  rw = rw * powf(1.0f - rwRat, 0.385f);
  if (hr > hl) rw = -rw;
  if ((hdRat < s2) & (hdWrRat < h2)) {
    const float w1 = fminf(fmaxf(hdRat - s1, 0.0f) / (s2 - s1), 1.0f);
    const float w2 = fminf(fmaxf(hdWrRat - h1, 0.0f) / (h2 - h1), 1.0f);
    const float nf = (rw * (1.0f - w1) + w1 * F.f0) * (1.0f - w2) + w2 * F.f0;
    float sc = (fabsf(F.f0) > 1.0e-30f) ? nf / F.f0 : 0.0f;
    sc = fmaxf(sc, 0.0f);
    F.f0 = nf;
    F.f1 *= fminf(sc, 10.0f);
    F.f2 *= fminf(sc, 10.0f);
  }
  if (fabsf(F.f0) > 0.0f) F.speed = sqrtf(g * (maxhd + weir_height)) + fabsf(F.f0 / (maxhd + 1.0e-12f));
}

}  // namespace agx
