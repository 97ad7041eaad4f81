// de_plain.cuh -- FP64 bodies of the DE timestep phases (plain form).
//
// Each body works on one cell, one edge or one boundary segment and is
// __host__ __device__ so the same code runs inside the CUDA kernels and in the
// CPU self-check harness.  Arithmetic follows the reference operation by
// operation (compile with --fmad=false / -ffp-contract=off): results are
// bit-identical to the reference's FP64 path on the same inputs.
//
// Reference functions restated (anuga_core paths):
//   protect          shallow_water/sw_domain_openmp.c:1096-1171
//   extrapolation    sw_domain_openmp.c:1336-1952 (+ helpers :1174-1284)
//   edge flux        sw_domain_openmp.c:65-268 (+ weir :324-426)
//   flux accumulation / CFL  sw_domain_openmp.c:456-772
//   Manning friction sw_domain_openmp.c:1954-2034, utilities/util_ext.h:52
//   Quantity.update  abstract_2d_finite_volumes/quantity.c:772-818
//   fix_negative_cells sw_domain_openmp.c:2037-2056
//   boundaries       shallow_water/boundaries.py:235-292,
//                    abstract_2d_finite_volumes/generic_boundary_conditions.py:173-264
//
// Restructurings that keep every result bit-identical:
//   * Each interior edge's central flux is evaluated once and applied to both
//     cells with its sign flipped.  Without fused multiply-add the KNP flux is
//     exactly antisymmetric under (left,right,n) -> (right,left,-n) in IEEE
//     arithmetic, its wave speed and pressure flux are exactly symmetric, and
//     the mesh normals of the two sides are exact negatives; edges for which
//     that does not hold (low-Froude scaling, riverwalls, meshes whose two
//     sides disagree) are evaluated per side.
//   * min_i radius/max(speed_i, eps) over a cell's edges is evaluated as
//     radius / max_i speed_i: correctly rounded division is monotone.
//   * Static geometry the reference recomputes every call (centroid offsets,
//     auxiliary-triangle differentials, 1/area2, 1/area) is computed once on
//     the host with the same operations.
//   * The limiter ratio q/dq and the wet/dry factor are only divided out when
//     a cheap comparison with margin cannot prove the clamp at 1 is active.
//   * Comparisons, minima and maxima of doubles in the extrapolation are made
//     on the integer bit patterns (dlt, dmax, ...): the same outcome as the
//     IEEE comparison for every value that is not a NaN, without using the
//     FP64 pipe, which bounds these kernels.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>
#include "soft64.cuh"

#ifdef __CUDACC__
#define AGX_HD __host__ __device__ __forceinline__
#else
#define AGX_HD inline
#endif

namespace agx {

// ---- FP64 comparisons on the integer pipe ---------------------------------
// For x not NaN, dkey(x) = bits ^ ((bits >> 63) logical>> 1) increases
// strictly with x, except that -0 (key -1) sorts just below +0 (key 0); the
// comparisons treat the two zeros as equal, as IEEE comparison does.  For a
// pair of opposite zeros dmax returns +0 and dmin -0.
AGX_HD int64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
AGX_HD int64_t dkey(double x) {
  const int64_t b = dbits(x);
  return b ^ (int64_t)((uint64_t)(b >> 63) >> 1);
}
AGX_HD bool both_zero(double a, double b) { return ((uint64_t)(dbits(a) | dbits(b)) << 1) == 0; }
AGX_HD bool dlt(double a, double b) { return dkey(a) < dkey(b) && !both_zero(a, b); }
AGX_HD bool dle(double a, double b) { return dkey(a) <= dkey(b) || both_zero(a, b); }
AGX_HD bool dgt(double a, double b) { return dlt(b, a); }
AGX_HD bool dge(double a, double b) { return dle(b, a); }
AGX_HD bool dgt0(double x) { return dbits(x) > 0; }             // x > 0
AGX_HD bool dge0(double x) { return dkey(x) >= -1; }            // x >= 0 (either zero)
AGX_HD bool dle0(double x) { return dkey(x) <= 0; }             // x <= 0
AGX_HD bool dnz(double x) { return ((uint64_t)dbits(x) << 1) != 0; }   // x != 0
AGX_HD double dmax(double a, double b) { return dkey(a) >= dkey(b) ? a : b; }
AGX_HD double dmin(double a, double b) { return dkey(a) <= dkey(b) ? a : b; }

// ---- FP64 division and square root ----------------------------------------
// Correctly rounded either way, so the results are the same bits.
// AGX_INT_DIVSQRT selects, for device code, which of the two are formed with
// integer instructions (soft64.cuh) instead of on the FP64 pipe, which bounds
// the FP64 kernels: bit 0 division, bit 1 square root.  Measured on GB300 (152
// SMs): 115 G divisions/s and 93 G square roots/s on the integer pipes against
// 70 G/s each on the FP64 pipe, and a plain DE1 step of 4.0M triangles
// 8.37 -> 6.63 ms with both (6.79 with division alone, 8.19 with the square
// root alone).
#ifndef AGX_INT_DIVSQRT
#define AGX_INT_DIVSQRT 3
#endif
AGX_HD double ddiv(double a, double b) {
#if defined(__CUDA_ARCH__) && (AGX_INT_DIVSQRT & 1)
  return soft64::div(a, b);
#else
  return a / b;
#endif
}
AGX_HD double dsqrt(double x) {
#if defined(__CUDA_ARCH__) && (AGX_INT_DIVSQRT & 2)
  return soft64::sqrt(x);
#else
  return sqrt(x);
#endif
}

// ---- boundary kinds ------------------------------------------------------
enum BoundaryKind : int {
  BK_NONE = 0,            // segment without a boundary object (values left as they are)
  BK_REFLECTIVE = 1,
  BK_TRANSMISSIVE = 2,    // edge values of the interior cell
  BK_TRANSMISSIVE_C = 3,  // centroid values of the interior cell
  BK_DIRICHLET = 4,       // constant (w, uh, vh)
  BK_TIME_SERIES = 5,     // piecewise-linear table of (t, w, uh, vh)
  BK_TRANSMISSIVE_N0 = 6, // transmissive stage/normal momentum, zero tangential
  BK_TRANSMISSIVE_SET_STAGE = 7,  // stage given, momenta of the edge
  BK_TRANSMISSIVE_ZERO_MOM = 8,   // stage of the edge, momenta zero
  BK_FLATHER = 9,                 // outside stage given, zero outside velocity (characteristics)
  BK_CHARACTERISTIC = 10,         // stage given, momentum of a simple incoming wave (Riemann invariant)
  BK_INFLOW = 11,                 // stage = edge bed + a depth, momenta given
};

// ---- per-cell meta bits (conn.w) -----------------------------------------
// bits 0-5   neighbour_edges of slots 0..2 (2 bits each)
// bit  8     tri_full_flag
// bits 9-11  slot i is evaluated per side (no shared edge flux)
// bits 12-14 surrogate of slot i precedes this cell in the reference order
// bits 16-17 number_of_boundaries
AGX_HD int meta_nedge(int meta, int i) { return (meta >> (2 * i)) & 3; }
AGX_HD int meta_full(int meta) { return (meta >> 8) & 1; }
AGX_HD int meta_nb(int meta) { return (meta >> 16) & 3; }
AGX_HD int meta_before(int meta, int i) { return (meta >> (12 + i)) & 1; }

struct Params {
  double g, epsilon, hmin;      // hmin = minimum_allowed_height
  double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
  double c_tmp, d_tmp;          // wet/dry factor constants (sw_domain_openmp.c:1362-1365)
  int velocity_extrapolation;   // extrapolate_velocity_second_order == 1
  int low_froude;
  int protect_zero_ymom;        // 1: both momenta (sw_domain_orig.c), 0: xmom only (openmp)
  int sloped_mannings;
  // betas at wet/dry factor 1 (beta_dry + (beta - beta_dry) * 1.0) and the
  // reciprocals the limiter needs, formed once by finish_params (0: not
  // positive, divided out per cell)
  double beta_w1, beta_uh1, beta_vh1;
  double inv_beta_w1, inv_beta_uh1, inv_beta_vh1, inv_beta_w;
};

AGX_HD double positive_inverse(double b) { return b > 0.0 ? 1.0 / b : 0.0; }

// Derived parameters, with the device's operations.
AGX_HD void finish_params(Params& P) {
  P.beta_w1 = P.beta_w_dry + (P.beta_w - P.beta_w_dry) * 1.0;
  P.beta_uh1 = P.beta_uh_dry + (P.beta_uh - P.beta_uh_dry) * 1.0;
  P.beta_vh1 = P.beta_vh_dry + (P.beta_vh - P.beta_vh_dry) * 1.0;
  P.inv_beta_w1 = positive_inverse(P.beta_w1);
  P.inv_beta_uh1 = positive_inverse(P.beta_uh1);
  P.inv_beta_vh1 = positive_inverse(P.beta_vh1);
  P.inv_beta_w = positive_inverse(P.beta_w);
}

// ---- protect + depth/velocity preparation --------------------------------
// Combines _openmp_protect (:1096-1171) with the first loop of the
// extrapolation (:1373-1402).  Writes the protected stage, zeroes momenta of
// (near-)dry cells, and the depth and reconstruction variable (velocity or
// momentum).  Returns the mass added by protection.
AGX_HD double prep_cell(const Params& P, int k, double* w, double* uh, double* vh,
                        const double* z, const double* area, double* h, double* u, double* v,
                        bool do_protect = true, bool do_prep = true) {
  double wk = w[k];
  const double zk = z[k];
  double uk = uh[k], vk = vh[k];
  double added = 0.0;
  const double depth = wk - zk;
  if (do_protect && dlt(depth, P.hmin * 1.0)) {
    uk = 0.0;
    if (P.protect_zero_ymom) vk = 0.0;
    if (dle0(depth)) {
      if (dlt(wk, zk)) {
        added = (zk - wk) * area[k];
        wk = zk;
      }
    }
  }
  if (!do_prep) {
    w[k] = wk;
    uh[k] = uk;
    vh[k] = vk;
    return added;
  }
  const double dk = dmax(wk - zk, 0.0);
  double ru = 0.0, rv = 0.0;
  if (dle(dk, P.hmin)) {
    uk = 0.0;
    vk = 0.0;
  } else if (P.velocity_extrapolation) {
    const double inv = ddiv(1.0, dk);
    ru = uk * inv;
    rv = vk * inv;
  } else {
    ru = uk;
    rv = vk;
  }
  w[k] = wk;
  uh[k] = uk;
  vh[k] = vk;
  h[k] = dk;
  u[k] = ru;
  v[k] = rv;
  return added;
}

// ---- limited reconstruction ----------------------------------------------
// __limit_gradient (:1195-1231).  `lo`/`hi` are the admissible jump range.
// min(floor, fl(n_i / d_i)) over the failing slots i (n_i = lo where
// d_i < 0, hi where d_i > 0).  The failing slots are gathered in order
// first, second, third and divided in that order, so that the lanes of a
// warp share one division for their first failing slot whichever slot it is.
AGX_HD double min_failing_ratio(const bool fail[3], const bool neg[3], double lo, double hi,
                                const double jump[3], double floor) {
  const double n0 = neg[0] ? lo : hi, n1 = neg[1] ? lo : hi, n2 = neg[2] ? lo : hi;
  // first failing slot, then the next ones
  const double na = fail[0] ? n0 : (fail[1] ? n1 : n2);
  const double da = fail[0] ? jump[0] : (fail[1] ? jump[1] : jump[2]);
  const bool two = fail[0] ? (fail[1] || fail[2]) : (fail[1] && fail[2]);
  const double nb = (fail[0] && fail[1]) ? n1 : n2;
  const double db = (fail[0] && fail[1]) ? jump[1] : jump[2];
  const bool three = fail[0] && fail[1] && fail[2];
  if (!(fail[0] || fail[1] || fail[2])) return floor;
  double r = dmin(ddiv(na, da), floor);
  if (two) r = dmin(ddiv(nb, db), r);
  if (three) r = dmin(ddiv(n2, jump[2]), r);
  return r;
}

// inv_known > 0 is 1/beta, formed beforehand; otherwise it is divided out.
AGX_HD double limiter_phi(const double jump[3], double lo, double hi, double beta, double inv_known) {
  const double tiny = 1.0e-100;
  // The reference's phi = fmin(fmin(floor, r_0, r_1, r_2) * beta, 1) over the
  // active ratios r_i (lo or hi over jump_i), floor = 1 if slot 0 is
  // inactive, else 1000.  A ratio hi/d with d > tiny satisfies
  // fl(fl(hi/d)*beta) >= 1 whenever hi >= d * (1/beta) * (1 + 2^-40) (the
  // margin dwarfs the three roundings): such a ratio "passes".  A passing
  // ratio can only be the minimum when phi is 1 whichever ratio is taken,
  // so only the failing ratios are divided out; with none failing and
  // floor*beta >= 1, phi is 1 without a division.
  const int64_t kneg = dkey(-tiny), kpos = dkey(tiny);
  bool neg[3], pos[3];
  for (int i = 0; i < 3; i++) {
    const int64_t kj = dkey(jump[i]);
    neg[i] = kj < kneg;            // jump < -tiny
    pos[i] = kj > kpos;            // jump > tiny
  }
  const double ratio_floor = (!neg[0] && !pos[0]) ? 1.0 : 1000.0;
  if (dbits(beta) == dbits(1.0)) {
    // beta 1: fl(fl(r)*1) >= 1 exactly when r >= 1, i.e. hi >= d (d > 0) or
    // lo <= d (d < 0); floor >= 1, so phi is 1 unless a ratio fails
    bool fail[3], any = false;
    for (int i = 0; i < 3; i++) {
      fail[i] = neg[i] ? !dle(lo, jump[i]) : (pos[i] && !dge(hi, jump[i]));
      any |= fail[i];
    }
    if (!any) return 1.0;
    return dmin(min_failing_ratio(fail, neg, lo, hi, jump, ratio_floor), 1.0);
  }
  if (dgt0(beta)) {
    const double inv_beta = dgt0(inv_known) ? inv_known : 1.0 / beta;
    const double need = inv_beta * (1.0 + 9.094947017729282e-13);
    bool fail[3], any = false;
    for (int i = 0; i < 3; i++) {
      // ratio lo/d with both negative: lo/d >= need  <=>  lo <= d*need
      fail[i] = neg[i] ? !dle(lo, jump[i] * need) : (pos[i] && !dge(hi, jump[i] * need));
      any |= fail[i];
    }
    if (!any && dle(inv_beta, ratio_floor)) return dmin(ratio_floor * beta, 1.0);
    return dmin(min_failing_ratio(fail, neg, lo, hi, jump, ratio_floor) * beta, 1.0);
  }
  double r = 1000.0, cand = 1.0;
  for (int i = 0; i < 3; i++) {
    if (neg[i]) cand = lo / jump[i];
    if (pos[i]) cand = hi / jump[i];
    r = dmin(cand, r);
  }
  return dmin(r * beta, 1.0);
}

// Extrapolation geometry of one cell (host-precomputed, same operations as
// sw_domain_openmp.c:1445-1484 / :1684-1696):
//   g[0..2] = edge midpoint x - centroid x,  g[3..5] = same for y
//   nb<=1 : g[6]=dx1 g[7]=dx2 g[8]=dy1 g[9]=dy2 g[10]=1/area2
//   nb==2 : g[6]=gradient factor x, g[7]=gradient factor y
constexpr int GEO_STRIDE = 11;

// Edge values qc + jump * phi (jump * 1 is jump: the product is skipped).
AGX_HD void limited_edges(double qc, const double jump[3], double phi, double out[3]) {
  if (dbits(phi) == dbits(1.0)) {
    for (int i = 0; i < 3; i++) out[i] = qc + jump[i];
  } else {
    for (int i = 0; i < 3; i++) out[i] = qc + jump[i] * phi;
  }
}

// Returns the limiter's phi (1 where the reconstruction is not limited).
AGX_HD double reconstruct3(double beta, double inv_known, double qc, double q0, double q1, double q2,
                           const double* G, double out[3]) {
  if (!dgt0(beta)) {
    out[0] = qc; out[1] = qc; out[2] = qc;
    return 1.0;
  }
  const double d0 = q0 - qc;
  const double d1 = q1 - q0;
  const double d2 = q2 - q0;
  double gx = G[9] * d1 - G[8] * d2;
  gx *= G[10];
  double gy = G[6] * d2 - G[7] * d1;
  gy *= G[10];
  double jump[3];
  for (int i = 0; i < 3; i++) jump[i] = gx * G[i] + gy * G[3 + i];
  const double hi = dmax(dmax(d0, dmax(d0 + d1, d0 + d2)), 0.0);
  const double lo = dmin(dmin(d0, dmin(d0 + d1, d0 + d2)), 0.0);
  const double phi = limiter_phi(jump, lo, hi, beta, inv_known);
  limited_edges(qc, jump, phi, out);
  return phi;
}

AGX_HD void reconstruct_towards(double beta, double inv_known, double qc, double qn, const double* G,
                                double out[3]) {
  const double d = qn - qc;
  const double gx = d * G[6];
  const double gy = d * G[7];
  double jump[3];
  for (int i = 0; i < 3; i++) jump[i] = gx * G[i] + gy * G[3 + i];
  double lo, hi;
  if (dge0(d)) { lo = 0.0; hi = d; } else { lo = d; hi = 0.0; }
  const double phi = limiter_phi(jump, lo, hi, beta, inv_known);
  limited_edges(qc, jump, phi, out);
}

// Wet/dry blending factor (:1537-1551).  In deep water it is exactly 1 and
// is decided by comparisons with margin instead of the three divisions.
AGX_HD double wet_dry_factor(const Params& P, double hc, double hlo, double hhi) {
  const double m = 1.0 + 9.094947017729282e-13;
  const double hc_e = dmax(hc, 1.0e-06);
  const double hhi_e = dmax(hhi, 1.0e-06);
  // A = c*max(hlo,0)/hc_e + d >= 1  <=>  hlo/hc_e >= (1-d)/c = 0.3 (a_tmp)
  // B = c*max(hc,0)/hhi_e + d >= 1 ; C = 1.2*(hlo-hmin)/(hlo+hmin) >= 1
  const bool a1 = dgt0(hlo) && dge(hlo, 0.30000000000000004 * hc_e * m);
  const bool b1 = dge(hc, 0.30000000000000004 * hhi_e * m);
  const bool c1 = dgt0(hlo) && dge(1.2 * (hlo - P.hmin), (hlo + 1.0 * P.hmin) * m);
  if (a1 && b1 && c1) return 1.0;
  // f = max(0, min(A, min(B, 1))), then min(C, f): a term proved >= 1 does
  // not change either minimum, so it is not divided out
  const double bt = b1 ? 1.0 : dmin(ddiv(P.c_tmp * dmax(hc, 0.0), hhi_e) + P.d_tmp, 1.0);
  const double at = a1 ? bt : dmin(ddiv(P.c_tmp * dmax(hlo, 0.0), hc_e) + P.d_tmp, bt);
  double f = dmax(0.0, at);
  if (!c1) f = dmin(ddiv(1.2 * dmax(hlo - P.hmin, 0.0), dmax(hlo, 0.0) + 1.0 * P.hmin), f);
  return f;
}

// "Surrounded by dry cells" test of :1486-1488 for cell s.
AGX_HD bool surrounded_dry(const Params& P, int s, const int4* surr, const double* h) {
  const int4 q = surr[s];
  return (dlt(h[q.x], P.hmin) | (q.x == s)) & (dlt(h[q.y], P.hmin) | (q.y == s)) &
         (dlt(h[q.z], P.hmin) | (q.z == s));
}

struct EdgeOut {       // edge values of one cell, slots 0..2
  double w[3], h[3], uh[3], vh[3], z[3];
};

// Reconstruction value of neighbour s as seen from cell k: the reference's
// in-order loop has already zeroed the velocity of a surrounded-dry cell s
// that precedes k.  Only consulted where that value can matter.
AGX_HD void neighbour_uv(const Params& P, int s, bool before, const int4* surr, const double* h,
                         const double* u, const double* v, double& us, double& vs) {
  us = u[s];
  vs = v[s];
  if (before && (dnz(us) || dnz(vs)) && surrounded_dry(P, s, surr, h)) {
    us = 0.0;
    vs = 0.0;
  }
}

// Main extrapolation loop body (:1418-1896) for cell k.  Returns true if the
// cell's centroid momenta must be zeroed (surrounded by dry cells).  *cls
// (if given) receives the branches the cell took: bits 0-1 the boundary
// class (0: at most one boundary edge, 1: two, 2: three), bit 2 a dry cell,
// bit 3 a wet/dry factor below 1, bits 4-7 a limited stage, height,
// x and y reconstruction.
AGX_HD bool extrap_cell(const Params& P, int k, const int4* conn, const int4* surr, const double* geo,
                        const double* w, const double* h, const double* u, const double* v,
                        EdgeOut& E, int* cls = nullptr) {
  const int4 s = surr[k];
  const int meta = conn[k].w;
  const int nb = meta_nb(meta);
  const double* G = geo + (size_t)GEO_STRIDE * k;
  const double hk = h[k];
  const bool sdry = (dlt(h[s.x], P.hmin) | (s.x == k)) & (dlt(h[s.y], P.hmin) | (s.y == k)) &
                    (dlt(h[s.z], P.hmin) | (s.z == k));
  double uk = u[k], vk = v[k];
  if (sdry) { uk = 0.0; vk = 0.0; }
  int c = (nb == 3 ? 2 : (nb == 2 ? 1 : 0)) | (dlt(hk, P.hmin) ? 4 : 0);
  if (nb == 3) {
    for (int i = 0; i < 3; i++) {
      E.w[i] = w[k]; E.uh[i] = uk; E.vh[i] = vk; E.h[i] = hk;
    }
  } else if (nb <= 1) {
    const double h0 = h[s.x], h1 = h[s.y], h2 = h[s.z];
    const double hlo = dmin(dmin(h0, dmin(h1, h2)), hk);
    const double hhi = dmax(dmax(h0, dmax(h1, h2)), hk);
    const double hf = wet_dry_factor(P, hk, hlo, hhi);
    // at hf == 1 the betas and their reciprocals are the precomputed ones
    const bool one = dbits(hf) == dbits(1.0);
    const double beta = one ? P.beta_w1 : P.beta_w_dry + (P.beta_w - P.beta_w_dry) * hf;
    const double ib = one ? P.inv_beta_w1 : 0.0;
    const double pw = reconstruct3(beta, ib, w[k], w[s.x], w[s.y], w[s.z], G, E.w);
    const double ph = reconstruct3(beta, ib, hk, h0, h1, h2, G, E.h);
    const double beta_u = one ? P.beta_uh1 : P.beta_uh_dry + (P.beta_uh - P.beta_uh_dry) * hf;
    const double beta_v = one ? P.beta_vh1 : P.beta_vh_dry + (P.beta_vh - P.beta_vh_dry) * hf;
    double u0 = u[s.x], u1 = u[s.y], u2 = u[s.z];
    double v0 = v[s.x], v1 = v[s.y], v2 = v[s.z];
    // Neighbour velocities can be stale-zeroed only for a dry cell k (a wet
    // neighbour rules out "surrounded by dry"); they matter only if the dry
    // reconstruction has a positive beta.
    if (dlt(hk, P.hmin) && (dgt0(beta_u) || dgt0(beta_v))) {
      neighbour_uv(P, s.x, meta_before(meta, 0) && s.x != k, surr, h, u, v, u0, v0);
      neighbour_uv(P, s.y, meta_before(meta, 1) && s.y != k, surr, h, u, v, u1, v1);
      neighbour_uv(P, s.z, meta_before(meta, 2) && s.z != k, surr, h, u, v, u2, v2);
      if (s.x == k) { u0 = uk; v0 = vk; }
      if (s.y == k) { u1 = uk; v1 = vk; }
      if (s.z == k) { u2 = uk; v2 = vk; }
    } else {
      if (s.x == k) { u0 = uk; v0 = vk; }
      if (s.y == k) { u1 = uk; v1 = vk; }
      if (s.z == k) { u2 = uk; v2 = vk; }
    }
    const double pu = reconstruct3(beta_u, one ? P.inv_beta_uh1 : 0.0, uk, u0, u1, u2, G, E.uh);
    const double pv = reconstruct3(beta_v, one ? P.inv_beta_vh1 : 0.0, vk, v0, v1, v2, G, E.vh);
    c |= (one ? 0 : 8) | (dbits(pw) != dbits(1.0) ? 16 : 0) | (dbits(ph) != dbits(1.0) ? 32 : 0) |
         (dbits(pu) != dbits(1.0) ? 64 : 0) | (dbits(pv) != dbits(1.0) ? 128 : 0);
  } else {
    int j = 0;
    const int sv[3] = {s.x, s.y, s.z};
    while (j < 2 && sv[j] == k) j++;
    const int kn = sv[j];
    reconstruct_towards(P.beta_w, P.inv_beta_w, w[k], w[kn], G, E.w);
    reconstruct_towards(P.beta_w, P.inv_beta_w, hk, h[kn], G, E.h);
    double un, vn;
    neighbour_uv(P, kn, meta_before(meta, j) != 0, surr, h, u, v, un, vn);
    reconstruct_towards(P.beta_w, P.inv_beta_w, uk, un, G, E.uh);
    reconstruct_towards(P.beta_w, P.inv_beta_w, vk, vn, G, E.vh);
  }
  if (P.velocity_extrapolation) {
    for (int i = 0; i < 3; i++) {
      const double dk = E.h[i];
      E.uh[i] = E.uh[i] * dk;
      E.vh[i] = E.vh[i] * dk;
    }
  }
  for (int i = 0; i < 3; i++) E.z[i] = E.w[i] - E.h[i];
  if (cls) *cls = c;
  return sdry;
}

AGX_HD void vertex_from_edges(const double e[3], double vx[3]) {
  vx[0] = e[1] + e[2] - e[0];
  vx[1] = e[0] + e[2] - e[1];
  vx[2] = e[0] + e[1] - e[2];
}

// ---- central flux ---------------------------------------------------------
struct FluxOut {
  double f[3];       // edge flux in the x/y frame, before the -length scaling
  double speed;      // max wave speed
  double pflux;      // pressure flux
};

AGX_HD void central_flux(const double ql[3], const double qr[3], double hl, double hr,
                         double hle, double hre, double n1, double n2, double eps, double ze,
                         double g, int low_froude, FluxOut& F) {
  if (!dnz(hl) && !dnz(hr)) {
    F.f[0] = F.f[1] = F.f[2] = 0.0;
    F.speed = 0.0;
    F.pflux = 0.0;
    return;
  }
  const double wl = ql[0], wr = qr[0];
  double uhl = n1 * ql[1] + n2 * ql[2];
  double vhl = -n2 * ql[1] + n1 * ql[2];
  double uhr = n1 * qr[1] + n2 * qr[2];
  double vhr = -n2 * qr[1] + n1 * qr[2];
  double ul, vl, ur, vr;
  if (dgt0(hle)) {
    const double inv = ddiv(1.0, hle);
    ul = uhl * inv;
    uhl = hl * ul;
    vl = vhl * inv;
    vhl = hl * inv * vhl;
  } else {
    ul = uhl = vhl = vl = 0.0;
  }
  if (dgt0(hre)) {
    const double inv = ddiv(1.0, hre);
    ur = uhr * inv;
    uhr = hr * ur;
    vr = vhr * inv;
    vhr = hr * inv * vhr;
  } else {
    ur = uhr = vhr = vr = 0.0;
  }
  const double cl = dsqrt(g * hl);
  const double cr = dsqrt(g * hr);
  double fs = 1.0;
  if (low_froude == 1) {
    fs = dsqrt(fmax(0.001, fmin(1.0, ddiv(ur * ur + ul * ul + vr * vr + vl * vl, cl * cl + cr * cr + 1.0e-10))));
  } else if (low_froude == 2) {
    fs = dsqrt(ddiv(ur * ur + ul * ul + vr * vr + vl * vl, cl * cl + cr * cr + 1.0e-10));
    fs = dsqrt(fmin(1.0, 0.01 + fmax(fs - 0.01, 0.0)));
  }
  double smax = dmax(ul + cl, ur + cr);
  if (dkey(smax) < -1) smax = 0.0;          // smax < 0
  double smin = dmin(ul - cl, ur - cr);
  if (dgt0(smin)) smin = 0.0;
  const double span = smax - smin;
  if (dlt(span, eps)) {
    F.f[0] = F.f[1] = F.f[2] = 0.0;
    F.speed = 0.0;
    F.pflux = 0.5 * g * 0.5 * (hl * hl + hr * hr);
    return;
  }
  F.speed = dmax(smax, -smin);
  const double inv_span = ddiv(1.0, dmax(span, 1.0e-100));
  const double fl0 = ul * hl, fl1 = ul * uhl, fl2 = ul * vhl;
  const double fr0 = ur * hr, fr1 = ur * uhr, fr2 = ur * vhr;
  double f0 = smax * fl0 - smin * fr0;
  f0 += (smax * smin) * (dmax(wr, ze) - dmax(wl, ze));
  f0 *= inv_span;
  double f1 = smax * fl1 - smin * fr1;
  f1 += fs * (smax * smin) * (uhr - uhl);
  f1 *= inv_span;
  double f2 = smax * fl2 - smin * fr2;
  f2 += fs * (smax * smin) * (vhr - vhl);
  f2 *= inv_span;
  F.pflux = 0.5 * g * (smax * hl * hl - smin * hr * hr) * inv_span;
  const double m2 = -n2;
  F.f[0] = f0;
  F.f[1] = n1 * f1 + m2 * f2;
  F.f[2] = -m2 * f1 + n1 * f2;
}

AGX_HD void weir_adjust(FluxOut& F, double hl, double hr, double g, double weir_height,
                        const double* hp) {
  const double Qfactor = hp[0], s1 = hp[1], s2 = hp[2], h1 = hp[3], h2 = hp[4];
  const double twothirds = 2.0 / 3.0;
  if ((hl <= 0.0) && (hr <= 0.0)) return;
  const double minhd = fmin(hl, hr);
  const double maxhd = fmax(hl, hr);
  double rw = Qfactor * twothirds * maxhd * sqrt(twothirds * g * maxhd);
  const double rw2 = Qfactor * twothirds * minhd * sqrt(twothirds * g * minhd);
  const double rwRat = rw2 / fmax(rw, 1.0e-100);
  const double hdRat = minhd / fmax(maxhd, 1.0e-100);
  const double hdWrRat = minhd / fmax(weir_height, 1.0e-100);
  rw = rw * pow(1.0 - rwRat, 0.385);
  if (hr > hl) rw *= -1.0;
  if ((hdRat < s2) & (hdWrRat < h2)) {
    const double w1 = fmin(fmax(hdRat - s1, 0.0) / (s2 - s1), 1.0);
    const double w2 = fmin(fmax(hdWrRat - h1, 0.0) / (h2 - h1), 1.0);
    const double nf = (rw * (1.0 - w1) + w1 * F.f[0]) * (1.0 - w2) + w2 * F.f[0];
    double sc = (fabs(F.f[0]) > 1.0e-100) ? nf / F.f[0] : 0.0;
    sc = fmax(sc, 0.0);
    F.f[0] = nf;
    F.f[1] *= fmin(sc, 10.0);
    F.f[2] *= fmin(sc, 10.0);
  }
  if (fabs(F.f[0]) > 0.0) F.speed = sqrt(g * (maxhd + weir_height)) + fabs(F.f[0] / (maxhd + 1.0e-12));
}

struct Riverwall {       // riverwall tables (all null when there are none)
  const int* counter;    // [3N] edge_river_wall_counter (1-based), 0 = ordinary edge
  const double* elevation;
  const int* row;        // riverwall_rowIndex
  const double* hyd;     // hydraulic properties, ncol per row
  int ncol;
};

// Left state of slot ki of cell k against its neighbour (or boundary value).
struct SlotResult {
  double f[3], speed, pflux, hleft;
};

// Flux across slot ki (cell k, edge i), evaluated from cell k's side
// (:536-653).  Also returns h_right (the neighbour side's Audusse depth).
AGX_HD void slot_flux(const Params& P, int k, int i, const int4& c, const double* we, const double* uhe,
                      const double* vhe, const double* ze, const double* he, const double* wb,
                      const double* uhb, const double* vhb, const double* normals, const double* wc,
                      const double* hc_arr, const double* zc_arr, const Riverwall& RW, SlotResult& R,
                      double& h_right) {
  const int ki = 3 * k + i;
  const double ql[3] = {we[ki], uhe[ki], vhe[ki]};
  const double zl = ze[ki];
  const double hle = he[ki];
  const int n = (i == 0) ? c.x : (i == 1) ? c.y : c.z;
  double qr[3], zr, hre;
  double hc_n = hc_arr[k];
  double zc_n = zc_arr[k];
  if (n < 0) {
    const int m = -n - 1;
    qr[0] = wb[m]; qr[1] = uhb[m]; qr[2] = vhb[m];
    zr = zl;
    hre = dmax(qr[0] - zr, 0.0);
  } else {
    hc_n = hc_arr[n];
    zc_n = zc_arr[n];
    const int nm = 3 * n + meta_nedge(c.w, i);
    qr[0] = we[nm]; qr[1] = uhe[nm]; qr[2] = vhe[nm];
    zr = ze[nm];
    hre = he[nm];
  }
  double z_half = dmax(zl, zr);
  int rw_id = RW.counter ? RW.counter[ki] : 0;
  if (rw_id > 0) z_half = fmax(RW.elevation[rw_id - 1], z_half);
  const double hl = dmax(hle + zl - z_half, 0.0);
  const double hr = dmax(hre + zr - z_half, 0.0);
  FluxOut F;
  central_flux(ql, qr, hl, hr, hle, hre, normals[2 * ki], normals[2 * ki + 1], P.epsilon, z_half,
               P.g, P.low_froude, F);
  if (rw_id > 0) {
    const double* hp = RW.hyd + (size_t)RW.row[rw_id - 1] * RW.ncol;
    const double wh = fmax(RW.elevation[rw_id - 1] - fmin(zl, zr), 0.0);
    const double hlt = fmax(wc[k] - z_half, 0.0);
    const double hrt = (n >= 0) ? fmax(wc[n] - z_half, 0.0) : fmax(hc_n + zr - z_half, 0.0);
    if (RW.elevation[rw_id - 1] > fmax(zc_arr[k], zc_n)) weir_adjust(F, hlt, hrt, P.g, wh, hp);
  }
  R.f[0] = F.f[0]; R.f[1] = F.f[1]; R.f[2] = F.f[2];
  R.speed = F.speed;
  R.pflux = F.pflux;
  R.hleft = hl;
  h_right = hr;
}

// Per-cell accumulation of the three slot results (:655-717).
struct CellFlux {
  double ew, euh, evh;   // explicit updates (already divided by area)
  double smax;           // max qualifying wave speed (0 if none)
  double bflux;          // contribution to boundary_flux_sum
};

AGX_HD void accum_cell(const Params& P, int k, const int4& c, const SlotResult R[3], const double* he,
                       const double* ze, const double* hc_arr, const double* zc_arr,
                       const double* normals, const double* lengths, double inv_area,
                       const int* full_of_neighbour, CellFlux& out) {
  double sw = 0.0, sx = 0.0, sy = 0.0, smax = 0.0, bflux = 0.0;
  const double hc = hc_arr[k], zc = zc_arr[k];
  const int full = meta_full(c.w);
  for (int i = 0; i < 3; i++) {
    const int ki = 3 * k + i;
    const double len = lengths[ki];
    const double e0 = -R[i].f[0] * len;
    const double e1 = -R[i].f[1] * len;
    const double e2 = -R[i].f[2] * len;
    const double hle = he[ki];
    const double zl = ze[ki];
    const double hl = R[i].hleft;
    const double pg = len * (-P.g * 0.5 * (hl * hl - hle * hle - (hle + hc) * (zl - zc)) + R[i].pflux);
    if (full == 1 && dgt(R[i].speed, P.epsilon)) smax = dmax(smax, R[i].speed);
    sw += e0;
    sx += e1;
    sy += e2;
    const int n = (i == 0) ? c.x : (i == 1) ? c.y : c.z;
    if (((n < 0) & (full == 1)) | ((n >= 0) && ((full == 1) & (full_of_neighbour[i] == 0)))) bflux += e0;
    sx -= normals[2 * ki] * pg;
    sy -= normals[2 * ki + 1] * pg;
  }
  out.ew = sw * inv_area;
  out.euh = sx * inv_area;
  out.evh = sy * inv_area;
  out.smax = smax;
  out.bflux = bflux;
}

// ---- boundary values --------------------------------------------------------
AGX_HD void boundary_value(int kind, double n1, double n2, double we, double uhe, double vhe, double ze,
                           double wc, double uhc, double vhc, double zc, double g, const double* val, double& wb,
                           double& uhb, double& vhb) {
  switch (kind) {
    case BK_TRANSMISSIVE_SET_STAGE:   // shallow_water/boundaries.py:295-383
      wb = val[0]; uhb = uhe; vhb = vhe;
      break;
    case BK_TRANSMISSIVE_ZERO_MOM:    // boundaries.py:520-552
      wb = we; uhb = 0.0; vhb = 0.0;
      break;
    case BK_INFLOW:                   // boundaries.py:902-992 (depth 1 above the edge bed)
      wb = ze + val[0]; uhb = val[1]; vhb = val[2];
      break;
    case BK_CHARACTERISTIC: {         // boundaries.py:757-848 (the vectorised form)
      const double wo = val[0];
      const double sqrt_g = sqrt(g);
      const double h_in = dmax(we - ze, 0.0);
      const double h_out = dmax(wo - ze, 0.0);
      if (!dnz(h_in) || !dnz(h_out)) {
        wb = wo;
        uhb = 0.0;
        vhb = 0.0;
      } else {
        const double uh_in = n1 * uhe + n2 * vhe;
        const double vh_in = n2 * uhe - n1 * vhe;
        const double u_in = uh_in / h_in;
        const double sh_in = sqrt(h_in), sh_out = sqrt(h_out);
        double h_m = 0.5 * (sh_in + sh_out) + u_in / 4.0 / sqrt_g;
        h_m = h_m * h_m;
        const double u_m = 0.5 * u_in + sqrt_g * (sh_in - sh_out);
        const double uh_m = h_m * u_m;
        const double vh_m = dgt0(uh_in) ? vh_in : 0.0;
        wb = h_m + ze;
        uhb = uh_m * n1 + vh_m * n2;
        vhb = uh_m * n2 - vh_m * n1;
      }
      break;
    }
    case BK_FLATHER: {                // boundaries.py:1242-1330 (the vectorised form)
      const double so = val[0];
      const double depth = dmax(we - zc, 0.0);
      if (!dnz(depth) || dgt(so, zc)) {
        wb = dle(zc, so) ? so : ze;
        uhb = 0.0 * uhe;
        vhb = 0.0 * vhe;
      } else {
        const double sg = sqrt(g / depth);
        const double ndotq = n1 * uhe + n2 * vhe;
        const double w1 = 0.0 - sg * so;
        const double w2 = dgt0(ndotq) ? (n2 * uhe - n1 * vhe) / depth : 0.0 * ndotq;
        const double w3 = ndotq / depth + sg * we;
        wb = (w3 - w1) / (2.0 * sg);
        const double qperp = (w3 + w1) / 2.0 * depth;
        const double qpar = w2 * depth;
        uhb = qperp * n1 + qpar * n2;
        vhb = qperp * n2 - qpar * n1;
      }
      break;
    }
    case BK_REFLECTIVE: {
      wb = we;
      const double q1 = uhe, q2 = vhe;
      const double r1 = -q1 * n1 - q2 * n2;
      const double r2 = -q1 * n2 + q2 * n1;
      uhb = n1 * r1 - n2 * r2;
      vhb = n2 * r1 + n1 * r2;
      break;
    }
    case BK_TRANSMISSIVE:
      wb = we; uhb = uhe; vhb = vhe;
      break;
    case BK_TRANSMISSIVE_C:
      wb = wc; uhb = uhc; vhb = vhc;
      break;
    case BK_DIRICHLET:
    case BK_TIME_SERIES:
      wb = val[0]; uhb = val[1]; vhb = val[2];
      break;
    case BK_TRANSMISSIVE_N0: {
      // Transmissive_n_momentum_zero_t_momentum_set_stage_boundary style:
      // stage from val[0], normal momentum transmitted, tangential zero
      // (shallow_water/boundaries.py:384-519).
      wb = val[0];
      const double ndotq = n1 * uhe + n2 * vhe;
      uhb = ndotq * n1;
      vhb = ndotq * n2;
      break;
    }
    default:
      break;
  }
}

// ---- friction + update + fix negative -------------------------------------
// h^(7/3) of the Manning term as h^2 * cbrt(h): within 3 ulp of the
// correctly rounded power (the reference's pow(h, 7.0/3.0) is within 1),
// at a fraction of pow's cost on the FP64 pipe.
AGX_HD double h_pow_7_3(double h) { return (h * h) * cbrt(h); }

AGX_HD double manning_S(const Params& P, double w, double z, double uh, double vh, double eta) {
  const double mom = dsqrt((uh * uh + vh * vh));
  double S = 0.0;
  if (dgt(eta, P.hmin)) {
    const double h = w - z;
    if (dge(h, P.hmin)) {
      S = -P.g * eta * eta * mom;
      S = ddiv(S, h_pow_7_3(h));
    }
  }
  return S;
}

AGX_HD double manning_S_sloped(const Params& P, double w, const double* zv3, const double* xv6,
                               double uh, double vh, double eta) {
  double S = 0.0;
  const double z0 = zv3[0], z1 = zv3[1], z2 = zv3[2];
  const double x0 = xv6[0], y0 = xv6[1], x1 = xv6[2], y1 = xv6[3], x2 = xv6[4], y2 = xv6[5];
  if (eta > P.hmin) {
    const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
    double zx = (y2 - y0) * (z1 - z0) - (y1 - y0) * (z2 - z0);
    zx = ddiv(zx, det);
    double zy = (x1 - x0) * (z2 - z0) - (x2 - x0) * (z1 - z0);
    zy = ddiv(zy, det);
    const double zs = dsqrt(1.0 + zx * zx + zy * zy);
    const double zbar = (z0 + z1 + z2) * (1.0 / 3.0);
    const double h = w - zbar;
    if (h >= P.hmin) {
      S = -P.g * eta * eta * zs * dsqrt((uh * uh + vh * vh));
      S = ddiv(S, h_pow_7_3(h));
    }
  }
  return S;
}

// Quantity.update for one cell; returns false on a non-positive denominator.
AGX_HD bool update_quantity(double& q, double expl, double& semi, double dt) {
  const double x = q;
  double s = semi;
  if (!dnz(x)) s = 0.0;
  else if (dnz(s)) s = ddiv(s, x);         // 0/x is a zero: the denominator below is then exactly 1
  q = q + dt * expl;
  const double den = 1.0 - dt * s;
  semi = 0.0;
  if (dle0(den)) return false;
  if (dbits(den) != dbits(1.0)) q = ddiv(q, den);
  return true;
}

}  // namespace agx
