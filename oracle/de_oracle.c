/*
 * de_oracle.c -- CPU oracle for the ANUGA DE (discontinuous-elevation) timestep.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the
 * reference's DE0/DE1 step, used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the parity checker.  The product (the
 * anuga_core_gb300 package and its CUDA library) never links or calls it.
 *
 * Every routine states the reference function it follows (paths relative to
 * the anuga_core project).  Arithmetic is written in the same operation order
 * as the reference so that, compiled with -ffp-contract=off, results are
 * bit-identical to the reference built the same way (tests/test_oracle_ref.py checks this).
 *
 * Serial semantics: the reference's OpenMP extrapolation loop lets a cell
 * zero the centroid velocity of a "surrounded by dry cells" triangle that
 * later cells then read (shallow_water/sw_domain_openmp.c:1486-1495).  With
 * one thread that is a well-defined in-index-order rule; this oracle runs that
 * loop in index order, which is the OMP_NUM_THREADS=1 behaviour.  Loops
 * without such a dependency carry OpenMP pragmas like the reference so the
 * timed CPU baseline can use every host core.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Field layout follows shallow_water/sw_domain.h:14-121 (struct domain):
 * [N,3] arrays are row-major, indices are int64. */
typedef struct {
  int64_t N;                 /* number_of_elements */
  int64_t B;                 /* boundary_length */
  double g, epsilon, minimum_allowed_height, H0;
  double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
  int64_t extrapolate_velocity_second_order;
  int64_t low_froude;
  int64_t ncol_riverwall_hydraulic_properties;
  /* mesh (read only) */
  const int64_t *neighbours, *neighbour_edges, *surrogate_neighbours;
  const int64_t *number_of_boundaries, *tri_full_flag;
  const double *normals, *edgelengths, *radii, *areas;
  const double *edge_coordinates, *centroid_coordinates;
  const int64_t *edge_flux_type, *edge_river_wall_counter, *riverwall_rowIndex;
  const double *riverwall_elevation, *riverwall_hydraulic_properties;
  /* quantities */
  double *stage_c, *xmom_c, *ymom_c, *bed_c, *height_c;
  double *stage_e, *xmom_e, *ymom_e, *bed_e, *height_e;
  double *stage_v, *xmom_v, *ymom_v, *bed_v, *height_v;
  double *stage_b, *xmom_b, *ymom_b;
  double *stage_x, *xmom_x, *ymom_x;      /* explicit_update */
  double *stage_s, *xmom_s, *ymom_s;      /* semi_implicit_update */
  double *max_speed, *x_work, *y_work;
  double *boundary_flux_sum;              /* [3] per substep */
} orc_domain;

static int g_parallel_extrapolation = 0;

/* 1: run the extrapolation's main loop with OpenMP like the reference does
 * (sw_domain_openmp.c:1408), accepting its order dependence; used only for
 * timing the CPU baseline.  0 (default): index order, the parity semantics. */
void orc_set_parallel_extrapolation(int on) { g_parallel_extrapolation = on; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Protect: shallow_water/sw_domain_openmp.c:1096-1171 (_openmp_protect).
 * zero_ymom=0 reproduces that routine, which writes xmomentum twice and never
 * ymomentum (:1139-1140); zero_ymom=1 follows sw_domain_orig.c:1251-1252,
 * which zeroes both.  Returns the mass added. */
double orc_protect(orc_domain *D, int zero_ymom) {
  double mass_error = 0.0;
  const double hmin = D->minimum_allowed_height;
  int64_t k;
#pragma omp parallel for schedule(static) reduction(+ : mass_error)
  for (k = 0; k < D->N; k++) {
    double depth = D->stage_c[k] - D->bed_c[k];
    if (depth < hmin * 1.0) {
      D->xmom_c[k] = 0.0;
      if (zero_ymom) D->ymom_c[k] = 0.0;
      if (depth <= 0.0) {
        double floor_z = D->bed_c[k];
        if (D->stage_c[k] < floor_z) {
          mass_error += (floor_z - D->stage_c[k]) * D->areas[k];
          D->stage_c[k] = floor_z;
          D->stage_v[3 * k + 0] = floor_z;
          D->stage_v[3 * k + 1] = floor_z;
          D->stage_v[3 * k + 2] = floor_z;
        }
      }
    }
  }
  return mass_error;
}

/* ------------------------------------------------------------------------ */
/* Limited linear reconstruction helpers:
 * __find_qmin_and_qmax  sw_domain_openmp.c:1174-1193
 * __limit_gradient      sw_domain_openmp.c:1195-1231
 * __calc_edge_values    sw_domain_openmp.c:1233-1284 */
static void limit_jumps(double jump[3], double lo, double hi, double beta) {
  const double tiny = 1.0e-100;
  double ratio = 1000.0, cand = 1.0;
  for (int i = 0; i < 3; i++) {
    if (jump[i] < -tiny) cand = lo / jump[i];
    if (jump[i] > tiny) cand = hi / jump[i];
    ratio = fmin(cand, ratio);
  }
  double phi = fmin(ratio * beta, 1.0);
  jump[0] = jump[0] * phi;
  jump[1] = jump[1] * phi;
  jump[2] = jump[2] * phi;
}

typedef struct {
  double dxv[3], dyv[3];      /* edge midpoint - centroid */
  double dx1, dx2, dy1, dy2;  /* auxiliary-triangle differentials */
  double inv_area2;
} aux_geom;

static void reconstruct3(double beta, double qc, double q0, double q1, double q2,
                         const aux_geom *G, double out[3]) {
  if (!(beta > 0.0)) {
    out[0] = qc; out[1] = qc; out[2] = qc;
    return;
  }
  double d0 = q0 - qc;
  double d1 = q1 - q0;
  double d2 = q2 - q0;
  double gx = G->dy2 * d1 - G->dy1 * d2;
  gx *= G->inv_area2;
  double gy = G->dx1 * d2 - G->dx2 * d1;
  gy *= G->inv_area2;
  double jump[3];
  for (int i = 0; i < 3; i++) jump[i] = gx * G->dxv[i] + gy * G->dyv[i];
  double hi = fmax(fmax(d0, fmax(d0 + d1, d0 + d2)), 0.0);
  double lo = fmin(fmin(d0, fmin(d0 + d1, d0 + d2)), 0.0);
  limit_jumps(jump, lo, hi, beta);
  for (int i = 0; i < 3; i++) out[i] = qc + jump[i];
}

/* One-neighbour gradient used when a triangle has two boundary edges:
 * sw_domain_openmp.c:1646-1842 (one quantity of that block). */
static void reconstruct_towards(double beta, double qc, double qn, double gdx,
                                double gdy, const aux_geom *G, double out[3]) {
  double d = qn - qc;
  double gx = d * gdx;
  double gy = d * gdy;
  double jump[3];
  for (int i = 0; i < 3; i++) jump[i] = gx * G->dxv[i] + gy * G->dyv[i];
  double lo, hi;
  if (d >= 0.0) { lo = 0.0; hi = d; } else { lo = d; hi = 0.0; }
  limit_jumps(jump, lo, hi, beta);
  for (int i = 0; i < 3; i++) out[i] = qc + jump[i];
}

/* ------------------------------------------------------------------------ */
/* Extrapolation: _openmp_extrapolate_second_order_edge_sw,
 * sw_domain_openmp.c:1336-1952.  The main loop runs in index order. */
int orc_extrapolate(orc_domain *D) {
  const int64_t N = D->N;
  const double hmin_allowed = D->minimum_allowed_height;
  const int velo = D->extrapolate_velocity_second_order == 1;
  const double a_tmp = 0.3, b_tmp = 0.1;
  const double c_tmp = 1.0 / (a_tmp - b_tmp);
  const double d_tmp = 1.0 - (c_tmp * a_tmp);
  int64_t k;

  /* depths and centroid velocities, :1373-1402 */
#pragma omp parallel for schedule(static)
  for (k = 0; k < N; k++) {
    double dk = fmax(D->stage_c[k] - D->bed_c[k], 0.0);
    D->height_c[k] = dk;
    D->x_work[k] = 0.0;
    D->y_work[k] = 0.0;
    if (dk <= hmin_allowed) {
      D->x_work[k] = 0.0;
      D->xmom_c[k] = 0.0;
      D->y_work[k] = 0.0;
      D->ymom_c[k] = 0.0;
    }
    if (velo && dk > hmin_allowed) {
      double inv = 1.0 / dk;
      D->x_work[k] = D->xmom_c[k];
      D->xmom_c[k] = D->xmom_c[k] * inv;
      D->y_work[k] = D->ymom_c[k];
      D->ymom_c[k] = D->ymom_c[k] * inv;
    }
  }

  /* reconstruction, :1418-1896 (in index order unless timing) */
#pragma omp parallel for schedule(static) if (g_parallel_extrapolation)
  for (k = 0; k < N; k++) {
    const int64_t k3 = 3 * k;
    const double xc = D->centroid_coordinates[2 * k];
    const double yc = D->centroid_coordinates[2 * k + 1];
    aux_geom G;
    for (int i = 0; i < 3; i++) {
      G.dxv[i] = D->edge_coordinates[6 * k + 2 * i] - xc;
      G.dyv[i] = D->edge_coordinates[6 * k + 2 * i + 1] - yc;
    }
    const int64_t s0 = D->surrogate_neighbours[k3 + 0];
    const int64_t s1 = D->surrogate_neighbours[k3 + 1];
    const int64_t s2 = D->surrogate_neighbours[k3 + 2];
    const double x0 = D->centroid_coordinates[2 * s0], y0 = D->centroid_coordinates[2 * s0 + 1];
    const double x1 = D->centroid_coordinates[2 * s1], y1 = D->centroid_coordinates[2 * s1 + 1];
    const double x2 = D->centroid_coordinates[2 * s2], y2 = D->centroid_coordinates[2 * s2 + 1];
    G.dx1 = x1 - x0;
    G.dx2 = x2 - x0;
    G.dy1 = y1 - y0;
    G.dy2 = y2 - y0;
    const double area2 = G.dy2 * G.dx1 - G.dy1 * G.dx2;

    const int dry0 = (D->height_c[s0] < hmin_allowed) | (s0 == k);
    const int dry1 = (D->height_c[s1] < hmin_allowed) | (s1 == k);
    const int dry2 = (D->height_c[s2] < hmin_allowed) | (s2 == k);
    if (dry0 & dry1 & dry2) {
      D->x_work[k] = 0.0;
      D->xmom_c[k] = 0.0;
      D->y_work[k] = 0.0;
      D->ymom_c[k] = 0.0;
    }

    const int64_t nb = D->number_of_boundaries[k];
    double ev[3];
    if (nb == 3) {
      for (int i = 0; i < 3; i++) {
        D->stage_e[k3 + i] = D->stage_c[k];
        D->xmom_e[k3 + i] = D->xmom_c[k];
        D->ymom_e[k3 + i] = D->ymom_c[k];
        D->height_e[k3 + i] = D->height_c[k];
      }
    } else if (nb <= 1) {
      const double hc = D->height_c[k];
      const double h0 = D->height_c[s0], h1 = D->height_c[s1], h2 = D->height_c[s2];
      const double hlo = fmin(fmin(h0, fmin(h1, h2)), hc);
      const double hhi = fmax(fmax(h0, fmax(h1, h2)), hc);
      double hfactor = fmax(0.0, fmin(c_tmp * fmax(hlo, 0.0) / fmax(hc, 1.0e-06) + d_tmp,
                                      fmin(c_tmp * fmax(hc, 0.0) / fmax(hhi, 1.0e-06) + d_tmp, 1.0)));
      hfactor = fmin(1.2 * fmax(hlo - hmin_allowed, 0.0) / (fmax(hlo, 0.0) + 1.0 * hmin_allowed), hfactor);
      G.inv_area2 = 1.0 / area2;

      double beta = D->beta_w_dry + (D->beta_w - D->beta_w_dry) * hfactor;
      reconstruct3(beta, D->stage_c[k], D->stage_c[s0], D->stage_c[s1], D->stage_c[s2], &G, ev);
      for (int i = 0; i < 3; i++) D->stage_e[k3 + i] = ev[i];
      reconstruct3(beta, D->height_c[k], D->height_c[s0], D->height_c[s1], D->height_c[s2], &G, ev);
      for (int i = 0; i < 3; i++) D->height_e[k3 + i] = ev[i];

      beta = D->beta_uh_dry + (D->beta_uh - D->beta_uh_dry) * hfactor;
      reconstruct3(beta, D->xmom_c[k], D->xmom_c[s0], D->xmom_c[s1], D->xmom_c[s2], &G, ev);
      for (int i = 0; i < 3; i++) D->xmom_e[k3 + i] = ev[i];

      beta = D->beta_vh_dry + (D->beta_vh - D->beta_vh_dry) * hfactor;
      reconstruct3(beta, D->ymom_c[k], D->ymom_c[s0], D->ymom_c[s1], D->ymom_c[s2], &G, ev);
      for (int i = 0; i < 3; i++) D->ymom_e[k3 + i] = ev[i];
    } else {
      /* two boundary edges: gradient towards the single interior neighbour */
      int64_t j = k3;
      while (j < k3 + 3 && D->surrogate_neighbours[j] == k) j++;
      if (j == k3 + 3) j = k3 + 2;  /* unreachable for nb==2 meshes; stay in bounds */
      const int64_t kn = D->surrogate_neighbours[j];
      const double ddx = D->centroid_coordinates[2 * kn] - xc;
      const double ddy = D->centroid_coordinates[2 * kn + 1] - yc;
      const double dist2 = ddx * ddx + ddy * ddy;
      double gdx = 1.0 / dist2;
      const double gdy = gdx * ddy;
      gdx *= ddx;
      reconstruct_towards(D->beta_w, D->stage_c[k], D->stage_c[kn], gdx, gdy, &G, ev);
      for (int i = 0; i < 3; i++) D->stage_e[k3 + i] = ev[i];
      reconstruct_towards(D->beta_w, D->height_c[k], D->height_c[kn], gdx, gdy, &G, ev);
      for (int i = 0; i < 3; i++) D->height_e[k3 + i] = ev[i];
      reconstruct_towards(D->beta_w, D->xmom_c[k], D->xmom_c[kn], gdx, gdy, &G, ev);
      for (int i = 0; i < 3; i++) D->xmom_e[k3 + i] = ev[i];
      reconstruct_towards(D->beta_w, D->ymom_c[k], D->ymom_c[kn], gdx, gdy, &G, ev);
      for (int i = 0; i < 3; i++) D->ymom_e[k3 + i] = ev[i];
    }

    if (velo) {
      for (int i = 0; i < 3; i++) {
        const double dk = D->height_e[k3 + i];
        D->xmom_e[k3 + i] = D->xmom_e[k3 + i] * dk;
        D->ymom_e[k3 + i] = D->ymom_e[k3 + i] * dk;
      }
    }
    for (int i = 0; i < 3; i++) D->bed_e[k3 + i] = D->stage_e[k3 + i] - D->height_e[k3 + i];

    /* vertex values from edge values (:1870-1892) */
    double *ed[5] = {D->stage_e, D->height_e, D->xmom_e, D->ymom_e, D->bed_e};
    double *vx[5] = {D->stage_v, D->height_v, D->xmom_v, D->ymom_v, D->bed_v};
    for (int q = 0; q < 5; q++) {
      const double e0 = ed[q][k3], e1 = ed[q][k3 + 1], e2 = ed[q][k3 + 2];
      vx[q][k3 + 0] = e1 + e2 - e0;
      vx[q][k3 + 1] = e0 + e2 - e1;
      vx[q][k3 + 2] = e0 + e1 - e2;
    }
  }

  /* restore centroid momenta, :1899-1949 */
  if (velo) {
#pragma omp parallel for schedule(static)
    for (k = 0; k < N; k++) {
      D->xmom_c[k] = D->x_work[k];
      D->ymom_c[k] = D->y_work[k];
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Central-upwind edge flux: __flux_function_central,
 * sw_domain_openmp.c:65-268 (Kurganov-Noelle-Petrova, rotated frame). */
static void edge_flux_central(const double ql[3], const double qr[3],
                              double hl, double hr, double hle, double hre,
                              double n1, double n2, double eps, double ze,
                              double g, int64_t low_froude,
                              double flux[3], double *speed, double *pflux) {
  if (hl == 0.0 && hr == 0.0) {
    flux[0] = flux[1] = flux[2] = 0.0;
    *speed = 0.0;
    *pflux = 0.0;
    return;
  }
  const double wl = ql[0], wr = qr[0];
  double uhl = n1 * ql[1] + n2 * ql[2];
  double vhl = -n2 * ql[1] + n1 * ql[2];
  double uhr = n1 * qr[1] + n2 * qr[2];
  double vhr = -n2 * qr[1] + n1 * qr[2];
  double ul, vl, ur, vr;
  if (hle > 0.0) {
    const double inv = 1.0 / hle;
    ul = uhl * inv;
    uhl = hl * ul;
    vl = vhl * inv;
    vhl = hl * inv * vhl;
  } else {
    ul = uhl = vhl = vl = 0.0;
  }
  if (hre > 0.0) {
    const double inv = 1.0 / hre;
    ur = uhr * inv;
    uhr = hr * ur;
    vr = vhr * inv;
    vhr = hr * inv * vhr;
  } else {
    ur = uhr = vhr = vr = 0.0;
  }
  const double cl = sqrt(g * hl);
  const double cr = sqrt(g * hr);
  double froude_scale;
  if (low_froude == 1) {
    froude_scale = sqrt(fmax(0.001, fmin(1.0, (ur * ur + ul * ul + vr * vr + vl * vl) /
                                                  (cl * cl + cr * cr + 1.0e-10))));
  } else if (low_froude == 2) {
    froude_scale = sqrt((ur * ur + ul * ul + vr * vr + vl * vl) / (cl * cl + cr * cr + 1.0e-10));
    froude_scale = sqrt(fmin(1.0, 0.01 + fmax(froude_scale - 0.01, 0.0)));
  } else {
    froude_scale = 1.0;
  }
  double smax = fmax(ul + cl, ur + cr);
  if (smax < 0.0) smax = 0.0;
  double smin = fmin(ul - cl, ur - cr);
  if (smin > 0.0) smin = 0.0;
  const double fl0 = ul * hl, fl1 = ul * uhl, fl2 = ul * vhl;
  const double fr0 = ur * hr, fr1 = ur * uhr, fr2 = ur * vhr;
  const double span = smax - smin;
  if (span < eps) {
    flux[0] = flux[1] = flux[2] = 0.0;
    *speed = 0.0;
    *pflux = 0.5 * g * 0.5 * (hl * hl + hr * hr);
    return;
  }
  *speed = fmax(smax, -smin);
  const double inv_span = 1.0 / fmax(span, 1.0e-100);
  double f0 = smax * fl0 - smin * fr0;
  f0 += (smax * smin) * (fmax(wr, ze) - fmax(wl, ze));
  f0 *= inv_span;
  double f1 = smax * fl1 - smin * fr1;
  f1 += froude_scale * (smax * smin) * (uhr - uhl);
  f1 *= inv_span;
  double f2 = smax * fl2 - smin * fr2;
  f2 += froude_scale * (smax * smin) * (vhr - vhl);
  f2 *= inv_span;
  *pflux = 0.5 * g * (smax * hl * hl - smin * hr * hr) * inv_span;
  /* rotate back (__rotate with (n1, -n2)) */
  const double m2 = -n2;
  flux[0] = f0;
  flux[1] = n1 * f1 + m2 * f2;
  flux[2] = -m2 * f1 + n1 * f2;
}

/* Villemonte weir correction: __adjust_edgeflux_with_weir,
 * sw_domain_openmp.c:324-426. */
static void weir_adjust(double flux[3], double hl, double hr, double g, double weir_height,
                        double Qfactor, double s1, double s2, double h1, double h2,
                        double *speed) {
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
    const double newFlux = (rw * (1.0 - w1) + w1 * flux[0]) * (1.0 - w2) + w2 * flux[0];
    double scale;
    if (fabs(flux[0]) > 1.0e-100) scale = newFlux / flux[0];
    else scale = 0.0;
    scale = fmax(scale, 0.0);
    flux[0] = newFlux;
    flux[1] *= fmin(scale, 10.0);
    flux[2] *= fmin(scale, 10.0);
  }
  if (fabs(flux[0]) > 0.0) *speed = sqrt(g * (maxhd + weir_height)) + fabs(flux[0] / (maxhd + 1.0e-12));
}

/* ------------------------------------------------------------------------ */
/* Fluxes, gravity terms and CFL timestep: _openmp_compute_fluxes_central,
 * sw_domain_openmp.c:456-772.  The substep is explicit (the reference keeps
 * it in a static counter, :492-505).  Returns the min edge timestep on
 * substep 0 and `timestep` unchanged otherwise. */
double orc_compute_fluxes(orc_domain *D, int64_t substep, double timestep) {
  const double g = D->g, eps = D->epsilon;
  const int64_t lf = D->low_froude;
  double local_timestep = 1.0e+100;
  double bsum = 0.0;
  int64_t k;
#pragma omp parallel for schedule(static) reduction(min : local_timestep) reduction(+ : bsum)
  for (k = 0; k < D->N; k++) {
    double speed_max_last = 0.0;
    D->stage_x[k] = 0.0;
    D->xmom_x[k] = 0.0;
    D->ymom_x[k] = 0.0;
    for (int i = 0; i < 3; i++) {
      const int64_t ki = 3 * k + i;
      double ql[3] = {D->stage_e[ki], D->xmom_e[ki], D->ymom_e[ki]};
      const double zl = D->bed_e[ki];
      const double hle = D->height_e[ki];
      const double hc = D->height_c[k];
      const double zc = D->bed_c[k];
      const int64_t n = D->neighbours[ki];
      double hc_n = hc;
      double zc_n = D->bed_c[k];
      double qr[3], zr, hre;
      if (n < 0) {
        const int64_t m = -n - 1;
        qr[0] = D->stage_b[m];
        qr[1] = D->xmom_b[m];
        qr[2] = D->ymom_b[m];
        zr = zl;
        hre = fmax(qr[0] - zr, 0.0);
      } else {
        hc_n = D->height_c[n];
        zc_n = D->bed_c[n];
        const int64_t nm = 3 * n + D->neighbour_edges[ki];
        qr[0] = D->stage_e[nm];
        qr[1] = D->xmom_e[nm];
        qr[2] = D->ymom_e[nm];
        zr = D->bed_e[nm];
        hre = D->height_e[nm];
      }
      double z_half = fmax(zl, zr);
      const int wall = D->edge_flux_type && D->edge_flux_type[ki] == 1;
      int64_t rw_id = 0;
      if (wall) {
        rw_id = D->edge_river_wall_counter[ki];
        z_half = fmax(D->riverwall_elevation[rw_id - 1], z_half);
      }
      const double h_left = fmax(hle + zl - z_half, 0.0);
      const double h_right = fmax(hre + zr - z_half, 0.0);
      const double nx = D->normals[2 * ki], ny = D->normals[2 * ki + 1];
      double flux[3], speed, pflux;
      edge_flux_central(ql, qr, h_left, h_right, hle, hre, nx, ny, eps, z_half, g, lf,
                        flux, &speed, &pflux);
      if (wall) {
        const int64_t row = D->riverwall_rowIndex[rw_id - 1] * D->ncol_riverwall_hydraulic_properties;
        const double *hp = D->riverwall_hydraulic_properties + row;
        const double weir_height = fmax(D->riverwall_elevation[rw_id - 1] - fmin(zl, zr), 0.0);
        const double hl_tmp = fmax(D->stage_c[k] - z_half, 0.0);
        const double hr_tmp = (n >= 0) ? fmax(D->stage_c[n] - z_half, 0.0)
                                       : fmax(hc_n + zr - z_half, 0.0);
        if (D->riverwall_elevation[rw_id - 1] > fmax(zc, zc_n))
          weir_adjust(flux, hl_tmp, hr_tmp, g, weir_height, hp[0], hp[1], hp[2], hp[3], hp[4], &speed);
      }
      const double len = D->edgelengths[ki];
      flux[0] = -flux[0] * len;
      flux[1] = -flux[1] * len;
      flux[2] = -flux[2] * len;
      const double pgrad = len * (-g * 0.5 * (h_left * h_left - hle * hle - (hle + hc) * (zl - zc)) + pflux);
      if (substep == 0) {
        const double edge_dt = D->radii[k] * 1.0 / fmax(speed, eps);
        if (D->tri_full_flag[k] == 1 && speed > eps) {
          local_timestep = fmin(local_timestep, edge_dt);
          speed_max_last = fmax(speed_max_last, speed);
        }
      }
      D->stage_x[k] += flux[0];
      D->xmom_x[k] += flux[1];
      D->ymom_x[k] += flux[2];
      if (((n < 0) & (D->tri_full_flag[k] == 1)) |
          ((n >= 0) && ((D->tri_full_flag[k] == 1) & (D->tri_full_flag[n] == 0))))
        bsum += flux[0];
      D->xmom_x[k] -= D->normals[2 * ki] * pgrad;
      D->ymom_x[k] -= D->normals[2 * ki + 1] * pgrad;
    }
    if (substep == 0) D->max_speed[k] = speed_max_last;
    const double inv_area = 1.0 / D->areas[k];
    D->stage_x[k] *= inv_area;
    D->xmom_x[k] *= inv_area;
    D->ymom_x[k] *= inv_area;
  }
  D->boundary_flux_sum[substep] = bsum;
  return substep == 0 ? local_timestep : timestep;
}

/* ------------------------------------------------------------------------ */
/* Manning friction, flat bed: _openmp_manning_friction_flat,
 * sw_domain_openmp.c:1954-1986. */
void orc_manning_flat(double g, double eps, int64_t N, const double *w, const double *z,
                      const double *uh, const double *vh, const double *eta,
                      double *xmom_s, double *ymom_s) {
  const double seven_thirds = 7.0 / 3.0;
  int64_t k;
#pragma omp parallel for schedule(static)
  for (k = 0; k < N; k++) {
    const double mom = sqrt((uh[k] * uh[k] + vh[k] * vh[k]));
    double S = 0.0;
    if (eta[k] > eps) {
      const double h = w[k] - z[k];
      if (h >= eps) {
        S = -g * eta[k] * eta[k] * mom;
        S /= pow(h, seven_thirds);
      }
    }
    xmom_s[k] += S * uh[k];
    ymom_s[k] += S * vh[k];
  }
}

/* Manning friction with bed slope: _openmp_manning_friction_sloped,
 * sw_domain_openmp.c:1988-2034 with _gradient, utilities/util_ext.h:52-92. */
void orc_manning_sloped(double g, double eps, int64_t N, const double *xv, const double *w,
                        const double *zv, const double *uh, const double *vh,
                        const double *eta, double *xmom_s, double *ymom_s) {
  const double one_third = 1.0 / 3.0;
  const double seven_thirds = 7.0 / 3.0;
  int64_t k;
#pragma omp parallel for schedule(static)
  for (k = 0; k < N; k++) {
    double S = 0.0;
    const double z0 = zv[3 * k], z1 = zv[3 * k + 1], z2 = zv[3 * k + 2];
    const double x0 = xv[6 * k], y0 = xv[6 * k + 1];
    const double x1 = xv[6 * k + 2], y1 = xv[6 * k + 3];
    const double x2 = xv[6 * k + 4], y2 = xv[6 * k + 5];
    if (eta[k] > eps) {
      const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
      double zx = (y2 - y0) * (z1 - z0) - (y1 - y0) * (z2 - z0);
      zx /= det;
      double zy = (x1 - x0) * (z2 - z0) - (x2 - x0) * (z1 - z0);
      zy /= det;
      const double zs = sqrt(1.0 + zx * zx + zy * zy);
      const double zbar = (z0 + z1 + z2) * one_third;
      const double h = w[k] - zbar;
      if (h >= eps) {
        S = -g * eta[k] * eta[k] * zs * sqrt((uh[k] * uh[k] + vh[k] * vh[k]));
        S /= pow(h, seven_thirds);
      }
    }
    xmom_s[k] += S * uh[k];
    ymom_s[k] += S * vh[k];
  }
}

/* ------------------------------------------------------------------------ */
/* Quantity.update: _update, abstract_2d_finite_volumes/quantity.c:772-818.
 * Returns -1 (like the reference) on a non-positive semi-implicit
 * denominator, after applying the explicit update to every cell and the
 * semi-implicit one to the cells before it. */
int orc_update(int64_t N, double dt, double *q, const double *expl, double *semi) {
  int64_t k;
  for (k = 0; k < N; k++) {
    const double x = q[k];
    if (x == 0.0) semi[k] = 0.0;
    else semi[k] /= x;
  }
  for (k = 0; k < N; k++) q[k] += dt * expl[k];
  for (k = 0; k < N; k++) {
    const double den = 1.0 - dt * semi[k];
    if (den <= 0.0) return -1;
    q[k] /= den;
  }
  memset(semi, 0, (size_t)N * sizeof(double));
  return 0;
}

/* fix_negative_cells: _openmp_fix_negative_cells, sw_domain_openmp.c:2037-2056. */
int64_t orc_fix_negative(orc_domain *D) {
  int64_t count = 0, k;
#pragma omp parallel for schedule(static) reduction(+ : count)
  for (k = 0; k < D->N; k++) {
    if ((D->stage_c[k] - D->bed_c[k] < 0.0) & (D->tri_full_flag[k] > 0)) {
      count = count + 1;
      D->stage_c[k] = D->bed_c[k];
      D->xmom_c[k] = 0.0;
      D->ymom_c[k] = 0.0;
    }
  }
  return count;
}

/* RK2 helpers: _backup_centroid_values / _saxpy_centroid_values,
 * quantity.c:735-770. */
void orc_backup(int64_t N, const double *q, double *q0) {
  for (int64_t k = 0; k < N; k++) q0[k] = q[k];
}

void orc_saxpy(int64_t N, double a, double b, double *q, const double *q0) {
  for (int64_t k = 0; k < N; k++) q[k] = a * q[k] + b * q0[k];
}

/* ------------------------------------------------------------------------ */
/* Boundary conditions on a list of boundary edges `ids` (indices into the
 * boundary arrays); vol/edge give the cell and edge of each boundary index. */

/* Reflective_boundary.evaluate_segment, shallow_water/boundaries.py:235-292
 * (stage and momenta; the elevation/height/velocity copies it also makes do
 * not enter the flux). */
void orc_bc_reflective(orc_domain *D, const int64_t *ids, int64_t n, const int64_t *vol,
                       const int64_t *edge) {
  for (int64_t j = 0; j < n; j++) {
    const int64_t m = ids[j];
    const int64_t ki = 3 * vol[m] + edge[m];
    const double n1 = D->normals[2 * ki], n2 = D->normals[2 * ki + 1];
    D->stage_b[m] = D->stage_e[ki];
    const double q1 = D->xmom_e[ki], q2 = D->ymom_e[ki];
    const double r1 = -q1 * n1 - q2 * n2;
    const double r2 = -q1 * n2 + q2 * n1;
    D->xmom_b[m] = n1 * r1 - n2 * r2;
    D->ymom_b[m] = n2 * r1 + n1 * r2;
  }
}

/* Transmissive_boundary.evaluate_segment,
 * abstract_2d_finite_volumes/generic_boundary_conditions.py:173-195. */
void orc_bc_transmissive(orc_domain *D, const int64_t *ids, int64_t n, const int64_t *vol,
                         const int64_t *edge, int centroid) {
  for (int64_t j = 0; j < n; j++) {
    const int64_t m = ids[j];
    if (centroid) {
      D->stage_b[m] = D->stage_c[vol[m]];
      D->xmom_b[m] = D->xmom_c[vol[m]];
      D->ymom_b[m] = D->ymom_c[vol[m]];
    } else {
      const int64_t ki = 3 * vol[m] + edge[m];
      D->stage_b[m] = D->stage_e[ki];
      D->xmom_b[m] = D->xmom_e[ki];
      D->ymom_b[m] = D->ymom_e[ki];
    }
  }
}

/* Dirichlet_boundary.evaluate_segment with the three conserved values,
 * generic_boundary_conditions.py:221-264. */
void orc_bc_dirichlet(orc_domain *D, const int64_t *ids, int64_t n, double w, double uh,
                      double vh) {
  for (int64_t j = 0; j < n; j++) {
    const int64_t m = ids[j];
    D->stage_b[m] = w;
    D->xmom_b[m] = uh;
    D->ymom_b[m] = vh;
  }
}
