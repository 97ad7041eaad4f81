// Host check of the plain path's limiter (de_plain.cuh limiter_phi: ratio
// tests with margin, failing ratios only, one division per call) against a
// direct restatement of the reference's __limit_gradient
// (shallow_water/sw_domain_openmp.c:1195-1231) on random and adversarial
// inputs: jumps around +-1e-100, zero and tiny ranges, near-equal ratios,
// betas 1, 0.5, 0.2 and random; and the wet/dry factor (wet_dry_factor:
// margin tests, unproved terms only) against the reference's formula
// (sw_domain_openmp.c:1537-1551) on depths across the thresholds.  Prints
// the number of mismatches (value mismatches; a zero's sign is not counted)
// and exits non-zero on any.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <random>
struct int4 { int x, y, z, w; };
#include "../../anuga_core_gb300/csrc/de_plain.cuh"

static double ref_phi(const double jump[3], double lo, double hi, double beta) {
  const double tiny = 1.0e-100;
  double r = 1000.0, r0 = 1.0;
  for (int i = 0; i < 3; i++) {
    if (jump[i] < -tiny) r0 = lo / jump[i];
    if (jump[i] > tiny) r0 = hi / jump[i];
    r = std::fmin(r0, r);
  }
  return std::fmin(r * beta, 1.0);
}

static double ref_wet_dry(const agx::Params& P, double hc, double hmin_n, double hmax_n) {
  double f = std::fmax(0.0, std::fmin(P.c_tmp * std::fmax(hmin_n, 0.0) / std::fmax(hc, 1.0e-06) + P.d_tmp,
                                      std::fmin(P.c_tmp * std::fmax(hc, 0.0) / std::fmax(hmax_n, 1.0e-06) + P.d_tmp, 1.0)));
  f = std::fmin(1.2 * std::fmax(hmin_n - P.hmin, 0.0) / (std::fmax(hmin_n, 0.0) + 1.0 * P.hmin), f);
  return f;
}

static long long check_wet_dry(std::mt19937_64& rng) {
  agx::Params P{};
  P.c_tmp = 1.0 / (0.3 - 0.1);
  P.d_tmp = 1.0 - (P.c_tmp * 0.3);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::uniform_int_distribution<int> e(-20, 3), pick(0, 9);
  long long bad = 0;
  for (int it = 0; it < 2000000; it++) {
    P.hmin = pick(rng) < 5 ? 1.0e-5 : 1.0e-12;
    double h[3];
    for (int i = 0; i < 3; i++) h[i] = pick(rng) == 0 ? 0.0 : std::ldexp(u(rng), e(rng));
    if (pick(rng) == 0) h[1] = 0.3 * h[0] * (1.0 + std::ldexp(u(rng) - 0.5, -38));   // at the 0.3 threshold
    if (pick(rng) == 0) h[1] = P.hmin * (11.0 + std::ldexp(u(rng) - 0.5, -30));      // at C's threshold
    const double hc = h[0];
    const double lo = std::fmin(h[1], std::fmin(h[2], hc)), hi = std::fmax(h[1], std::fmax(h[2], hc));
    const double got = agx::wet_dry_factor(P, hc, lo, hi), want = ref_wet_dry(P, hc, lo, hi);
    if (!(got == want)) {
      if (bad < 10) std::printf("wet/dry mismatch: hc=%.17g lo=%.17g hi=%.17g got %.17g want %.17g\n", hc, lo, hi, got, want);
      bad++;
    }
  }
  return bad;
}

int main() {
  std::mt19937_64 rng(777);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> e(-12, 4), pick(0, 9);
  long long bad = 0, n = 0, partial = 0;
  const double betas[] = {1.0, 0.5, 0.2, 0.7, 0.999999};
  for (int it = 0; it < 4000000; it++) {
    double jump[3], lo, hi, beta;
    const int mode = pick(rng);
    for (int i = 0; i < 3; i++) {
      jump[i] = std::ldexp(u(rng), e(rng));
      if (pick(rng) == 0) jump[i] = (pick(rng) < 5 ? 1.0 : -1.0) * 1.0e-100 * (1.0 + 0.5 * u(rng));
      if (pick(rng) == 0) jump[i] = 0.0;
    }
    hi = std::fabs(std::ldexp(u(rng), e(rng)));
    lo = -std::fabs(std::ldexp(u(rng), e(rng)));
    if (mode == 1) hi = 0.0;
    if (mode == 2) lo = 0.0;
    if (mode == 3) {               // near-equal ratios: jump_b = jump_a * (hi/hi') rounded
      jump[1] = std::fabs(jump[0]) * (1.0 + std::ldexp(u(rng), -50));
      jump[2] = std::nextafter(jump[1], 2.0);
      jump[0] = std::fabs(jump[0]);
    }
    if (mode == 4) {               // ratios within rounding of 1 / beta
      beta = betas[pick(rng) % 5];
      for (int i = 0; i < 3; i++) jump[i] = std::fabs(jump[i]) + 1e-300;
      hi = jump[0] / beta;
      if (pick(rng) < 5) hi = std::nextafter(hi, 0.0);
    } else {
      beta = pick(rng) < 8 ? betas[pick(rng) % 5] : std::fabs(u(rng));
    }
    const double inv = pick(rng) < 5 ? agx::positive_inverse(beta) : 0.0;
    const double got = agx::limiter_phi(jump, lo, hi, beta, inv);
    const double want = ref_phi(jump, lo, hi, beta);
    n++;
    if (want < 1.0) partial++;
    if (!(got == want)) {
      if (bad < 10) std::printf("mismatch: j=(%.17g %.17g %.17g) lo=%.17g hi=%.17g beta=%.17g got %.17g want %.17g\n",
                                jump[0], jump[1], jump[2], lo, hi, beta, got, want);
      bad++;
    }
  }
  std::printf("cases %lld limited %lld mismatches %lld\n", n, partial, bad);
  const long long wd = check_wet_dry(rng);
  std::printf("wet/dry mismatches %lld\n", wd);
  bad += wd;
  return bad == 0 ? 0 : 1;
}
