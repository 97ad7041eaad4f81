// Host check of the integer-pipe FP64 comparisons of de_plain.cuh against
// IEEE comparisons: special values (both zeros, subnormals, infinities,
// extremes) in every pair, then random bit patterns and random values of
// mixed magnitude.  Prints the number of mismatches (0 expected) and exits
// non-zero if there are any.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <vector>
#include <random>
#include <limits>
struct int4 { int x, y, z, w; };     // the CUDA vector type the header's kernels take
#include "../../anuga_core_gb300/csrc/de_plain.cuh"

using namespace agx;

static long long g_bad = 0;

static bool same_or_equal_zero(double a, double b) {
  // dmax/dmin may differ from fmax/fmin only in the sign of a zero result
  if (a == 0.0 && b == 0.0) return true;
  return std::memcmp(&a, &b, sizeof a) == 0;
}

static void check_pair(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return;
  if (dlt(a, b) != (a < b)) g_bad++;
  if (dle(a, b) != (a <= b)) g_bad++;
  if (dgt(a, b) != (a > b)) g_bad++;
  if (dge(a, b) != (a >= b)) g_bad++;
  if (!same_or_equal_zero(dmax(a, b), std::fmax(a, b))) g_bad++;
  if (!same_or_equal_zero(dmin(a, b), std::fmin(a, b))) g_bad++;
  // opposite zeros: dmax gives +0, dmin -0
  if (a == 0.0 && b == 0.0 && std::signbit(a) != std::signbit(b)) {
    if (std::signbit(dmax(a, b)) || !std::signbit(dmin(a, b))) g_bad++;
  }
}

static void check_one(double x) {
  if (std::isnan(x)) return;
  if (dgt0(x) != (x > 0.0)) g_bad++;
  if (dge0(x) != (x >= 0.0)) g_bad++;
  if (dle0(x) != (x <= 0.0)) g_bad++;
  if (dnz(x) != (x != 0.0)) g_bad++;
  if ((dkey(x) < -1) != (x < 0.0)) g_bad++;
}

int main() {
  const double inf = std::numeric_limits<double>::infinity();
  const double dmin_sub = std::numeric_limits<double>::denorm_min();
  const double dmin_norm = std::numeric_limits<double>::min();
  const double dmax_v = std::numeric_limits<double>::max();
  std::vector<double> sp = {0.0, -0.0, dmin_sub, -dmin_sub, dmin_norm, -dmin_norm, 1.0e-100, -1.0e-100,
                            1.0e-12, -1.0e-12, 0.5, -0.5, 1.0, -1.0, std::nextafter(1.0, 2.0),
                            std::nextafter(1.0, 0.0), 1000.0, -1000.0, dmax_v, -dmax_v, inf, -inf};
  for (double a : sp) {
    check_one(a);
    for (double b : sp) check_pair(a, b);
  }
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> e(-320, 320);
  for (int i = 0; i < 2000000; i++) {
    uint64_t ba = rng(), bb = rng();
    double a, b;
    std::memcpy(&a, &ba, 8);
    std::memcpy(&b, &bb, 8);
    check_one(a);
    check_pair(a, b);
    const double x = std::ldexp(u(rng), e(rng)), y = std::ldexp(u(rng), e(rng));
    check_one(x);
    check_pair(x, y);
    check_pair(x, x);
    check_pair(x, -x);
    check_pair(x, std::nextafter(x, inf));
  }
  std::printf("mismatches %lld\n", g_bad);
  return g_bad == 0 ? 0 : 1;
}
