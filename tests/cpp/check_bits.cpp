// Host check of the integer-pipe conversions of the mixed-precision update
// (anuga_core_gb300/csrc/bits.cuh): f2d_bits against the IEEE conversion for
// every normal float and zero (subnormals give signed zero), d2f_bits against
// a 64-bit restatement of round-to-nearest-ties-away with flush to zero and
// against the IEEE conversion (equal except on exact ties), and half_sum
// against 0.5*a + 0.5*b bit for bit, over special values and random bit
// patterns.  Prints the number of mismatches and exits non-zero on any.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include "../../anuga_core_gb300/csrc/bits.cuh"

using namespace agx;

static float d2f_ref(double x) {      // round |x| to 24 bits, ties away; flush below FLT_MIN
  uint64_t b;
  std::memcpy(&b, &x, 8);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  b &= 0x7fffffffffffffffull;
  b += (1ull << 28);
  const int e = (int)(b >> 52) - 896;
  uint32_t r;
  if (e <= 0) r = sign;
  else if (e >= 255) r = sign | 0x7f800000u;
  else r = sign | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
  float f;
  std::memcpy(&f, &r, 4);
  return f;
}

static bool same(double a, double b) { return std::memcmp(&a, &b, 8) == 0; }
static bool samef(float a, float b) { return std::memcmp(&a, &b, 4) == 0; }

int main() {
  long long bad = 0, ties = 0;
  std::mt19937_64 rng(4242);
  // f2d_bits: every float bit pattern
  for (uint64_t u = 0; u <= 0xffffffffull; u += 7) {
    const uint32_t b = (uint32_t)u;
    float f;
    std::memcpy(&f, &b, 4);
    const double got = f2d_bits(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0) {
      if (!(got == 0.0 && std::signbit(got) == std::signbit(f))) bad++;
    } else if (std::isnan(f)) {
      if (!std::isnan(got)) bad++;
    } else if (!same(got, (double)f)) {
      bad++;
    }
  }
  // d2f_bits and half_sum on random doubles of every magnitude and specials
  const double sp[] = {0.0, -0.0, 1.0, -1.0, std::numeric_limits<double>::denorm_min(),
                       std::numeric_limits<double>::min(), std::numeric_limits<double>::max(),
                       std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                       (double)std::numeric_limits<float>::min(), (double)std::numeric_limits<float>::max(),
                       std::nextafter((double)std::numeric_limits<float>::max(), 1e300)};
  for (double a : sp)
    for (double b : sp) {
      if (!samef(d2f_bits(a), d2f_ref(a))) bad++;
      const double h = half_sum(a, b), r = 0.5 * a + 0.5 * b;
      if (!(same(h, r) || (std::isnan(h) && std::isnan(r)))) bad++;
    }
  std::uniform_int_distribution<int> ex(-1100, 1100);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  for (int i = 0; i < 4000000; i++) {
    uint64_t bb = rng();
    double a;
    std::memcpy(&a, &bb, 8);
    const double x = std::ldexp(u(rng), ex(rng) % 140), y = std::ldexp(u(rng), ex(rng));
    for (double v : {a, x, y}) {
      if (std::isnan(v)) continue;
      const float g = d2f_bits(v);
      if (!samef(g, d2f_ref(v))) bad++;
      const double av = std::fabs(v);
      if (av >= (double)std::numeric_limits<float>::min() && av <= (double)std::numeric_limits<float>::max()) {
        const float ieee = (float)v;
        if (!samef(g, ieee)) {
          // only an exact tie may round differently (away from zero vs to even)
          const double lo = (double)std::nextafter(ieee, 0.0f), hi2 = (double)ieee;
          const double mid = 0.5 * (lo + hi2);
          if (v == mid || v == 0.5 * (hi2 + (double)std::nextafter(ieee, ieee * 2.0f))) ties++;
          else bad++;
        }
      }
    }
    const double h = half_sum(x, y), r = 0.5 * x + 0.5 * y;
    if (!same(h, r)) bad++;
    const double h2 = half_sum(a, y), r2 = 0.5 * a + 0.5 * y;
    if (!(same(h2, r2) || (std::isnan(h2) && std::isnan(r2)))) bad++;
  }
  std::printf("mismatches %lld (exact ties rounded away: %lld)\n", bad, ties);
  return bad == 0 ? 0 : 1;
}
