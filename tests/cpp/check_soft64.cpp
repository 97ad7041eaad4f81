// Host check of the integer-only binary64 arithmetic (anuga_core_gb300/csrc/
// soft64.cuh) against the processor's IEEE-754 arithmetic (round to nearest,
// no contraction): add, sub, mul, div and sqrt on special values and their
// neighbours, on random bit patterns (every exponent, subnormals, infinities,
// NaNs), on random values with nearby exponents (cancellation, ties) and on
// subnormal results.  A NaN result only has to be a NaN.  Prints the number of
// mismatches per operation and exits non-zero on any.
//   check_soft64 [cases per operation and class]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#include "../../anuga_core_gb300/csrc/soft64.cuh"

static uint64_t B(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
}
static double D(uint64_t b) {
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

static long long mism[5];
static long long shown = 0;

static void check(int op, double a, double b) {
  volatile double va = a, vb = b;    // the compiler must not fold the reference
  double ref, got;
  switch (op) {
    case 0: ref = va + vb; got = soft64::add(a, b); break;
    case 1: ref = va - vb; got = soft64::sub(a, b); break;
    case 2: ref = va * vb; got = soft64::mul(a, b); break;
    case 3: ref = va / vb; got = soft64::div(a, b); break;
    default: ref = std::sqrt(va); got = soft64::sqrt(a); break;
  }
  const bool ok = (std::isnan(ref) && std::isnan(got)) || B(ref) == B(got);
  if (!ok) {
    mism[op]++;
    if (shown++ < 20)
      std::printf("op %d a=%016llx b=%016llx ref=%016llx got=%016llx\n", op, (unsigned long long)B(a),
                  (unsigned long long)B(b), (unsigned long long)B(ref), (unsigned long long)B(got));
  }
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? std::atoll(argv[1]) : 1000000;
  std::mt19937_64 rng(20261204);
  std::vector<double> special = {0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, 1.5, 0.1, 1e308, -1e308, 1e-308,
                                 4.9406564584124654e-324, -4.9406564584124654e-324, 2.2250738585072014e-308,
                                 2.2250738585072009e-308, 1.7976931348623157e308, INFINITY, -INFINITY, NAN,
                                 9007199254740993.0, 4503599627370496.0, 0.9999999999999999, 1.0000000000000002};
  const size_t ns = special.size();
  for (size_t i = 0; i < ns; i++) {       // the specials and their neighbours
    const double x = special[i];
    special.push_back(std::nextafter(x, INFINITY));
    special.push_back(std::nextafter(x, -INFINITY));
  }
  for (int op = 0; op < 5; op++)
    for (double a : special)
      for (double b : special) check(op, a, b);
  std::uniform_int_distribution<uint64_t> u64;
  std::uniform_int_distribution<int> sh(0, 63);
  {  // significands at the ends of their range (reciprocal and root estimates at their worst)
    std::vector<uint64_t> m = {0, 1, 2, 3, 0xfffffffffffffull, 0xffffffffffffeull, 0x8000000000000ull,
                               0x7ffffffffffffull, 0x0000000000fffull, 0xfff0000000000ull};
    for (int k = 0; k < 40; k++) m.push_back(u64(rng) & 0xfffffffffffffull);
    for (uint64_t ma : m)
      for (uint64_t mb : m)
        for (int ea : {1, 1022, 1023, 1024, 2000})
          for (int eb : {1, 1023, 1046}) {
            const double a = D(((uint64_t)ea << 52) | ma), b = D(((uint64_t)eb << 52) | mb);
            for (int op = 0; op < 5; op++) check(op, a, b);
            check(3, D(ma), b);          // subnormal numerators
            check(4, D(ma), 0.0);
          }
  }
  for (long long i = 0; i < n; i++) {
    // random bit patterns
    const double a = D(u64(rng)), b = D(u64(rng));
    for (int op = 0; op < 5; op++) check(op, a, b);
    // nearby exponents (cancellation, carries, ties)
    const uint64_t ab = u64(rng);
    const int de = (int)(u64(rng) % 70) - 35;
    uint64_t bb = (u64(rng) & 0x800fffffffffffffull) | (((ab >> 52 & 0x7ff) + de) & 0x7ff) << 52;
    if ((u64(rng) & 7) == 0) bb = (ab & ~0xffull) | (u64(rng) & 0xff);      // almost equal magnitudes
    check(0, D(ab), D(bb));
    check(1, D(ab), D(bb));
    // moderate values whose products and quotients may round to ties
    const double c = (double)(int64_t)(u64(rng) >> sh(rng)) * std::ldexp(1.0, (int)(u64(rng) % 200) - 100);
    const double d = (double)(int64_t)(u64(rng) >> sh(rng) | 1) * std::ldexp(1.0, (int)(u64(rng) % 200) - 100);
    for (int op = 0; op < 5; op++) check(op, c, d);
    // results near and below the normal range
    const double e = std::ldexp((double)(u64(rng) >> 11) / 9007199254740992.0 + 0.5, -(int)(u64(rng) % 60) - 990);
    const double f = std::ldexp((double)(u64(rng) >> 11) / 9007199254740992.0 + 0.5, -(int)(u64(rng) % 60));
    check(2, e, f);
    check(3, e, 1.0 / f);
    check(0, e, -e * (1.0 + std::ldexp(1.0, -(int)(u64(rng) % 52))));
  }
  long long total = 0;
  const char* names[5] = {"add", "sub", "mul", "div", "sqrt"};
  for (int op = 0; op < 5; op++) {
    std::printf("%s mismatches %lld\n", names[op], mism[op]);
    total += mism[op];
  }
  std::printf("mismatches %lld\n", total);
  return total ? 1 : 0;
}
