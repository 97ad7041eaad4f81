// bits.cuh -- float <-> double conversions and the RK2 halving done with
// integer operations on the IEEE-754 bit layouts (sign, biased exponent,
// mantissa), so that the mixed-precision update runs on the integer pipe
// instead of the FP64 pipe (1/54 of the FP32 rate on GB300).
//
// The same source compiles for the host (tests/cpp/check_bits.cpp checks it
// against the IEEE operations it replaces).
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define AGX_BITS __host__ __device__ __forceinline__
#define AGX_BITS_COLD __host__ __device__ __noinline__
#else
#define AGX_BITS inline
#define AGX_BITS_COLD __attribute__((noinline))
#endif

namespace agx {

AGX_BITS uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
AGX_BITS double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
AGX_BITS uint32_t bits_of(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
#endif
}
AGX_BITS float float_of(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}

// float -> double: exact for normal numbers and zero; float subnormals
// become signed zero, infinities and NaNs stay infinities and NaNs.
AGX_BITS double f2d_bits(float f) {
  const uint32_t b = bits_of(f);
  const uint32_t e = (b >> 23) & 0xffu;
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint64_t mant = (uint64_t)(b & 0x7fffffu) << 29;
  const uint64_t ex = (e == 255u) ? 2047ull : (uint64_t)(e + 896u);
  const uint64_t r = (e == 0u) ? sign : (sign | (ex << 52) | mant);
  return double_of(r);
}

// double -> float, rounded to nearest with ties away from zero; results
// below the float normal range become signed zero, above it infinity.  The
// 64-bit magnitude is handled as two 32-bit halves (a 64-bit mask of the
// sign is turned into an FP64 absolute value by the compiler).
AGX_BITS float d2f_bits(double x) {
  const uint64_t b = bits_of(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const uint32_t mlo = lo + (1u << 28);                     // half an ulp of the float mantissa
  const uint32_t mhi = (hi & 0x7fffffffu) + (mlo < lo ? 1u : 0u);
  const int e = (int)(mhi >> 20) - 896;
  if (e <= 0) return float_of(sign);
  if (e >= 255) return float_of(sign | 0x7f800000u);
  return float_of(sign | ((uint32_t)e << 23) | ((mhi & 0xfffffu) << 3) | (mlo >> 29));
}

AGX_BITS bool negative_bits(double x) { return (int64_t)bits_of(x) < 0; }

AGX_BITS_COLD double half_sum_products(double a, double b) { return 0.5 * a + 0.5 * b; }

// 0.5 a + 0.5 b with one FP64 add: halving by decrementing the exponent is
// exact for normal numbers, so the result is bitwise that of the product form
// (which rounds once, after two exact halvings); zero, subnormal and
// non-finite operands take the product form, out of line so that it costs
// nothing where no lane needs it.
AGX_BITS double half_sum(double a, double b) {
  const int ea = (int)((bits_of(a) >> 52) & 0x7ff);
  const int eb = (int)((bits_of(b) >> 52) & 0x7ff);
  const double s = a + b;
  const uint64_t sb = bits_of(s);
  const int es = (int)((sb >> 52) & 0x7ff);
  if (ea > 1 && eb > 1 && es > 1 && es < 0x7ff && ea < 0x7ff && eb < 0x7ff) return double_of(sb - (1ull << 52));
  return half_sum_products(a, b);
}

}  // namespace agx
