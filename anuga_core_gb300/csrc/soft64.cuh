// soft64.cuh -- IEEE-754 binary64 addition, subtraction, multiplication,
// division and square root carried out with integer instructions, correctly
// rounded (round to nearest, ties to even), with signed zeros, subnormal
// operands and results, and infinities as IEEE-754 (2008) specifies.  NaN
// results are a quiet NaN (the first NaN operand made quiet, or the default
// NaN for an invalid operation); their payload is not that of any hardware.
//
// Why: GB300 executes FP64 at 1/54 of its FP32 rate (measured over its 152
// SMs: DFMA 525 G op/s, DDIV and DSQRT 70 G op/s), while its integer pipes
// issue several warp instructions per clock per SM.  An exact binary64
// operation built from 32- and 64-bit integer arithmetic therefore runs beside
// the FP64 pipe.  Measured on the same part: division 115 G op/s and square
// root 93 G op/s this way, faster than the FP64 pipe's; addition (276 G op/s)
// and multiplication (384 G op/s) slower, and no faster split between the
// two paths, since both take issue slots.  So the FP64 kernels divide and
// take square roots with these functions and add and multiply on the pipe.  Every non-NaN result is bitwise the
// IEEE result; tests/cpp/check_soft64.cpp checks that on the host against the
// processor's own IEEE arithmetic.
//
// Methods.  Addition and multiplication align or multiply the significands
// exactly in 64- or 128-bit integers, keep a sticky bit for everything shifted
// out, and round once with guard, round and sticky bits (Goldberg, "What every
// computer scientist should know about floating-point arithmetic", 1991).
// Division multiplies by a reciprocal seeded in FP32 and refined by
// Newton-Raphson steps in 64-bit fixed point, then corrects the quotient by
// its exact 128-bit remainder to the truncated quotient, whose remainder gives
// the sticky bit; the square root likewise from an inverse square root
// refined by Newton-Raphson steps, corrected by its exact remainder.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#ifdef __CUDACC__
#define SF_HD __host__ __device__ __forceinline__
#else
#define SF_HD inline
#endif

namespace soft64 {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t EXP_MASK = 0x7ff0000000000000ull;
constexpr uint64_t FRAC = 0x000fffffffffffffull;
constexpr uint64_t HIDDEN = 0x0010000000000000ull;
constexpr uint64_t QUIET = 0x0008000000000000ull;
constexpr uint64_t DEFAULT_NAN = 0x7ff8000000000000ull;

SF_HD uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
SF_HD double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}

SF_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// the high 64 bits of the 128-bit product a * b
SF_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// x >> n with every bit shifted out ORed into bit 0 (n >= 0)
SF_HD uint64_t shr_jam(uint64_t x, int n) {
  if (n <= 0) return x;
  if (n >= 64) return x != 0;
  return (x >> n) | ((x << (64 - n)) != 0);
}

// Round to 53 bits and pack.  The exact result is (-1)^sign * sig * 2^(e - 1085):
// when sig's leading one is at bit 62, e is the result's biased exponent.  sig
// is non-zero with its leading one at bit 62 or below; bit 0 is a sticky bit
// (set when any non-zero bits lay below it).
SF_HD uint64_t round_pack(uint64_t sign, int e, uint64_t sig) {
  const int lz = clz64(sig) - 1;
  if (lz > 0) {                       // leading one to bit 62
    sig <<= lz;
    e -= lz;
  }
  if (e <= 0) {                       // below the normal range: as if e were 1
    sig = shr_jam(sig, 1 - e);
    e = 1;
  }
  const uint64_t low = sig & 0x3ff;   // the 10 bits below the 53-bit significand
  uint64_t r = (sig + 0x200) >> 10;   // add half an ulp, truncate
  if (low == 0x200) r &= ~1ull;       // exactly half: to even
  // r: the significand with its hidden bit at bit 52 (bit 53 when rounding
  // carried, bit 52 clear for a subnormal result); the sum carries into the
  // exponent field where needed
  const uint64_t out = ((uint64_t)(e - 1) << 52) + r;
  if (out >= EXP_MASK) return sign | EXP_MASK;      // overflow: infinity
  return sign | out;
}

// A finite non-zero operand as significand m (leading one at bit 52) and
// biased exponent e (below 1 for subnormal operands).
SF_HD void unpack(uint64_t a, uint64_t& m, int& e) {
  e = (int)((a >> 52) & 0x7ff);
  m = a & FRAC;
  if (e == 0) {
    const int s = clz64(m) - 11;
    m <<= s;
    e = 1 - s;
  } else {
    m |= HIDDEN;
  }
}

SF_HD uint64_t nan_of(uint64_t a, uint64_t b) {
  if ((a & ~SIGN) > EXP_MASK) return a | QUIET;
  if ((b & ~SIGN) > EXP_MASK) return b | QUIET;
  return DEFAULT_NAN;
}

SF_HD uint64_t add_bits(uint64_t a, uint64_t b) {
  const uint64_t aa = a & ~SIGN, ab = b & ~SIGN;
  if (aa >= EXP_MASK || ab >= EXP_MASK) {
    if (aa > EXP_MASK || ab > EXP_MASK) return nan_of(a, b);
    if (aa == EXP_MASK && ab == EXP_MASK) return ((a ^ b) & SIGN) ? DEFAULT_NAN : a;   // inf - inf
    return aa == EXP_MASK ? a : b;
  }
  if (aa == 0) return ab == 0 ? (a & b) : b;        // +0 + -0 = +0
  if (ab == 0) return a;
  uint64_t x = a, y = b;                            // |x| >= |y|
  if (ab > aa) {
    x = b;
    y = a;
  }
  uint64_t mx, my;
  int ex, ey;
  unpack(x, mx, ex);
  unpack(y, my, ey);
  mx <<= 10;                                        // leading ones at bit 62
  my = shr_jam(my << 10, ex - ey);
  uint64_t s;
  if ((x ^ y) & SIGN) {
    s = mx - my;
    if (s == 0) return 0;                           // exact cancellation: +0
  } else {
    s = mx + my;
    if (s >> 63) {
      s = shr_jam(s, 1);
      ex += 1;
    }
  }
  return round_pack(x & SIGN, ex, s);
}

SF_HD uint64_t sub_bits(uint64_t a, uint64_t b) { return add_bits(a, b ^ SIGN); }

SF_HD uint64_t mul_bits(uint64_t a, uint64_t b) {
  const uint64_t sign = (a ^ b) & SIGN;
  const uint64_t aa = a & ~SIGN, ab = b & ~SIGN;
  if (aa >= EXP_MASK || ab >= EXP_MASK) {
    if (aa > EXP_MASK || ab > EXP_MASK) return nan_of(a, b);
    if (aa == 0 || ab == 0) return DEFAULT_NAN;     // inf * 0
    return sign | EXP_MASK;
  }
  if (aa == 0 || ab == 0) return sign;
  uint64_t ma, mb;
  int ea, eb;
  unpack(a, ma, ea);
  unpack(b, mb, eb);
  // ma * (mb << 11) lies in [2^115, 2^117): its high word has the leading
  // one at bit 51 or 52; move it to bit 61 or 62 with the next 10 bits and a
  // sticky bit for the rest
  const uint64_t bb = mb << 11;
  const uint64_t lo = ma * bb;
  const uint64_t hi = mulhi64(ma, bb);
  const uint64_t sig = (hi << 10) | (lo >> 54) | (uint64_t)((lo << 10) != 0);
  return round_pack(sign, ea + eb - 1022, sig);
}

// r ~ 2^127 / d for d in [2^63, 2^64): a 23-bit FP32 seed refined by two
// Newton-Raphson steps r <- r + r (1 - d r / 2^127) in fixed point.  The
// result is within a few units of its last place; the quotient built from it
// is corrected exactly by its remainder.
// FP32 seeds, rounded to nearest whatever the build's FP32 division and
// square root flags (fast approximations, flush to zero) say
SF_HD float recip_rn(float x) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}
SF_HD float sqrt_rn(float x) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(x);
#else
  return sqrtf(x);
#endif
}

SF_HD uint64_t recip64(uint64_t d) {
  const float x = (float)(d >> 40) * (1.0f / 8388608.0f);            // d / 2^63 in [1, 2)
  uint64_t r = (uint64_t)(recip_rn(x) * 2147483520.0f) << 33;        // ~ 2^64 / x, below 2^64
  for (int it = 0; it < 2; it++) {
    const uint64_t t = mulhi64(d, r);            // ~ d r / 2^64 ~ 2^63
    if (t <= (1ull << 63)) r += mulhi64(r, ((1ull << 63) - t) << 1);
    else r -= mulhi64(r, (t - (1ull << 63)) << 1);
  }
  return r;
}

SF_HD uint64_t div_bits(uint64_t a, uint64_t b) {
  const uint64_t sign = (a ^ b) & SIGN;
  const uint64_t aa = a & ~SIGN, ab = b & ~SIGN;
  if (aa >= EXP_MASK || ab >= EXP_MASK) {
    if (aa > EXP_MASK || ab > EXP_MASK) return nan_of(a, b);
    if (aa == EXP_MASK) return ab == EXP_MASK ? DEFAULT_NAN : (sign | EXP_MASK);   // inf / x
    return sign;                                                                    // x / inf
  }
  if (ab == 0) return aa == 0 ? DEFAULT_NAN : (sign | EXP_MASK);                    // x / 0
  if (aa == 0) return sign;
  uint64_t ma, mb;
  int ea, eb;
  unpack(a, ma, ea);
  unpack(b, mb, eb);
  const uint64_t n = ma << 11, d = mb << 11;        // both in [2^63, 2^64)
  const uint64_t r = recip64(d);
  uint64_t q = mulhi64(n, r);                        // ~ 2^63 n / d, in (2^62, 2^64), a few units off
  // the remainder R = 2^63 n - q d in 128 bits (two's complement)
  const uint64_t nh = n >> 1, nl = (n & 1) << 63;
  {
    // one Newton step on the quotient, q += R / d = R r / 2^127, from the
    // top bits of R (|R| < 2^70 here, so R >> 7 fits a signed 64-bit word)
    const uint64_t pl = q * d, ph = mulhi64(q, d);
    const uint64_t rl = nl - pl;
    const uint64_t rh = nh - ph - (uint64_t)(nl < pl);
    const int64_t v = (int64_t)((rh << 57) | (rl >> 7));
    const uint64_t dq = mulhi64(v < 0 ? 0ull - (uint64_t)v : (uint64_t)v, r) >> 56;
    q = v < 0 ? q - dq : q + dq;
  }
  // then to floor(2^63 n / d) exactly: 0 <= R < d
  uint64_t sticky = 0;
  for (int it = 0; it < 4; it++) {
    const uint64_t pl = q * d, ph = mulhi64(q, d);
    const uint64_t rl = nl - pl;
    const uint64_t rh = nh - ph - (uint64_t)(nl < pl);
    if ((int64_t)rh < 0) {                 // remainder negative: q too large
      q -= 1;
    } else if (rh != 0 || rl >= d) {       // remainder at least d: q too small
      q += 1;
    } else {
      sticky = rl != 0;
      break;
    }
  }
  // the quotient is q / 2^63 * 2^(ea - eb), q's leading one at bit 63 or 62
  if (q >> 63) return round_pack(sign, ea - eb + 1023, (q >> 1) | (q & 1) | sticky);
  return round_pack(sign, ea - eb + 1022, q | sticky);
}

// y ~ 2^62 / sqrt(s / 2^64) for s in [2^62, 2^64): an FP32 seed refined by two
// Newton-Raphson steps y <- y + y (1 - x y^2) / 2 in fixed point.
SF_HD uint64_t rsqrt64(uint64_t s) {
  const float x = (float)(s >> 40) * (1.0f / 16777216.0f);          // s / 2^64 in [1/4, 1)
  uint64_t y = (uint64_t)(recip_rn(sqrt_rn(x)) * 1073741824.0f) << 32;   // ~ 2^62 / sqrt(x), at most 2^63
  for (int it = 0; it < 2; it++) {
    const uint64_t t = mulhi64(s, mulhi64(y, y));    // ~ x y^2 * 2^60
    if (t <= (1ull << 60)) y += mulhi64(y, ((1ull << 60) - t) << 3);
    else y -= mulhi64(y, (t - (1ull << 60)) << 3);
  }
  return y;
}

SF_HD uint64_t sqrt_bits(uint64_t a) {
  const uint64_t aa = a & ~SIGN;
  if (aa > EXP_MASK) return a | QUIET;                  // NaN
  if (aa == 0) return a;                                // +0, -0
  if (a & SIGN) return DEFAULT_NAN;                     // negative
  if (aa == EXP_MASK) return a;                         // +inf
  uint64_t m;
  int e;
  unpack(a, m, e);
  int k = e - 1023;                                     // a = (m / 2^52) 2^k
  uint64_t s = m << 10;                                 // s / 2^62 = m / 2^52, in [1, 2)
  if (k & 1) {                                          // an even power of two
    s <<= 1;
    k -= 1;
  }
  // sqrt(a) = sqrt(s * 2^62) / 2^62 * 2^(k/2); r = floor(sqrt(s * 2^62)) in [2^62, 2^63)
  const uint64_t y = rsqrt64(s);
  uint64_t r = mulhi64(s, y) << 1;                      // a few units off
  const uint64_t nh = s >> 2, nl = s << 62;             // s * 2^62
  {
    // one Newton step, r += R / (2 r) = R y / 2^126 with R = s 2^62 - r^2
    // (|R| < 2^70 here: R >> 7 fits a signed 64-bit word)
    const uint64_t ql = r * r, qh = mulhi64(r, r);
    const uint64_t rl = nl - ql;
    const uint64_t rh = nh - qh - (uint64_t)(nl < ql);
    const int64_t v = (int64_t)((rh << 57) | (rl >> 7));
    const uint64_t dr = mulhi64(v < 0 ? 0ull - (uint64_t)v : (uint64_t)v, y) >> 55;
    r = v < 0 ? r - dr : r + dr;
  }
  uint64_t sticky = 0;
  for (int it = 0; it < 4; it++) {
    const uint64_t ql = r * r, qh = mulhi64(r, r);
    if (qh > nh || (qh == nh && ql > nl)) {             // r^2 above: too large
      r -= 1;
      continue;
    }
    const uint64_t tl = ql + 2 * r + 1;                 // (r + 1)^2
    const uint64_t th = qh + (uint64_t)(tl < ql);
    if (th < nh || (th == nh && tl <= nl)) {            // (r + 1)^2 not above: too small
      r += 1;
      continue;
    }
    sticky = (qh != nh || ql != nl);
    break;
  }
  return round_pack(0, k / 2 + 1023, r | sticky);
}

SF_HD double add(double a, double b) { return from_bits(add_bits(bits(a), bits(b))); }
SF_HD double sub(double a, double b) { return from_bits(sub_bits(bits(a), bits(b))); }
SF_HD double mul(double a, double b) { return from_bits(mul_bits(bits(a), bits(b))); }
SF_HD double div(double a, double b) { return from_bits(div_bits(bits(a), bits(b))); }
SF_HD double sqrt(double a) { return from_bits(sqrt_bits(bits(a))); }

}  // namespace soft64
