/*
 * Exact binary64 helpers that keep work off GB300's narrow FP64 pipe.
 *
 * The FP64 pipe retires about 0.05 warp-instructions per clock per SM and
 * each FP64 instruction (including DSETP comparisons) is charged for all 32
 * lanes, while integer instructions issue roughly a hundred times faster.
 * Every helper here returns exactly what the plain IEEE-754 operation it
 * replaces returns, for every input.
 */
#pragma once
#include <cstdint>

namespace shapes {

/* Order-preserving key of a binary64: for non-NaN a, b,
 * a < b  <=>  okey(a) < okey(b), and a == b <=> okey(a) == okey(b)
 * (-0 and +0 map to the same key). */
__device__ __forceinline__ uint64_t okey(double d) {
  uint64_t u = (uint64_t)__double_as_longlong(d);
  if (u == 0x8000000000000000ull) u = 0;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ bool nan_bits(double x) {
  return ((uint64_t)__double_as_longlong(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

/* a <= b and a < b as IEEE comparisons (false when either is NaN). */
__device__ __forceinline__ bool f_le(double a, double b) {
  return !nan_bits(a) && !nan_bits(b) && okey(a) <= okey(b);
}
__device__ __forceinline__ bool f_lt(double a, double b) {
  return !nan_bits(a) && !nan_bits(b) && okey(a) < okey(b);
}

/* Finite (not infinite, not NaN). */
__device__ __forceinline__ bool finite_bits(double x) {
  return ((uint64_t)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

/* 0.0 * x for finite x: a zero with x's sign. */
__device__ __forceinline__ double signed_zero(double x) {
  return __longlong_as_double(__double_as_longlong(x) & (long long)0x8000000000000000ull);
}

/* x + z for finite x and a signed zero z: x unless x is a zero, and the sum
 * of two zeros is -0 only when both are -0 (round to nearest). */
__device__ __forceinline__ double add_zero(double x, double z) {
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  if (ux & 0x7fffffffffffffffull) return x;
  return __longlong_as_double((long long)(ux & (uint64_t)__double_as_longlong(z)));
}

/* x + 0.0: only -0 changes (to +0); NaN stays NaN. */
__device__ __forceinline__ double plus_zero(double x) {
  return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}

__device__ __forceinline__ int exp_field(double x) {
  return (int)(((uint64_t)__double_as_longlong(x) >> 52) & 0x7ff);
}

/* |x| < 2^500: finite and far from overflow. */
__device__ __forceinline__ bool small_mag(double x) { return exp_field(x) < 1523; }

/* |x| < 2. */
__device__ __forceinline__ bool below_two(double x) { return exp_field(x) < 1024; }

/* 2^-500 <= |b| < 2^500: denominators whose reciprocal is used by div_rn. */
__device__ __forceinline__ bool recip_ok(double b) {
  const int e = exp_field(b);
  return e >= 523 && e < 1523;
}

/* a / b, correctly rounded (round to nearest even), given y = RN(1/b) and
 * recip_ok(b).  Markstein's theorem (P. Markstein, "IA-64 and Elementary
 * Functions", 2000, Thm 8.10; the basis of the IA-64 division sequences): if
 * y is within half an ulp of 1/b and q is within one ulp of a/b, then
 * r = a - b q is exact when computed with one fused multiply-add, and
 * RN(q + r y) is the correctly rounded quotient.  q0 = RN(a y) is within one
 * ulp of a/b.  The fast path is taken when a is a normal number with
 * 2^-400 <= |a| < 2^400, so nothing overflows or underflows (|q| stays
 * within 2^+-900 and |r| above 2^-460); zeros, NaN, infinities and extreme
 * magnitudes use the hardware division, and so does any b outside
 * recip_ok (signalled by y == 0).  Three dependent FP64 instructions
 * replace the division's longer sequence.  Explicit __fma_rn: the fused
 * operations here are part of this algorithm, not contractions of the
 * reference's expressions. */
__device__ __forceinline__ double div_rn(double a, double b, double y) {
  const int ea = exp_field(a);
  if (ea >= 623 && ea < 1423 && __double_as_longlong(y) != 0) {
    const double q0 = __dmul_rn(a, y);
    const double r = __fma_rn(-q0, b, a);
    return __fma_rn(r, y, q0);
  }
  return a / b;
}

/* a * b in binary64, round to nearest even, computed on the integer pipe.
 * Measured on GB300: 4.8e11 of these per second against 5.3e11 hardware
 * products, on a separate pipe, so a kernel bound by FP64 throughput at high
 * occupancy gains by moving part of its products here (a latency-bound
 * dependency chain loses: the sequence is about 30 instructions long).  Fast path: both operands normal with biased exponents in
 * [512, 1534] (the product is then normal, or overflows to infinity exactly
 * as IEEE rounding does), or one operand a zero and the other finite (a
 * signed zero).  The 106-bit product of the 53-bit significands comes from
 * four 32 x 32 -> 64 products; the result keeps 53 bits, rounds on the next
 * bit with the rest as sticky (ties to even), and a carry out of the
 * significand moves into the exponent field.  Everything else (subnormals,
 * extreme exponents, infinities, NaN) uses the hardware multiply. */
__device__ __forceinline__ double mul_rn_int(double a, double b) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  if (ea - 512u <= 1022u && eb - 512u <= 1022u) {
    const uint64_t ma = (ua & 0x000fffffffffffffull) | 0x0010000000000000ull;
    const uint64_t mb = (ub & 0x000fffffffffffffull) | 0x0010000000000000ull;
    const uint64_t lo = ma * mb;
    const uint64_t hi = __umul64hi(ma, mb); /* product in [2^104, 2^106): hi in [2^40, 2^42) */
    const uint32_t top = (uint32_t)(hi >> 41);
    const uint32_t sh = 52u + top;
    const uint64_t m = (hi << (64u - sh)) | (lo >> sh); /* 53 bits, leading one at bit 52 */
    const uint64_t rem = lo & ((1ull << sh) - 1ull);
    const uint64_t half = 1ull << (sh - 1u);
    const uint64_t up = (rem > half || (rem == half && (m & 1ull))) ? 1ull : 0ull;
    const uint64_t e = (uint64_t)(ea + eb + top) - 1024ull; /* biased exponent - 1 */
    return __longlong_as_double((long long)(((e << 52) + m + up) | sign));
  }
  if (((ua << 1) == 0 && eb < 0x7ffu) || ((ub << 1) == 0 && ea < 0x7ffu))
    return __longlong_as_double((long long)sign);
  return __dmul_rn(a, b);
}

/* a + b in binary64, round to nearest even, computed on the integer pipe
 * (host and device: the same integer steps, so the host can check it against
 * its own hardware addition).  Fast path: both operands normal with biased
 * exponents in [64, 1982]; the result is then normal (an exact cancellation
 * gives +0, as IEEE round-to-nearest does), and nothing overflows.
 * Algorithm (the textbook one with guard bits and a sticky bit): order the
 * operands by magnitude; significands with the implicit one, shifted left by
 * 10 so that the leading one sits at bit 62 and 10 guard bits lie below the
 * last place; the smaller is shifted right by the exponent difference with
 * every bit shifted out ORed into bit 0 (sticky); add the significands for
 * equal signs (a carry out of bit 62 shifts right by one, again keeping a
 * sticky bit), subtract them otherwise (renormalising left by the leading
 * zero count); keep 53 bits and round on the 10 bits below, ties to even.
 * When a sticky bit was set, the sum is an odd number of guard units and the
 * exact value lies within one unit of it, so it falls on the same side of the
 * rounding midpoint (an even number of units) and never on it.  The rounding
 * carry moves into the exponent field by integer addition.  Anything else
 * (zeros, subnormals, extreme exponents, infinities, NaN) uses the hardware
 * addition. */
__host__ __device__ __forceinline__ double add_rn_int(double a, double b) {
#if defined(__CUDA_ARCH__)
  uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
#else
  uint64_t ua, ub;
  __builtin_memcpy(&ua, &a, 8);
  __builtin_memcpy(&ub, &b, 8);
#endif
  uint64_t xa = ua & 0x7fffffffffffffffull, xb = ub & 0x7fffffffffffffffull;
  const uint32_t ea0 = (uint32_t)(xa >> 52), eb0 = (uint32_t)(xb >> 52);
  if (ea0 - 64u <= 1918u && eb0 - 64u <= 1918u) {
    if (xa < xb) { /* |a| >= |b| from here on */
      const uint64_t t = ua;
      ua = ub;
      ub = t;
      const uint64_t tx = xa;
      xa = xb;
      xb = tx;
    }
    const uint32_t ea = (uint32_t)(xa >> 52), d = ea - (uint32_t)(xb >> 52);
    const uint64_t ma = ((xa & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
    uint64_t mb = ((xb & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
    if (d >= 63u) {
      mb = 1ull; /* only the sticky bit is left */
    } else if (d) {
      const uint64_t sticky = (mb << (64u - d)) != 0ull ? 1ull : 0ull;
      mb = (mb >> d) | sticky;
    }
    uint64_t sm;
    int64_t e = (int64_t)ea;
    if (((ua ^ ub) >> 63) == 0ull) {
      sm = ma + mb;
      if (sm >> 63) {
        sm = (sm >> 1) | (sm & 1ull);
        e += 1;
      }
    } else {
      sm = ma - mb;
      if (sm == 0ull) return 0.0;
#if defined(__CUDA_ARCH__)
      const int lz = __clzll((long long)sm) - 1;
#else
      const int lz = __builtin_clzll(sm) - 1;
#endif
      sm <<= lz;
      e -= lz;
    }
    const uint64_t m = sm >> 10, rem = sm & 0x3ffull;
    const uint64_t up = (rem > 0x200ull || (rem == 0x200ull && (m & 1ull))) ? 1ull : 0ull;
    const uint64_t r = ((((uint64_t)(e - 1)) << 52) + m + up) | (ua & 0x8000000000000000ull);
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)r);
#else
    double out;
    __builtin_memcpy(&out, &r, 8);
    return out;
#endif
  }
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

}  // namespace shapes
