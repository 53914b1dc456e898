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

}  // namespace shapes
