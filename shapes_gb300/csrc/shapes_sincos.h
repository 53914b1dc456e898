/*
 * Deterministic sine/cosine pair shared by the CUDA step and by the CPU oracle.
 *
 * The reference builds each body's rotation matrix from libm cos/sin
 * (shapes/src/Physics/Linear.hs:353-357, rotate22 via cosDouble#/sinDouble#).
 * libm is not available on the device and CUDA's sin/cos round differently,
 * so both sides of the parity contract call this one function instead.
 *
 * Method (published, restated here from the mathematics):
 *   - Cody & Waite additive range reduction (W. J. Cody, W. Waite,
 *     "Software Manual for the Elementary Functions", 1980): k = rint(x * 2/pi),
 *     r = x - k*(P1 + P2 + P3) with pi/2 ~ P1 + P2 + P3, P1 and P2 holding
 *     30 significant bits each so that k*P1 and k*P2 are exact for |k| < 2^23;
 *     the remainder is kept as a head + tail pair, split exactly with Knuth's
 *     TwoSum.
 *   - Taylor series of sin and cos on |r| <= pi/4, evaluated by Horner's rule
 *     (terms to r^17 and r^18; truncation below 1e-20 relative), with the
 *     first-order tail corrections sin(h+l) ~ sin h + l cos h and
 *     cos(h+l) ~ cos h - l sin h, and the rounding error of 1 - r^2/2
 *     recovered exactly.
 *   - Quadrant selection by k mod 4.
 * Accuracy is within 1 ulp of the true value for |x| < 1.3e7 rad; beyond that
 * the reduction loses accuracy but stays deterministic.  |x| >= 2^52,
 * infinities and NaN give NaN for both results.
 *
 * Every operation is a single IEEE-754 binary64 add or multiply in source
 * order; callers must compile with contraction disabled (host
 * -ffp-contract=off, device -fmad=false) so that host and device produce
 * identical bits.
 */
#ifndef SHAPES_SINCOS_H
#define SHAPES_SINCOS_H

#if defined(__CUDACC__)
#define SHAPES_HD __host__ __device__ __forceinline__
#else
#define SHAPES_HD static inline
#include <math.h>
#endif

SHAPES_HD void shapes_sincos(double x, double* s_out, double* c_out) {
  const double two_over_pi = 0x1.45f306dc9c883p-1;
  const double P1 = 0x1.921fb54000000p+0;  /* pi/2, first 30 bits  */
  const double P2 = 0x1.10b4611800000p-30; /* next 30 bits          */
  const double P3 = 0x1.313198a2e0370p-61; /* remainder to 53 bits  */
  double ax = x < 0.0 ? -x : x;
  if (!(ax < 0x1p52)) { /* NaN, infinities and huge arguments */
    double nan = 0.0 / 0.0;
    *s_out = nan;
    *c_out = nan;
    return;
  }
  if (ax == 0.0) { /* keeps the sign of a zero argument, as libm does */
    *s_out = x;
    *c_out = 1.0;
    return;
  }
  double k = rint(x * two_over_pi);
  /* r = x - k*pi/2 as an unevaluated sum rh + rl.  k*P1 and k*P2 are exact;
   * t - u is split exactly by TwoSum (Knuth); k*P3 adds a rounded tail. */
  double t = x - k * P1;
  double u = -(k * P2);
  double r1 = t + u;
  double bp = r1 - t;
  double e1 = (t - (r1 - bp)) + (u - bp);
  double rl0 = e1 - k * P3;
  double rh = r1 + rl0;
  double rl = rl0 - (rh - r1);
  long long q = (long long)k;
  double z = rh * rh;
  /* sin r = r - r^3/3! + ... + r^17/17!;  sin(rh + rl) ~ sin rh + rl*cos rh */
  double ps = 0x1.952c77030ad4ap-49;           /* 1/17! */
  ps = -0x1.ae7f3e733b81fp-41 + z * ps;          /* 1/15! */
  ps = 0x1.6124613a86d09p-33 + z * ps;           /* 1/13! */
  ps = -0x1.ae64567f544e4p-26 + z * ps;          /* 1/11! */
  ps = 0x1.71de3a556c734p-19 + z * ps;           /* 1/9!  */
  ps = -0x1.a01a01a01a01ap-13 + z * ps;          /* 1/7!  */
  ps = 0x1.1111111111111p-7 + z * ps;            /* 1/5!  */
  ps = -0x1.5555555555555p-3 + z * ps;           /* 1/3!  */
  double sr = rh + ((rh * z) * ps + rl * (1.0 - 0.5 * z));
  /* cos r = 1 - r^2/2 + r^4/4! - ... + r^18/18!;  cos(rh + rl) ~ cos rh - rl*rh.
   * The rounding error of 1 - r^2/2 is recovered exactly and added back. */
  double pc = -0x1.6827863b97d97p-53;          /* 1/18! */
  pc = 0x1.ae7f3e733b81fp-45 + z * pc;           /* 1/16! */
  pc = -0x1.93974a8c07c9dp-37 + z * pc;          /* 1/14! */
  pc = 0x1.1eed8eff8d898p-29 + z * pc;           /* 1/12! */
  pc = -0x1.27e4fb7789f5cp-22 + z * pc;          /* 1/10! */
  pc = 0x1.a01a01a01a01ap-16 + z * pc;           /* 1/8!  */
  pc = -0x1.6c16c16c16c17p-10 + z * pc;          /* 1/6!  */
  pc = 0x1.5555555555555p-5 + z * pc;            /* 1/4!  */
  double hz = 0.5 * z;
  double wc = 1.0 - hz;
  double cr = wc + ((((1.0 - wc) - hz) + (z * z) * pc) - rh * rl);
  switch ((int)(q & 3)) {
    case 0: *s_out = sr; *c_out = cr; break;
    case 1: *s_out = cr; *c_out = -sr; break;
    case 2: *s_out = -sr; *c_out = -cr; break;
    default: *s_out = -cr; *c_out = sr; break;
  }
}

#endif /* SHAPES_SINCOS_H */
