/*
 * Correctly rounded sine/cosine pair, shared by the CUDA step and the CPU oracle.
 *
 * The reference builds each body's rotation matrix from libm cos/sin
 * (shapes/src/Physics/Linear.hs:353-357, rotate22 via cosDouble#/sinDouble#).
 * libm has no device version and CUDA's sin/cos round differently, so both
 * sides of the parity contract call this function instead.  It returns
 * sin(x) and cos(x) correctly rounded to nearest (ties to even) for every
 * finite x, so it agrees with any libm wherever that libm is correctly
 * rounded (glibc's sin/cos are, on all but a tiny fraction of arguments).
 * Because the result is the unique correctly rounded value, the host and
 * device builds give identical bits by construction.
 *
 * Method (Ziv's strategy: a fast phase with a rounding test, then an
 * accurate phase for the rare arguments the test cannot decide):
 *   - Fast phase, |x| < 2^16: N = rint(|x| 512/pi) and r = |x| - N pi/512 as
 *     an unevaluated double-double rh + rl, by Cody & Waite's reduction with
 *     pi/512 split in four parts (the first two of 29 bits, so N*P1 and N*P2
 *     are exact) and exact TwoSum/TwoProduct steps (Knuth; Dekker, with FMA).
 *     |r| <= pi/1024.  With a = N pi/512 = q pi/2 + i pi/512, sin a and cos a
 *     come from a 257-entry double-double table of sin(i pi/512), and
 *     sin(a + r) = sin a cos r + cos a sin r, cos(a + r) = cos a cos r -
 *     sin a sin r, with cos r - 1 and sin r - r from their Taylor series (to
 *     r^6 and r^7; truncation below 2^-80 relative).  The result is a
 *     double-double hi + lo with relative error below 2^-67 (checked on 10^8
 *     arguments against the accurate phase); if hi + lo -/+ 2^-65 |hi| round
 *     to the same double, that double is the correctly rounded result.
 *   - Accurate phase (the test failed, |x| >= 2^16, or r nearly cancelled):
 *     128-bit fixed-point arithmetic on the integer pipe.  Payne & Hanek's
 *     reduction multiplies the 53-bit significand by a 320-bit window of 2/pi
 *     (1280 bits stored), giving the quadrant and the reduced fraction with at
 *     least 255 bits below the binary point; r = f pi/2 is normalised to a
 *     128-bit significand; sin r = r P_s(r^2) and cos r = P_c(r^2) are summed
 *     by Horner's rule in Q1.127 (Taylor series to r^33 and r^32); the
 *     128-bit results (relative error below 2^-120) are rounded to nearest.
 *   - |x| < 2^-27: sin x = x and cos x = 1 exactly rounded; NaN and
 *     infinities give NaN for both.
 * The constants (tables, 2/pi, pi/2, pi/512 split, 1/n!) are generated with
 * exact integer arithmetic by gen_sincos_tables.py into shapes_sincos_tables.h.
 *
 * The explicit fma() calls are part of the algorithm (exact product errors);
 * every other operation is a single IEEE-754 binary64 add or multiply, so
 * callers may compile with contraction disabled (host -ffp-contract=off,
 * device -fmad=false) without changing any result.
 */
#ifndef SHAPES_SINCOS_H
#define SHAPES_SINCOS_H

#include <stdint.h>
#include <string.h>

#include "shapes_sincos_tables.h"

#if defined(__CUDACC__)
#define SHAPES_HD __host__ __device__ __forceinline__
#define SHAPES_HD_NOINLINE static __host__ __device__ __noinline__
#else
#define SHAPES_HD static inline
#define SHAPES_HD_NOINLINE static
#include <math.h>
#endif

typedef unsigned __int128 shapes_u128;
typedef struct {
  double s, c;
} shapes_sc_pair;

static const double shapes_sin_tab_h[514] = SHAPES_SIN_TABLE;
static const uint64_t shapes_two_over_pi_h[20] = SHAPES_TWO_OVER_PI_WORDS;
static const uint64_t shapes_inv_fact_h[68] = SHAPES_INV_FACT_Q127;
#if defined(__CUDACC__)
static __device__ const double shapes_sin_tab_d[514] = SHAPES_SIN_TABLE;
static __device__ const uint64_t shapes_two_over_pi_d[20] = SHAPES_TWO_OVER_PI_WORDS;
static __constant__ uint64_t shapes_inv_fact_d[68] = SHAPES_INV_FACT_Q127;
#endif

SHAPES_HD double shapes_sc_tab(int k) {
#if defined(__CUDA_ARCH__)
  return __ldg(&shapes_sin_tab_d[k]);
#else
  return shapes_sin_tab_h[k];
#endif
}
SHAPES_HD uint64_t shapes_sc_2opi(int k) {
#if defined(__CUDA_ARCH__)
  return shapes_two_over_pi_d[k];
#else
  return shapes_two_over_pi_h[k];
#endif
}
SHAPES_HD shapes_u128 shapes_sc_invfact(int n) {
#if defined(__CUDA_ARCH__)
  return ((shapes_u128)shapes_inv_fact_d[2 * n] << 64) | shapes_inv_fact_d[2 * n + 1];
#else
  return ((shapes_u128)shapes_inv_fact_h[2 * n] << 64) | shapes_inv_fact_h[2 * n + 1];
#endif
}

SHAPES_HD uint64_t shapes_sc_bits(double x) {
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
}
SHAPES_HD double shapes_sc_from_bits(uint64_t u) {
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
}
SHAPES_HD int shapes_sc_clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

/* High 128 bits of a 128 x 128-bit product. */
SHAPES_HD shapes_u128 shapes_sc_mulhi(shapes_u128 a, shapes_u128 b) {
  const uint64_t a1 = (uint64_t)(a >> 64), a0 = (uint64_t)a, b1 = (uint64_t)(b >> 64), b0 = (uint64_t)b;
  const shapes_u128 p00 = (shapes_u128)a0 * b0, p01 = (shapes_u128)a0 * b1;
  const shapes_u128 p10 = (shapes_u128)a1 * b0, p11 = (shapes_u128)a1 * b1;
  const shapes_u128 mid = (p00 >> 64) + (uint64_t)p01 + (uint64_t)p10; /* < 3 * 2^64 */
  return p11 + (p01 >> 64) + (p10 >> 64) + (mid >> 64);
}

SHAPES_HD int shapes_sc_clz128(shapes_u128 v) {
  const uint64_t h = (uint64_t)(v >> 64);
  return h ? shapes_sc_clz64(h) : 64 + shapes_sc_clz64((uint64_t)v);
}

/* Normalises the 256-bit product a*b (nonzero, top bit at 128 or above) to
 * a 128-bit significand with its top bit set (truncated); adds the shift to *e. */
SHAPES_HD shapes_u128 shapes_sc_norm_prod(shapes_u128 a, shapes_u128 b, int* e) {
  const shapes_u128 hi = shapes_sc_mulhi(a, b);
  const shapes_u128 lo = a * b;
  const int lz = shapes_sc_clz128(hi);
  *e += 128 - lz;
  return lz ? (hi << lz) | (lo >> (128 - lz)) : hi;
}

/* Rounds S 2^e (S in [2^127, 2^128)) to the nearest double (the results of
 * this function are far from the subnormal and overflow ranges). */
SHAPES_HD double shapes_sc_round(shapes_u128 S, int e) {
  uint64_t m = (uint64_t)(S >> 75); /* 53 bits */
  const shapes_u128 rem = S & ((((shapes_u128)1) << 75) - 1);
  const shapes_u128 half = ((shapes_u128)1) << 74;
  if (rem > half || (rem == half && (m & 1))) m += 1;
  e += 75;
  if (m >> 53) {
    m >>= 1;
    e += 1;
  }
  const uint64_t be = (uint64_t)(e + 52 + 1023);
  return shapes_sc_from_bits((be << 52) | (m & ((1ull << 52) - 1)));
}

/* Accurate phase: sin x and cos x for a finite x with |x| >= 2^-27, from
 * 128-bit fixed-point arithmetic (see the header comment). */
SHAPES_HD_NOINLINE shapes_sc_pair shapes_sincos_accurate_v(double x) {
  const uint64_t bits = shapes_sc_bits(x);
  const int neg = (int)(bits >> 63);
  const uint64_t M = (bits & ((1ull << 52) - 1)) | (1ull << 52);
  const int E = (int)((bits >> 52) & 0x7ff) - 1075; /* |x| = M 2^E */
  int q = 0, rneg = 0;
  shapes_u128 R;
  int eR;
  const double ax = neg ? -x : x;
  if (ax < 0x1.921fb54442d18p-1) { /* |x| < pi/4: r = |x| */
    R = (shapes_u128)M << 75;
    eR = E - 75;
  } else {
    /* Payne-Hanek: ACC = M * (words k0 .. k0+4 of 2/pi), binary point at
     * bit p = 64 (k0 + 5) - E; words before k0 only add multiples of 4. */
    const int k0 = E >= 2 ? (E - 2) / 64 : 0;
    uint64_t A[6] = {0, 0, 0, 0, 0, 0};
    for (int t = 0; t < 5; ++t) {
      const shapes_u128 P = (shapes_u128)M * shapes_sc_2opi(k0 + t);
      int idx = 4 - t;
      shapes_u128 acc = (shapes_u128)A[idx] + (uint64_t)P;
      A[idx] = (uint64_t)acc;
      acc = (acc >> 64) + (shapes_u128)A[idx + 1] + (uint64_t)(P >> 64);
      A[idx + 1] = (uint64_t)acc;
      for (int w = idx + 2; w < 6; ++w) {
        acc = (acc >> 64) + A[w];
        A[w] = (uint64_t)acc;
      }
    }
    const int p = 64 * (k0 + 5) - E; /* 255 <= p <= 374 */
    /* integer part mod 4: bits p and p + 1 (p + 1 <= 375 < 384) */
    q = (int)((A[p / 64] >> (p % 64)) & 1) | (int)(((A[(p + 1) / 64] >> ((p + 1) % 64)) & 1) << 1);
    /* shift the fraction (bits below p) to the top of a 384-bit number G */
    const int sh = 384 - p; /* 10 .. 129 */
    uint64_t G[6];
    {
      const int ws = sh / 64, bs = sh % 64;
      for (int w = 5; w >= 0; --w) {
        const int src = w - ws;
        uint64_t v = 0;
        if (src >= 0) {
          v = A[src] << bs;
          if (bs && src - 1 >= 0) v |= A[src - 1] >> (64 - bs);
        }
        G[w] = v;
      }
    }
    if (G[5] >> 63) { /* fraction >= 1/2: next quadrant, f = fraction - 1 */
      q = (q + 1) & 3;
      rneg = 1;
      unsigned carry = 1;
      for (int w = 0; w < 6; ++w) {
        const uint64_t v = ~G[w];
        G[w] = v + carry;
        carry = carry && G[w] == 0;
      }
    }
    int top = 5;
    while (top > 0 && G[top] == 0) --top;
    if (G[top] == 0) { /* cannot happen for a double (pi is irrational) */
      R = 0;
      eR = -1000;
    } else {
      const int lz = shapes_sc_clz64(G[top]);
      /* 128 bits starting at the leading one */
      uint64_t h1 = G[top] << lz, h0 = 0;
      if (lz && top >= 1) h1 |= G[top - 1] >> (64 - lz);
      if (top >= 1) h0 = G[top - 1] << lz;
      if (lz && top >= 2) h0 |= G[top - 2] >> (64 - lz);
      const shapes_u128 F = ((shapes_u128)h1 << 64) | h0;
      /* |f| = F 2^(eF),  eF = 64 (top + 1) - lz - 128 - 384 */
      const int eF = 64 * (top + 1) - lz - 128 - 384;
      const shapes_u128 PIO2 = ((shapes_u128)SHAPES_PIO2_Q126_HI << 64) | SHAPES_PIO2_Q126_LO;
      eR = eF - 126;
      R = shapes_sc_norm_prod(F, PIO2, &eR);
    }
  }
  /* r = (-1)^rneg R 2^eR, |r| <= pi/4.  u = r^2 in Q0.128. */
  shapes_u128 u = 0;
  {
    const int shift = -(2 * eR + 128); /* >= 128 */
    const shapes_u128 r2 = shapes_sc_mulhi(R, R); /* R^2 >> 128 */
    if (shift - 128 < 128) u = r2 >> (shift - 128);
  }
  shapes_u128 ps = shapes_sc_invfact(33), pc = shapes_sc_invfact(32);
  for (int k = 15; k >= 0; --k) {
    ps = shapes_sc_invfact(2 * k + 1) - shapes_sc_mulhi(u, ps);
    pc = shapes_sc_invfact(2 * k) - shapes_sc_mulhi(u, pc);
  }
  double sr = 0.0, cr;
  if (R != 0) {
    int eS = eR - 127;
    const shapes_u128 S = shapes_sc_norm_prod(R, ps, &eS); /* |sin r| */
    sr = shapes_sc_round(S, eS);
    if (rneg) sr = -sr;
  }
  {
    const int lz = shapes_sc_clz128(pc);
    cr = shapes_sc_round(pc << lz, -127 - lz);
  }
  double s, c;
  switch (q) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
  }
  shapes_sc_pair out;
  out.s = neg ? -s : s;
  out.c = c;
  return out;
}

SHAPES_HD void shapes_sincos_accurate(double x, double* s_out, double* c_out) {
  const shapes_sc_pair r = shapes_sincos_accurate_v(x);
  *s_out = r.s;
  *c_out = r.c;
}

/* Fast phase for 2^-27 <= |x| < 2^16: sin x ~ sh + sl and cos x ~ ch + cl
 * (each pair renormalised, relative error below 2^-67).  Returns 0 when the
 * reduced argument nearly cancelled (the accurate phase must be used). */
SHAPES_HD int shapes_sincos_fast2(double x, double& sh, double& sl, double& ch, double& cl) {
  const double ax = fabs(x);
  const double N = rint(ax * SHAPES_512_OVER_PI);
  /* Cody-Waite: r = ax - N (P1 + P2 + P3 + P4) = rh + rl */
  const double t1 = ax - N * SHAPES_PI512_P1; /* exact */
  const double t2 = N * SHAPES_PI512_P2;      /* exact */
  const double s1 = t1 - t2;
  const double b1 = s1 - t1;
  const double e1 = (t1 - (s1 - b1)) + (-t2 - b1);
  const double p3h = N * SHAPES_PI512_P3;
  const double p3l = fma(N, SHAPES_PI512_P3, -p3h);
  const double u1 = s1 - p3h;
  const double b2 = u1 - s1;
  const double v1 = (s1 - (u1 - b2)) + (-p3h - b2);
  const double lo = ((e1 + v1) - p3l) - N * SHAPES_PI512_P4;
  const double rh = u1 + lo;
  const double rl = lo - (rh - u1);
  if (N != 0.0 && fabs(rh) < 0x1p-40) return 0;
  const int n = (int)N;
  const int q = (n >> 8) & 3, i = n & 255;
  const double sah = shapes_sc_tab(2 * i), sal = shapes_sc_tab(2 * i + 1);
  const double cah = shapes_sc_tab(2 * (256 - i)), cal = shapes_sc_tab(2 * (256 - i) + 1);
  const double z = rh * rh;
  /* cos r - 1 and sin r - rh (Taylor; |r| <= pi/1024) */
  const double cm1 = z * (-0.5 + z * (0x1.5555555555555p-5 + z * -0x1.6c16c16c16c17p-10));
  const double sm = (rh * z) * (-0x1.5555555555555p-3 + z * (0x1.1111111111111p-7 + z * -0x1.a01a01a01a01ap-13));
  const double cc = cm1 - rh * rl;
  const double rs = rl + sm;
  /* sin(a + r) = sa + (sa cc + ca rh + ca rs) */
  const double ph = cah * rh;
  const double pl = fma(cah, rh, -ph);
  double Sh = sah + ph;
  double bs = Sh - sah;
  const double Se = (sah - (Sh - bs)) + (ph - bs);
  double Sl = Se + (pl + (sal + (cal * rh + (sah * cc + cah * rs))));
  /* cos(a + r) = ca + (ca cc - sa rh - sa rs) */
  const double qh = sah * rh;
  const double ql = fma(sah, rh, -qh);
  double Ch = cah - qh;
  double bc = Ch - cah;
  const double Ce = (cah - (Ch - bc)) + (-qh - bc);
  double Cl = Ce + (-ql + (cal + (-(sal * rh) + (cah * cc - sah * rs))));
  /* renormalise (Fast2Sum) */
  double t = Sh + Sl;
  Sl = Sl - (t - Sh);
  Sh = t;
  t = Ch + Cl;
  Cl = Cl - (t - Ch);
  Ch = t;
  double s0, s1_, c0, c1;
  switch (q) {
    case 0: s0 = Sh; s1_ = Sl; c0 = Ch; c1 = Cl; break;
    case 1: s0 = Ch; s1_ = Cl; c0 = -Sh; c1 = -Sl; break;
    case 2: s0 = -Sh; s1_ = -Sl; c0 = -Ch; c1 = -Cl; break;
    default: s0 = -Ch; s1_ = -Cl; c0 = Sh; c1 = Sl; break;
  }
  if (x < 0.0) {
    s0 = -s0;
    s1_ = -s1_;
  }
  sh = s0;
  sl = s1_;
  ch = c0;
  cl = c1;
  return 1;
}

SHAPES_HD int shapes_sincos_fast(double x, double out[4]) {
  return shapes_sincos_fast2(x, out[0], out[1], out[2], out[3]);
}

/* 1 when every value within 2^-65 |hi| of hi + lo rounds to hi + lo's nearest double. */
SHAPES_HD int shapes_sc_decided(double hi, double lo) {
  const double e = fabs(hi) * 0x1p-65;
  return hi + (lo + e) == hi + (lo - e);
}

SHAPES_HD void shapes_sincos(double x, double* s_out, double* c_out) {
  const double ax = fabs(x);
  if (!(ax < 0x1p16)) {
    if (!(ax <= 0x1.fffffffffffffp+1023)) { /* NaN and infinities */
      const double nan = 0.0 / 0.0;
      *s_out = nan;
      *c_out = nan;
      return;
    }
    const shapes_sc_pair r = shapes_sincos_accurate_v(x);
    *s_out = r.s;
    *c_out = r.c;
    return;
  }
  if (ax < 0x1p-27) { /* sin x = x, cos x = 1 after rounding (keeps the sign of a zero) */
    *s_out = x;
    *c_out = 1.0;
    return;
  }
  double sh, sl, ch, cl;
  if (shapes_sincos_fast2(x, sh, sl, ch, cl) && shapes_sc_decided(sh, sl) && shapes_sc_decided(ch, cl)) {
    *s_out = sh + sl;
    *c_out = ch + cl;
    return;
  }
  const shapes_sc_pair r = shapes_sincos_accurate_v(x);
  *s_out = r.s;
  *c_out = r.c;
}

#endif /* SHAPES_SINCOS_H */
