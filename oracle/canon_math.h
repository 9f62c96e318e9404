/*
 * Canonical FP64 exp / log / pow for the oracle's "canonical" mode -- test
 * infrastructure.
 *
 * The reference calls the platform's exp/log/pow, whose last-bit results
 * differ between glibc and CUDA.  Because the RKC controller turns last-bit
 * differences into different accept/reject decisions within a few
 * milliseconds, bit-identical comparison of the GPU path with the oracle
 * needs one agreed implementation of these functions.  This one is:
 *
 *   exp: x = k ln2 + r with k = rint(x / ln2) and a two-part ln2 (40-bit high
 *        part, Cody & Waite 1980); e^r by its degree-13 Taylor polynomial
 *        (|r| <= ln2/2, truncation < 5e-18) in Horner form with fused
 *        multiply-adds; scaling by 2^k from the exponent bits.
 *   log: x = 2^e m with m in [sqrt(1/2), sqrt(2)]; log m = 2 atanh(s),
 *        s = (m-1)/(m+1), by the odd series 2s + s * sum_{k=1..11}
 *        2 z^k / (2k+1), z = s^2 (|s| <= 0.1716, truncation < 1e-18);
 *        plus e ln2 with the same two-part ln2.
 *   pow: exp(y log x) for x >= 0.
 *
 * The canonical step-size controller evaluates err^(1/3) once per step with
 * cm_cbrt (below), takes err^(2/3) as its square and reuses the cube root of
 * the previous error (the reference calls pow three times,
 * solve_rkc.cu:1038-1051).
 *
 * Measured error against the exact result (tests/test_canon_math.py): exp
 * within 0.76 ulp, log within 1.8 ulp, pow(x, 1/3) within 7 ulp, cm_cbrt
 * within 4 ulp over the controller's range.  The CUDA product carries its own copy of the same
 * algorithm (csrc/canon_math.cuh); the GPU parity tests, bit-exact through
 * whole trajectories, check that the two agree.  Compile with
 * -ffp-contract=off: every fma here is explicit.
 */
#ifndef ORACLE_CANON_MATH_H
#define ORACLE_CANON_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#define CM_LN2_HI 0x1.62e42fefa2000p-1
#define CM_LN2_LO 0x1.9ef35793c7673p-41
#define CM_INV_LN2 0x1.71547652b82fep+0
#define CM_SQRT2 0x1.6a09e667f3bcdp+0

static inline uint64_t cm_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double cm_from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

static inline double cm_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return HUGE_VAL;
  if (x < -745.1332191019412) return 0.0;
  double kd = rint(x * CM_INV_LN2);
  double r = fma(-kd, CM_LN2_HI, x);
  r = fma(-kd, CM_LN2_LO, r);
  double p = 0x1.6124613a86d09p-33;          /* 1/13! */
  p = fma(p, r, 0x1.1eed8eff8d898p-29);      /* 1/12! */
  p = fma(p, r, 0x1.ae64567f544e4p-26);      /* 1/11! */
  p = fma(p, r, 0x1.27e4fb7789f5cp-22);      /* 1/10! */
  p = fma(p, r, 0x1.71de3a556c734p-19);      /* 1/9!  */
  p = fma(p, r, 0x1.a01a01a01a01ap-16);      /* 1/8!  */
  p = fma(p, r, 0x1.a01a01a01a01ap-13);      /* 1/7!  */
  p = fma(p, r, 0x1.6c16c16c16c17p-10);      /* 1/6!  */
  p = fma(p, r, 0x1.1111111111111p-7);       /* 1/5!  */
  p = fma(p, r, 0x1.5555555555555p-5);       /* 1/4!  */
  p = fma(p, r, 0x1.5555555555555p-3);       /* 1/3!  */
  p = fma(p, r, 0x1.0000000000000p-1);       /* 1/2!  */
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  int k = (int)kd;
  if (k > 1023) { p *= 2.0; k -= 1; }
  if (k < -1022) { p *= 0x1p-54; k += 54; }
  return p * cm_from_bits((uint64_t)(k + 1023) << 52);
}

static inline double cm_log(double x) {
  if (!(x > 0.0)) return (x == 0.0) ? -HUGE_VAL : (x - x) / (x - x);
  if (x == HUGE_VAL) return x;
  int e = 0;
  if (x < 0x1p-1022) { x *= 0x1p54; e = -54; }
  uint64_t u = cm_bits(x);
  e += (int)((u >> 52) & 0x7ff) - 1023;
  double m = cm_from_bits((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > CM_SQRT2) { m *= 0.5; e += 1; }
  double f = m - 1.0;
  double s = f / (2.0 + f);
  double z = s * s;
  double R = 0x1.642c8590b2164p-4;           /* 2/23 */
  R = fma(R, z, 0x1.8618618618618p-4);       /* 2/21 */
  R = fma(R, z, 0x1.af286bca1af28p-4);       /* 2/19 */
  R = fma(R, z, 0x1.e1e1e1e1e1e1ep-4);       /* 2/17 */
  R = fma(R, z, 0x1.1111111111111p-3);       /* 2/15 */
  R = fma(R, z, 0x1.3b13b13b13b14p-3);       /* 2/13 */
  R = fma(R, z, 0x1.745d1745d1746p-3);       /* 2/11 */
  R = fma(R, z, 0x1.c71c71c71c71cp-3);       /* 2/9  */
  R = fma(R, z, 0x1.2492492492492p-2);       /* 2/7  */
  R = fma(R, z, 0x1.999999999999ap-2);       /* 2/5  */
  R = fma(R, z, 0x1.5555555555555p-1);       /* 2/3  */
  R = R * z;
  double lm = fma(s, R, 2.0 * s);
  double ed = (double)e;
  return fma(ed, CM_LN2_HI, fma(ed, CM_LN2_LO, lm));
}

static inline double cm_pow(double x, double y) { return cm_exp(y * cm_log(x)); }

#define CM_FN static inline
/* Cube root for the step-size controller's err^(1/3), err >= 0.
 * x = 2^e m with m in [1, 2); e = 3q + r (r = 0, 1, 2) and z = 2^r m in
 * [1, 8), so cbrt(x) = 2^q cbrt(z).  The reciprocal cube root y = z^(-1/3)
 * is seeded in FP32 by a least-squares quadratic in z (relative error below
 * 0.09), refined by three FP32 Newton steps y <- y (4 - z y^3) / 3 (error
 * ~3e-7, the FP32 rounding level) and two FP64 steps Y <- Y + Y (1 - Z Y^3)/3
 * (quadratic convergence: below 1e-25 before rounding); then
 * cbrt(z) = Z Y Y and the exact scaling by 2^q.  No division.  Every
 * operation is written out (FP32 products unfused, FP64 fma explicit), so
 * host and device give the same bits.  Measured against 60-digit
 * arithmetic: within 4 ulp, 0.7 ulp on average (tests/test_canon_math.py).  0, +inf and NaN
 * return themselves. */
CM_FN double cm_cbrt(double x) {
  if (!(x > 0.0) || x == HUGE_VAL) return x;
  int e = 0;
  if (x < 0x1p-1022) { x *= 0x1p54; e = -54; }
  const uint64_t u = cm_bits(x);
  e += (int)((u >> 52) & 0x7ff) - 1023;
  const int q = (e >= 0) ? e / 3 : -((2 - e) / 3);
  const int r = e - 3 * q;
  const double Z = cm_from_bits((u & 0x000fffffffffffffULL) | ((uint64_t)(1023 + r) << 52));
  const float zf = (float)Z;
  float y = 0x1.0b5c7ap+0f;
  y = y + (-0x1.1bfbb8p-3f) * zf;
  y = y + (0x1.2a6c02p-7f) * zf * zf;
  for (int k = 0; k < 3; k++) {
    const float y3 = y * y * y;
    const float t = 4.0f - zf * y3;
    y = (y * t) * 0x1.555556p-2f;
  }
  double Y = (double)y;
  for (int k = 0; k < 2; k++) {
    const double Y3 = (Y * Y) * Y;
    const double d = fma(-Z, Y3, 1.0);
    Y = fma(Y * d, 0x1.5555555555555p-2, Y);
  }
  const double c = (Z * Y) * Y;
  return c * cm_from_bits((uint64_t)(q + 1023) << 52);
}
#undef CM_FN


#endif
