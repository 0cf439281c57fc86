/*
 * kgb_detmath.h - deterministic elementary functions of the engine's numerics contract.
 *
 * The engine's decisions (a ray's direction cell, a glass pane's transmittance byte, the sky bin an escaping path
 * falls into) must come out bit for bit the same on the GPU and on any host that restates them. CUDA's sincospif /
 * powf / asinf / atan2f / logf and the host C library's differ in the last ulp, so the few functions those decisions
 * use are written here once, from textbook series (Taylor series after exact range reduction; log through
 * 2 atanh((m-1)/(m+1)); atan with two argument halvings), as a fixed sequence of IEEE-754 operations: a caller must
 * compile them without floating-point contraction (nvcc -fmad=false; gcc -ffp-contract=off). Division and square root
 * are the correctly rounded IEEE operations on both sides (nvcc -prec-div=true -prec-sqrt=true, its default).
 *
 * Accuracy: a few ulps in float, ~1e-15 relative for the double exp/log used by kgb_powf.
 */
#ifndef KGB_DETMATH_H
#define KGB_DETMATH_H

#if defined(__CUDACC__)
#define KGB_HD __host__ __device__ __forceinline__
#else
#define KGB_HD static inline
#include <math.h>
#endif

/* pi / 180 and friends as float / double literals (rounded by the compiler, identically on both sides). */
#define KGB_PI_D 3.14159265358979323846
#define KGB_PI_F 3.14159265358979323846f

/* sin(pi x), cos(pi x): x = q/2 + r exactly (|r| <= 1/4, |x| < 2^22), then Taylor series of sin / cos at pi r. */
KGB_HD void kgb_sincospi(float x, float* s, float* c) {
  const float q = rintf(2.0f * x);
  const float r = x - 0.5f * q;
  const int iq = ((int)q) & 3;
  const float z = r * r;
  /* sin(pi r) = pi r (1 - (pi r)^2/3! + (pi r)^4/5! - ...), cos(pi r) = 1 - (pi r)^2/2! + ... */
  const float s1 = 3.14159265358979f, s3 = -5.16771278004997f, s5 = 2.55016403987735f, s7 = -0.599264529320792f,
              s9 = 0.0821458866111282f, s11 = -0.00737043094571435f;
  const float c2 = -4.93480220054468f, c4 = 4.05871212641677f, c6 = -1.33526276885459f, c8 = 0.235330630358893f,
              c10 = -0.0258068913900856f, c12 = 0.00192957430940392f;
  const float sp = r * (s1 + z * (s3 + z * (s5 + z * (s7 + z * (s9 + z * s11)))));
  const float cp = 1.0f + z * (c2 + z * (c4 + z * (c6 + z * (c8 + z * (c10 + z * c12)))));
  switch (iq) {
    case 0: *s = sp; *c = cp; break;
    case 1: *s = cp; *c = -sp; break;
    case 2: *s = -sp; *c = -cp; break;
    default: *s = -cp; *c = sp; break;
  }
}

/* atan(z) for |z| <= 1: two halvings atan(z) = 2 atan(z / (1 + sqrt(1 + z^2))) bring |z| under tan(pi/16), then the
 * Taylor series z - z^3/3 + z^5/5 - ... to z^13. */
KGB_HD float kgb_atan_unit(float z) {
  float y = z / (1.0f + sqrtf(1.0f + z * z));
  y = y / (1.0f + sqrtf(1.0f + y * y));
  const float w = y * y;
  const float p = y * (1.0f + w * (-0.333333333333333f + w * (0.2f + w * (-0.142857142857143f + w * (0.111111111111111f +
                  w * (-0.0909090909090909f + w * 0.0769230769230769f))))));
  return 4.0f * p;
}

/* atan2(y, x) in (-pi, pi]; atan2(0, 0) = 0. */
KGB_HD float kgb_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  if (ax == 0.0f && ay == 0.0f) return 0.0f;
  float a = ay <= ax ? kgb_atan_unit(ay / ax) : 1.57079632679490f - kgb_atan_unit(ax / ay);
  if (x < 0.0f) a = 3.14159265358979f - a;
  return y < 0.0f ? -a : a;
}

/* asin(x) for x in [-1, 1]: 2 atan(x / (1 + sqrt(1 - x^2))). */
KGB_HD float kgb_asin(float x) {
  return 2.0f * kgb_atan_unit(x / (1.0f + sqrtf(1.0f - x * x)));
}

/* ln(x) for finite x > 0 in float: x = m 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s = (m-1)/(m+1). */
KGB_HD float kgb_logf(float x) {
  int e = 0;
  float m = frexpf(x, &e); /* x = m 2^e, m in [0.5, 1) */
  if (m < 0.707106781186548f) { m = 2.0f * m; e -= 1; }
  const float s = (m - 1.0f) / (m + 1.0f), z = s * s;
  const float t = 2.0f * s * (1.0f + z * (0.333333333333333f + z * (0.2f + z * (0.142857142857143f + z * 0.111111111111111f))));
  const float fe = (float)e;
  return fe * 0.693145751953125f + (fe * 1.42860682030941723e-6f + t); /* ln 2 = hi + lo */
}

/* ln(x) in double, x > 0 finite: the same reduction, series to s^25. */
KGB_HD double kgb_log_d(double x) {
  int e = 0;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752) { m = 2.0 * m; e -= 1; }
  const double s = (m - 1.0) / (m + 1.0), z = s * s;
  double p = 1.0 / 25.0;
  for (int k = 23; k >= 1; k -= 2) p = 1.0 / (double)k + z * p;
  return (double)e * 0.69314718055994530942 + 2.0 * s * p;
}

/* exp(x) in double for |x| < 700: x = k ln2 + r, |r| <= ln2 / 2, Taylor series of e^r to r^16 by Horner's rule, times
 * 2^k. Every multiply-add is an explicit fma (one rounding, the same on both sides): 18 fused operations. */
KGB_HD double kgb_exp_d(double x) {
  const double k = rint(x * 1.44269504088896340736);
  const double r = fma(-k, 1.90821492927058770002e-10, fma(-k, 0.693147180369123816490, x)); /* x - k ln 2, ln 2 = hi + lo */
  double p = 1.0 / 20922789888000.0; /* 1/16! */
  const double inv[16] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040, 1.0 / 40320,
                          1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800, 1.0 / 479001600, 1.0 / 6227020800.0,
                          1.0 / 87178291200.0, 1.0 / 1307674368000.0};
  for (int j = 15; j >= 0; --j) p = fma(r, p, inv[j]);
  return ldexp(p, (int)k);
}

/* x^y for x > 0 (0 -> 0), as float(exp(y ln x)) in double. */
KGB_HD float kgb_powf(float x, float y) {
  if (!(x > 0.0f)) return 0.0f;
  return (float)kgb_exp_d((double)y * kgb_log_d((double)x));
}

#endif /* KGB_DETMATH_H */
