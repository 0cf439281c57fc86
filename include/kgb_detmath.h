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
 * Accuracy: a few ulps in float; ~1e-15 relative for the double logarithm (kgb_log_d) that kgb_powf's ln x comes from.
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

/* e^(th + tl) in float, th + tl a float pair with |th| < 87: k = round(th log2 e), r = th - k ln 2 + tl with
 * ln 2 = hi + lo (hi has 15 significant bits, so k hi is exact), the Taylor series of e^r to r^8 (|r| <= 0.35: the
 * first term left out is below 2^-32) by fused Horner steps, times 2^k. A few float ulps; every multiply-add is an
 * explicit fmaf, so every machine gets the same bits. */
KGB_HD float kgb_expf_pair(float th, float tl) {
  const float k = rintf(th * 1.44269504f);
  float r = fmaf(-k, 0.693145751953125f, th);
  r = fmaf(-k, 1.42860677e-06f, r) + tl;
  float p = 1.0f / 40320.0f;
  p = fmaf(p, r, 1.0f / 5040.0f);
  p = fmaf(p, r, 1.0f / 720.0f);
  p = fmaf(p, r, 1.0f / 120.0f);
  p = fmaf(p, r, 1.0f / 24.0f);
  p = fmaf(p, r, 1.0f / 6.0f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  return ldexpf(p, (int)k);
}

/* ln x as a float pair (hi = float(ln x), lo = float(ln x - hi)) from the double logarithm, x > 0. */
KGB_HD void kgb_ln_pair(float x, float* hi, float* lo) {
  const double l = kgb_log_d((double)x);
  *hi = (float)l;
  *lo = (float)(l - (double)*hi);
}

/* x^y = e^(y ln x) for x > 0 given ln x as a float pair: y ln x formed exactly as a pair (fmaf), then kgb_expf_pair. */
KGB_HD float kgb_pow_ln(float lnh, float lnl, float y) {
  const float th = y * lnh;
  const float tl = fmaf(y, lnh, -th) + y * lnl;
  return kgb_expf_pair(th, tl);
}

/* x^y for x > 0 (0 -> 0): kgb_pow_ln with ln x from kgb_ln_pair. */
KGB_HD float kgb_powf(float x, float y) {
  if (!(x > 0.0f)) return 0.0f;
  float h, l;
  kgb_ln_pair(x, &h, &l);
  return kgb_pow_ln(h, l, y);
}

#endif /* KGB_DETMATH_H */
