/* Portable, bit-reproducible scalar math for the oracle (test infrastructure).
 *
 * The reference raises the embedded error estimate to a power in its PI step-size
 * controller (perform_step/gpu_tsit5_perform_step.jl:127-128, `EEst^beta1`,
 * `qold^beta2`).  libm's powf and CUDA's powf are different functions, so an adaptive
 * run would drift apart in the last bits after the first controller decision.  In
 * parity mode both the oracle and the kernels use the functions below instead: they
 * are built only from IEEE +, -, *, / and exact bit manipulation, evaluated in the same
 * order, and compiled without FMA contraction, so CPU and GPU produce identical bits.
 *
 * Method (textbook, e.g. Muller, "Elementary Functions", ch. 6):
 *   log:  x = m 2^e with m in [sqrt(1/2), sqrt(2)),  s = (m-1)/(m+1),
 *         ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ... + s^13/13)
 *   exp:  y = n ln2 + r, |r| <= ln2/2, e^r by its Taylor series to r^9/9!, scaled by 2^n.
 *   pow:  x^y = exp(y ln x)   (x > 0)
 *   sin/cos (Box-Muller angles): argument in turns, quadrant reduction, Taylor series.
 * Accuracy is a few float ulps -- ample for step-size control and normal variates.
 */
#pragma once
#include <stdint.h>
#include <string.h>

static inline float pm_bits_to_float(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t pm_float_to_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

/* natural log for finite x > 0 (normal or subnormal) */
static inline float pm_logf(float x) {
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; } /* scale subnormals by 2^24 */
  uint32_t b = pm_float_to_bits(x);
  e += (int)((b >> 23) & 0xff) - 127;
  float m = pm_bits_to_float((b & 0x007fffffu) | 0x3f800000u); /* m in [1,2) */
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float poly = 1.0f / 13.0f;
  poly = poly * s2 + 1.0f / 11.0f;
  poly = poly * s2 + 1.0f / 9.0f;
  poly = poly * s2 + 1.0f / 7.0f;
  poly = poly * s2 + 1.0f / 5.0f;
  poly = poly * s2 + 1.0f / 3.0f;
  poly = poly * s2 + 1.0f;
  float lnm = 2.0f * s * poly;
  float ef = (float)e;
  return ef * 0.693145752f + (ef * 1.42860677e-06f + lnm); /* ln2 split hi+lo */
}

/* exp for finite y; clamps to 0 / +inf outside the float range */
static inline float pm_expf(float y) {
  if (y > 88.7f) return pm_bits_to_float(0x7f800000u);
  if (y < -103.0f) return 0.0f;
  float t = y * 1.44269504f;
  int n = (int)(t >= 0.0f ? t + 0.5f : t - 0.5f);
  float nf = (float)n;
  float r = (y - nf * 0.693145752f) - nf * 1.42860677e-06f;
  float p = 1.0f / 362880.0f;
  p = p * r + 1.0f / 40320.0f;
  p = p * r + 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  /* scale by 2^n in two exact steps so that n down to -149 works */
  int n1 = n / 2, n2 = n - n1;
  float s1 = pm_bits_to_float((uint32_t)(n1 + 127) << 23);
  float s2 = pm_bits_to_float((uint32_t)(n2 + 127) << 23);
  return (p * s1) * s2;
}

/* x^y for x >= 0 (the controller only raises non-negative error norms) */
static inline float pm_powf(float x, float y) {
  if (x == 0.0f) return 0.0f;
  if (!(x == x)) return x; /* NaN propagates */
  if (x > 3.40282347e38f) return x; /* +inf */
  return pm_expf(y * pm_logf(x));
}

/* sin and cos of 2*pi*v for v in [0, 1] */
static inline void pm_sincos_turns(float v, float* s, float* c) {
  float w = v >= 0.5f ? v - 1.0f : v;     /* [-0.5, 0.5) turns */
  float w4 = w * 4.0f;                    /* quarter turns, exact */
  int q = (int)(w4 >= 0.0f ? w4 + 0.5f : w4 - 0.5f);
  float r = (w4 - (float)q) * 1.57079633f; /* |r| <= pi/4 */
  float r2 = r * r;
  float sp = -1.0f / 39916800.0f;
  sp = sp * r2 + 1.0f / 362880.0f;
  sp = sp * r2 - 1.0f / 5040.0f;
  sp = sp * r2 + 1.0f / 120.0f;
  sp = sp * r2 - 1.0f / 6.0f;
  sp = sp * r2 + 1.0f;
  float sr = r * sp;
  float cp = 1.0f / 3628800.0f;
  cp = cp * r2 - 1.0f / 40320.0f;
  cp = cp * r2 + 1.0f / 720.0f;
  cp = cp * r2 - 1.0f / 24.0f;
  cp = cp * r2 + 0.5f;
  float cr = 1.0f - r2 * cp;
  int qm = q & 3;
  if (qm == 0) { *s = sr; *c = cr; }
  else if (qm == 1) { *s = cr; *c = -sr; }
  else if (qm == 2) { *s = -sr; *c = -cr; }
  else { *s = -cr; *c = sr; }
}
