/* The library's own FP32 elementary functions (annealing_gb300/csrc/sb_math.cuh), operation for
 * operation, for the CPU oracle — TEST INFRASTRUCTURE ONLY. Compile with -ffp-contract=off: every
 * product and sum below is one correctly rounded FP32 operation and every fmaf is fused, exactly as
 * the device code's _rn intrinsics, so host and device give identical bits. */
#ifndef SB_MATH_ORACLE_H
#define SB_MATH_ORACLE_H

#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint32_t om_bits(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
}
static inline float om_float(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}

/* log(u), u in [0, 1]: u = 2^e m, m in [sqrt(1/2), sqrt(2)), e ln 2 + 2 atanh((m-1)/(m+1)) */
static inline float om_log_unit(float u) {
  if (!(u > 0.0f)) return -INFINITY;
  const uint32_t b = om_bits(u);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  float m = om_float((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 0x1.6a09e6p+0f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float q = fmaf(z, 0x1.c71c72p-4f, 0x1.24924ap-3f);
  q = fmaf(z, q, 0x1.99999ap-3f);
  q = fmaf(z, q, 0x1.555556p-2f);
  const float at = fmaf(s * z, q, s);
  const float fe = (float)e;
  return fmaf(fe, 0x1.62e4p-1f, fmaf(fe, 0x1.7f7d1cp-20f, 2.0f * at));
}

/* sin t, cos t: k = rint(t 2/pi), two-part pi/2, Taylor to r^9 / r^8, quadrant k mod 4 */
static inline void om_sincos(float t, float *s_out, float *c_out) {
  const float k = rintf(t * 0x1.45f306p-1f);
  float r = fmaf(k, -0x1.921fb6p+0f, t);
  r = fmaf(k, 0x1.777a5cp-25f, r);
  const float z = r * r;
  float ps = fmaf(z, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
  ps = fmaf(z, ps, 0x1.111112p-7f);
  ps = fmaf(z, ps, -0x1.555556p-3f);
  const float sn = fmaf(r * z, ps, r);
  float pc = fmaf(z, 0x1.a01a02p-16f, -0x1.6c16c2p-10f);
  pc = fmaf(z, pc, 0x1.555556p-5f);
  pc = fmaf(z, pc, -0.5f);
  const float cs = fmaf(z, pc, 1.0f);
  const int q = (int)k & 3;
  *s_out = q == 0 ? sn : (q == 1 ? cs : (q == 2 ? -sn : -cs));
  *c_out = q == 0 ? cs : (q == 1 ? -sn : (q == 2 ? -cs : sn));
}

/* expm1(y), y in [-20, 0]: k = rint(y log2 e), two-part ln 2, Taylor to r^8, 2^k em + (2^k - 1) */
static inline float om_expm1_neg(float y) {
  const float k = rintf(y * 0x1.715476p+0f);
  float r = fmaf(k, -0x1.62e4p-1f, y);
  r = fmaf(k, -0x1.7f7d1cp-20f, r);
  float p = fmaf(r, 0x1.a01a02p-16f, 0x1.a01a02p-13f);
  p = fmaf(r, p, 0x1.6c16c2p-10f);
  p = fmaf(r, p, 0x1.111112p-7f);
  p = fmaf(r, p, 0x1.555556p-5f);
  p = fmaf(r, p, 0x1.555556p-3f);
  p = fmaf(r, p, 0.5f);
  const float em = fmaf(r * r, p, r);
  const int ki = (int)k;
  if (ki == 0) return em;
  const float two_k = om_float((uint32_t)(127 + ki) << 23);
  return fmaf(two_k, em, two_k - 1.0f);
}

/* tanh x = -e / (2 + e), e = expm1(-2|x|); +-1 beyond |x| = 10; NaN stays NaN */
static inline float om_tanh(float x) {
  const float ax = fabsf(x);
  if (ax != ax) return x;
  if (ax > 10.0f) return copysignf(1.0f, x);
  const float e = om_expm1_neg(-2.0f * ax);
  return copysignf(-e / (2.0f + e), x);
}

#endif
