// This library's own FP32 elementary functions for the annealers whose results are compared bit
// for bit with the CPU oracle (SQA acceptance thresholds, NMFA noise and mean-field update). Each
// is a fixed sequence of correctly rounded FP32 operations (explicit _rn intrinsics, no
// contraction), and oracle/sb_math_oracle.h carries the same sequences, so host and device give
// identical bits. The methods are textbook: range reduction by a power of two or by a multiple of
// a two-part constant, then a truncated Taylor series.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace sbm {

// log(u) for u in [0, 1] (0 gives -inf): u = 2^e m with m in [sqrt(1/2), sqrt(2)),
// log u = e ln 2 + 2 atanh((m - 1) / (m + 1)), atanh by its series to s^9.
__device__ __forceinline__ float log_unit(float u) {
  if (!(u > 0.0f)) return -INFINITY;
  const uint32_t b = __float_as_uint(u);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 0x1.6a09e6p+0f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float z = __fmul_rn(s, s);
  float q = __fmaf_rn(z, 0x1.c71c72p-4f, 0x1.24924ap-3f);
  q = __fmaf_rn(z, q, 0x1.99999ap-3f);
  q = __fmaf_rn(z, q, 0x1.555556p-2f);
  const float at = __fmaf_rn(__fmul_rn(s, z), q, s);
  const float fe = (float)e;
  return __fmaf_rn(fe, 0x1.62e4p-1f, __fmaf_rn(fe, 0x1.7f7d1cp-20f, __fmul_rn(2.0f, at)));
}

// sin t and cos t for finite t of moderate size (the noise angles lie in [0, 2 pi]):
// t = k pi/2 + r with k = rint(t 2/pi), r by a two-part pi/2, |r| <= pi/4; the Taylor series of
// sin to r^9 and of cos to r^8 (truncation below 2e-9), then the quadrant k mod 4.
__device__ __forceinline__ void sincos_f(float t, float &s_out, float &c_out) {
  const float k = rintf(__fmul_rn(t, 0x1.45f306p-1f));
  float r = __fmaf_rn(k, -0x1.921fb6p+0f, t);
  r = __fmaf_rn(k, 0x1.777a5cp-25f, r);
  const float z = __fmul_rn(r, r);
  float ps = __fmaf_rn(z, 0x1.71de3ap-19f, -0x1.a01a02p-13f);  // 1/9!, -1/7!
  ps = __fmaf_rn(z, ps, 0x1.111112p-7f);                        // 1/5!
  ps = __fmaf_rn(z, ps, -0x1.555556p-3f);                       // -1/3!
  const float sn = __fmaf_rn(__fmul_rn(r, z), ps, r);
  float pc = __fmaf_rn(z, 0x1.a01a02p-16f, -0x1.6c16c2p-10f);   // 1/8!, -1/6!
  pc = __fmaf_rn(z, pc, 0x1.555556p-5f);                        // 1/4!
  pc = __fmaf_rn(z, pc, -0.5f);                                 // -1/2!
  const float cs = __fmaf_rn(z, pc, 1.0f);
  const int q = (int)k & 3;
  s_out = q == 0 ? sn : (q == 1 ? cs : (q == 2 ? -sn : -cs));
  c_out = q == 0 ? cs : (q == 1 ? -sn : (q == 2 ? -cs : sn));
}

// expm1(y) for y in [-20, 0]: y = k ln 2 + r (k = rint(y log2 e), r by a two-part ln 2,
// |r| <= ln2 / 2), expm1(r) by its Taylor series to r^8, then 2^k expm1(r) + (2^k - 1).
__device__ __forceinline__ float expm1_neg(float y) {
  const float k = rintf(__fmul_rn(y, 0x1.715476p+0f));
  float r = __fmaf_rn(k, -0x1.62e4p-1f, y);
  r = __fmaf_rn(k, -0x1.7f7d1cp-20f, r);
  float p = __fmaf_rn(r, 0x1.a01a02p-16f, 0x1.a01a02p-13f);  // 1/8!, 1/7!
  p = __fmaf_rn(r, p, 0x1.6c16c2p-10f);                      // 1/6!
  p = __fmaf_rn(r, p, 0x1.111112p-7f);                       // 1/5!
  p = __fmaf_rn(r, p, 0x1.555556p-5f);                       // 1/4!
  p = __fmaf_rn(r, p, 0x1.555556p-3f);                       // 1/3!
  p = __fmaf_rn(r, p, 0.5f);                                 // 1/2!
  const float em = __fmaf_rn(__fmul_rn(r, r), p, r);
  const int ki = (int)k;
  if (ki == 0) return em;
  const float two_k = __uint_as_float((uint32_t)(127 + ki) << 23);
  return __fmaf_rn(two_k, em, __fsub_rn(two_k, 1.0f));
}

// tanh x = -e / (2 + e) with e = expm1(-2 |x|), the sign of x restored; +-1 beyond |x| = 10
// (where 1 - tanh |x| < 2^-27); NaN stays NaN.
__device__ __forceinline__ float tanh_f(float x) {
  const float ax = fabsf(x);
  if (ax != ax) return x;
  if (ax > 10.0f) return copysignf(1.0f, x);
  const float e = expm1_neg(__fmul_rn(-2.0f, ax));
  return copysignf(__fdiv_rn(-e, __fadd_rn(2.0f, e)), x);
}

// XORWOW (Marsaglia, "Xorshift RNGs", p. 5) on words w[0..3] and the additive counter w[4], in the
// update order of NMFA/CUDA_GPU/src/nmfa.cu:29-40.
__device__ __forceinline__ uint32_t xorwow(uint32_t (&w)[5]) {
  uint32_t t = w[3];
  t ^= t >> 2;
  t ^= t << 1;
  w[3] = w[2];
  w[2] = w[1];
  w[1] = w[0];
  t ^= w[0];
  t ^= w[0] << 4;
  w[0] = t;
  w[4] += 362437u;
  return t + w[4];
}

// The stage's two Gaussian samples by the Box-Muller transform (NMFA/CUDA_GPU/src/nmfa.cu:103-109):
// two words a, b, radius sqrt(-2 log(a / 2^32)) noise, angle 2 pi b / 2^32; z0 = sin(angle) radius,
// z1 = cos(angle) radius.
__device__ __forceinline__ void nmfa_gauss(uint32_t (&w)[5], float noise, float &z0, float &z1) {
  const uint32_t a = xorwow(w);
  const uint32_t b = xorwow(w);
  const float u = __fmul_rn(__uint2float_rn(a), 0x1p-32f);
  const float rad = __fmul_rn(__fsqrt_rn(__fmul_rn(-2.0f, sbm::log_unit(u))), noise);
  const float ang = __fmul_rn(__uint2float_rn(b), 0x1.921fb6p-30f);
  float sn, cs;
  sbm::sincos_f(ang, sn, cs);
  z0 = __fmul_rn(sn, rad);
  z1 = __fmul_rn(cs, rad);
}

// One mean-field update (NMFA/CUDA_GPU/src/nmfa.cu:124-128): field f, row norm, noise z:
// s' = keep s + mix tanh(beta (f norm + z)), keep = 1 - alpha, mix = alpha.
__device__ __forceinline__ float nmfa_update(float f, float norm, float z, float beta, float keep, float mix,
                                             float s) {
  const float mf = __fadd_rn(__fmul_rn(f, norm), z);
  const float th = tanh_f(__fmul_rn(mf, beta));
  return __fadd_rn(__fmul_rn(keep, s), __fmul_rn(mix, th));
}

}  // namespace sbm
