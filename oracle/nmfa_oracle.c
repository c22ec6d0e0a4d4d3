/* CPU restatement of NMFA (noisy mean-field annealing) — TEST INFRASTRUCTURE ONLY.
 *
 * Follows NMFA/CUDA_GPU/src/nmfa.cu (gpu_nmfa_kernel :54-140) and the schedule of
 * NMFA/CUDA_GPU/Ising.cpp:37-43, with the semantics and arithmetic this library's CUDA path uses,
 * so that the two agree bit for bit:
 *   oracle_nmfa_seed      nmfa.cu:62-76  per-(sample, spin) XORWOW words: t = seed + n r + i,
 *                                        four xorshift32 steps (:43-47) give words 0..3, counter 0
 *   oracle_nmfa_xorwow    nmfa.cu:29-40  XORWOW (Marsaglia, "Xorshift RNGs", p. 5)
 *   oracle_nmfa_gauss     nmfa.cu:103-109 Box-Muller: radius sqrt(-2 log(a/2^32)) noise,
 *                                        angle 2 pi b / 2^32, z0 = sin * radius, z1 = cos * radius
 *   oracle_nmfa_run       nmfa.cu:85-139 norm_i = -1/sqrt(sum_j |J_ij|) (here in double, 0 for an
 *                                        empty row), per stage two sweeps with z0 then z1:
 *                                        s <- (1 - alpha) s + alpha tanh(beta (norm f + z)), f = J s,
 *                                        sample = s > 0 ? +1 : -1
 *   oracle_nmfa_schedule  Ising.cpp:37-43
 * Differences from the reference, by design of the library (stated in its C header):
 *   * a sweep reads the previous sweep's states (the reference's two sweeps of a stage have no
 *     barrier between warps; for n <= 32, one warp, it computes exactly this);
 *   * log, sin, cos and tanh are the library's own FP32 functions (sb_math_oracle.h), the
 *     reference's are CUDA fast-math intrinsics;
 *   * the field f_i = sum_j J_ij s_j is summed in the order of the library's kernel: 32 partial
 *     sums, partial l taking the groups of four j = 4g .. 4g+3 with g = l mod 32 in increasing g
 *     (one fused multiply-add per term), then combined pairwise v[l] + v[l ^ o] for o = 16, 8, 4,
 *     2, 1 — the kernel's lanes and its butterfly.
 * Compiled with -ffp-contract=off. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sb_math_oracle.h"

void oracle_nmfa_schedule(int stages, float *betas) {
  const float increase = (8 - 1 / (float)16) / (float)stages;
  float beta = 1 / (float)16;
  for (int i = 0; i < stages; ++i) {
    betas[i] = beta;
    beta += increase;
  }
}

/* w: [R][n][5] */
void oracle_nmfa_seed(int n, int R, uint32_t seed, uint32_t *w) {
  for (int r = 0; r < R; ++r)
    for (int i = 0; i < n; ++i) {
      uint32_t t = seed + (uint32_t)n * (uint32_t)r + (uint32_t)i;
      uint32_t *s = w + ((size_t)r * n + i) * 5;
      for (int q = 0; q < 4; ++q) {
        t ^= t << 13;
        t ^= t >> 17;
        t ^= t << 5;
        s[q] = t;
      }
      s[4] = 0u;
    }
}

uint32_t oracle_nmfa_xorwow(uint32_t *w) {
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

void oracle_nmfa_gauss(uint32_t *w, float noise, float *z0, float *z1) {
  const uint32_t a = oracle_nmfa_xorwow(w);
  const uint32_t b = oracle_nmfa_xorwow(w);
  const float u = (float)a * 0x1p-32f;
  const float rad = sqrtf(-2.0f * om_log_unit(u)) * noise;
  const float ang = (float)b * 0x1.921fb6p-30f;
  float sn, cs;
  om_sincos(ang, &sn, &cs);
  *z0 = sn * rad;
  *z1 = cs * rad;
}

float oracle_nmfa_tanh(float x) { return om_tanh(x); }
void oracle_nmfa_sincos(float t, float *s, float *c) { om_sincos(t, s, c); }

/* f = sum_j J[j] s[j] over jp = n rounded up to 4 (J, s zero beyond n), in the kernel's order */
static float field(const float *Jrow, const float *s, int n, int jp) {
  float v[32], w[32];
  for (int l = 0; l < 32; ++l) v[l] = 0.0f;
  for (int g = 0; g < jp / 4; ++g) {
    const int l = g & 31;
    for (int c = 0; c < 4; ++c) {
      const int j = 4 * g + c;
      const float jv = j < n ? Jrow[j] : 0.0f;
      v[l] = fmaf(jv, s[j], v[l]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int l = 0; l < 32; ++l) w[l] = v[l] + v[l ^ o];
    memcpy(v, w, sizeof(v));
  }
  return v[0];
}

/* J: [n][n] row-major. states: [R][n] final states; samples: [R][n] +-1; trace (may be NULL):
 * [stages][R][n] states after each stage. Returns 0, or -1 on bad sizes / allocation failure. */
int oracle_nmfa_run(int n, const float *J, int R, const float *betas, int stages, float noise, float recombination,
                    uint32_t seed, float *states, int32_t *samples, float *trace) {
  if (n < 1 || R < 1 || stages < 1) return -1;
  const int jp = (n + 3) & ~3;
  float *norm = (float *)malloc((size_t)n * sizeof(float));
  float *cur = (float *)calloc((size_t)R * jp, sizeof(float));
  float *nxt = (float *)calloc((size_t)R * jp, sizeof(float));
  float *z1 = (float *)malloc((size_t)R * n * sizeof(float));
  uint32_t *w = (uint32_t *)malloc((size_t)R * n * 5 * sizeof(uint32_t));
  if (!norm || !cur || !nxt || !z1 || !w) {
    free(norm);
    free(cur);
    free(nxt);
    free(z1);
    free(w);
    return -1;
  }
  for (int i = 0; i < n; ++i) {
    double a = 0.0;
    for (int j = 0; j < n; ++j) a += fabs((double)J[(size_t)i * n + j]);
    norm[i] = a > 0.0 ? (float)(-1.0 / sqrt(a)) : 0.0f;
  }
  oracle_nmfa_seed(n, R, seed, w);
  const float keep = (float)(1.0 - (double)recombination), mix = recombination;
  for (int t = 0; t < stages; ++t) {
    for (int k = 0; k < 2; ++k) {
      for (int r = 0; r < R; ++r)
        for (int i = 0; i < n; ++i) {
          const float f = field(J + (size_t)i * n, cur + (size_t)r * jp, n, jp);
          float z;
          if (k == 0) {
            float zz1;
            oracle_nmfa_gauss(w + ((size_t)r * n + i) * 5, noise, &z, &zz1);
            z1[(size_t)r * n + i] = zz1;
          } else {
            z = z1[(size_t)r * n + i];
          }
          const float mf = f * norm[i] + z;
          const float th = om_tanh(mf * betas[t]);
          nxt[(size_t)r * jp + i] = keep * cur[(size_t)r * jp + i] + mix * th;
        }
      float *tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
    if (trace)
      for (int r = 0; r < R; ++r) memcpy(trace + ((size_t)t * R + r) * n, cur + (size_t)r * jp, (size_t)n * sizeof(float));
  }
  for (int r = 0; r < R; ++r)
    for (int i = 0; i < n; ++i) {
      const float v = cur[(size_t)r * jp + i];
      if (states) states[(size_t)r * n + i] = v;
      if (samples) samples[(size_t)r * n + i] = v > 0.0f ? 1 : -1;
    }
  free(norm);
  free(cur);
  free(nxt);
  free(z1);
  free(w);
  return 0;
}
