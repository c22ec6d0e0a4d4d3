/* CPU oracle for fully-connected simulated quantum annealing (SQA) — TEST INFRASTRUCTURE ONLY.
 *
 * Imported by tests/ (through oracle/binding.py) and bench.py's CPU baseline; never by the solver.
 * Compiled with -ffp-contract=off so every float operation rounds where the source says.
 *
 * Restates SQA_fully/fully_test/pre_calculate.cu (the "reduced sum" GPU SQA of the reference):
 *   - spins s[m][i] = +-1 in M Trotter slices, couplings J integer (the reference reads them as
 *     char, :164-179), no fields (:176 asserts a != b);
 *   - per annealing step p (:217-226): Gamma = G0 (1 - p / STEP), J_perp = -0.5 log(tanh(Gamma / M
 *     * beta)) / beta, beta += (8 - 1/16) / STEP after the step, G0 = 8, beta starts at 1/16;
 *   - each step runs M + N - 1 wavefront iterations a (:221-224); in iteration a slice m updates
 *     spin (a - m) mod N (:63), so the M slices never touch the same spin and all of them update at
 *     once: field f = sum_i J[target][i] s[m][i] from the state before the iteration (the reduce
 *     kernel, :99-149, then the sum over its block partials, :68-69), energy change
 *     delta = 2 M s (f - M J_perp (s[m-1] + s[m+1])) with periodic slices (:73-77), flip when
 *     -log(u) / beta > delta (:79-81);
 *   - the energy reported after every step is the coupling energy of slice 0,
 *     E = -sum_{i<j} J_ij s_i s_j (:230-236).
 * Reference-mode random numbers: per-spin xorshift32 states seeded with the spin index (:186-191),
 * advanced M times per trial to draw the initial slices (:38-51, :213); the acceptance test reads
 * the spin's state without advancing it (:71, :79, :83), so each spin keeps one random number for
 * the whole run. Hash mode (the build's own default) draws an independent uniform for every
 * (replica, step, iteration, slice) and the initial spins from a counter hash.
 *
 * The natural log of the acceptance test is this file's own (sqa_log: exponent split and the
 * atanh series), shared bit for bit with the device code; the schedule uses the C library's
 * tanhf / logf as the reference's host code does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sb_math_oracle.h"

/* pre_calculate.cu:28-36 */
static uint32_t sqa_xorshift32(uint32_t *state) {
  uint32_t x = *state;
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  *state = x;
  return x;
}

static uint64_t sqa_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* log(u) for u in [0, 1]: u = 2^e m with m in [sqrt(1/2), sqrt(2)), log u = e ln 2 + 2 atanh(s),
 * s = (m - 1) / (m + 1), atanh(s) = s + s^3/3 + s^5/5 + s^7/7 + s^9/9 (|s| <= 0.172: the next
 * term is below 2^-27). ln 2 = hi + lo with hi exact in 16 bits. log(0) = -inf. */
float oracle_sqa_log(float u) { return om_log_unit(u); /* sb_math_oracle.h */ }

/* pre_calculate.cu:206-207, :210, :218-219, :225 */
void oracle_sqa_schedule(int steps, int M, float *beta_out, float *jperp_out) {
  const float increase = (8 - 1 / (float)16) / (float)steps;
  const float G0 = 8.;
  float beta = 1 / (float)16;
  for (int p = 0; p < steps; ++p) {
    const float Gamma = (float)(G0 * (1. - (double)((float)p / (float)steps)));
    const float J_perp = (float)(-0.5 * (double)logf(tanhf((Gamma / (float)M) * beta)) / (double)beta);
    beta_out[p] = beta;
    jperp_out[p] = J_perp;
    beta += increase;
  }
}

/* pre_calculate.cu:38-51 with :186-191, :213: trial r of the TIMES loop continues every spin's
 * xorshift state, so replica r takes calls r M + 1 .. (r + 1) M for its slices and keeps the
 * state after them as its spin's fixed random number. spins [R][M][n], rnd [R][n]. */
void oracle_sqa_init_reference(int n, int M, int R, int8_t *spins, uint32_t *rnd) {
  for (int i = 0; i < n; ++i) {
    uint32_t st = (uint32_t)i;
    for (int r = 0; r < R; ++r) {
      for (int m = 0; m < M; ++m)
        spins[((size_t)r * M + m) * n + i] = (int8_t)(((sqa_xorshift32(&st) & 1u) << 1) - 1);
      rnd[(size_t)r * n + i] = st;
    }
  }
}

void oracle_sqa_init_hash(int n, int M, int R, uint64_t seed, int8_t *spins) {
  for (int r = 0; r < R; ++r)
    for (int m = 0; m < M; ++m)
      for (int i = 0; i < n; ++i) {
        const uint64_t e = ((uint64_t)r * M + m) * n + i;
        const uint64_t z = sqa_mix64(seed + 0x9E3779B97F4A7C15ULL * (e + 1));
        spins[((size_t)r * M + m) * n + i] = (z >> 63) ? -1 : 1;
      }
}

float oracle_sqa_uniform(uint64_t seed, int r, int steps, int p, int iters, int a, int M, int m) {
  const uint64_t e = ((((uint64_t)r * steps + p) * iters + a) * M) + m;
  const uint64_t z = sqa_mix64((seed ^ 0xD1B54A32D192ED03ULL) + 0x9E3779B97F4A7C15ULL * (e + 1));
  return (float)(z >> 40) * 0x1p-24f;
}

/* pre_calculate.cu:231-235 on slice 0 (accumulated in int64 instead of int) */
int64_t oracle_sqa_energy(int n, const int8_t *J, const int8_t *s) {
  int64_t e = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) e -= (int64_t)s[i] * s[j] * J[(size_t)i * n + j];
  return e;
}

/* One run of `steps` annealing steps for R replicas (trials). spins [R][M][n] in / out;
 * trace [R][steps]: slice-0 energy after each step. rng 0: reference random numbers rnd [R][n];
 * rng 1: hash uniforms from seed. Returns 0, or -1 for bad sizes / M > n. */
int oracle_sqa_run(int n, const int8_t *J, int M, int steps, const float *beta_t, const float *jperp_t, int R,
                   int rng, const uint32_t *rnd, uint64_t seed, int8_t *spins, int64_t *trace) {
  if (n < 2 || M < 1 || M > n || steps < 0 || R < 1) return -1;
  const int iters = M + n - 1;
  int32_t *field = (int32_t *)malloc(sizeof(int32_t) * (size_t)M);
  uint8_t *flip = (uint8_t *)malloc((size_t)M);
  for (int r = 0; r < R; ++r) {
    int8_t *S = spins + (size_t)r * M * n;
    for (int p = 0; p < steps; ++p) {
      const float beta = beta_t[p], jp = jperp_t[p];
      for (int a = 0; a < iters; ++a) {
        for (int m = 0; m < M; ++m) {
          const int target = ((a - m) % n + n) % n;
          const int8_t *Jr = J + (size_t)target * n;
          const int8_t *sm = S + (size_t)m * n;
          int32_t f = 0;
          for (int i = 0; i < n; ++i) f += (int32_t)Jr[i] * (int32_t)sm[i];
          field[m] = f;
        }
        for (int m = 0; m < M; ++m) {
          const int target = ((a - m) % n + n) % n;
          const int up = m == 0 ? M - 1 : m - 1, lo = m == M - 1 ? 0 : m + 1;
          const int s = S[(size_t)m * n + target];
          const int nb = S[(size_t)up * n + target] + S[(size_t)lo * n + target];
          /* :76-77 — the float sum of the integer partials is exact; the product with the
           * double 2 M s is exact in double and rounds once to float */
          const float inner = (float)field[m] - ((float)M * jp) * (float)nb;
          const float delta = (float)(2. * (double)M * (double)s * (double)inner);
          float u;
          if (rng == 0) {
            u = (float)rnd[(size_t)r * n + target] / (float)4294967295.0;
          } else {
            u = oracle_sqa_uniform(seed, r, steps, p, iters, a, M, m);
          }
          const float thr = -oracle_sqa_log(u) / beta;
          flip[m] = thr > delta;
        }
        for (int m = 0; m < M; ++m) {
          if (!flip[m]) continue;
          const int target = ((a - m) % n + n) % n;
          S[(size_t)m * n + target] = (int8_t)-S[(size_t)m * n + target];
        }
      }
      if (trace) trace[(size_t)r * steps + p] = oracle_sqa_energy(n, J, S);
    }
  }
  free(field);
  free(flip);
  return 0;
}
