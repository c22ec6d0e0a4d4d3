/*
 * CPU oracle for the SB step loop — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library, and
 * only to verify results or as the timed CPU baseline. The solver never calls it.
 *
 * What it restates (reference file:line, paths inside strongshih/Annealing):
 *   oracle_xorshift32 / oracle_init_reference   SB/CUDA_GPU/m2_opt.cu:38-56 (xorshift32,
 *       prepare_points) with the per-spin seeds initRand[i] = i of m2_opt.cu:136-137; trial r of
 *       the TIMES loop (m2_opt.cu:152-154) continues each spin's xorshift stream, so replica r takes
 *       draws 2r+1 (x) and 2r+2 (y).
 *   oracle_asb_local                            SB/CUDA_GPU/m2_opt.cu:58-75 (UpdateTwice). The
 *       constants K, detune, deltaT are double literals in the reference (m2_opt.cu:16-19), so C's
 *       usual conversions evaluate the update in double and round to float on assignment; this does
 *       the same.
 *   oracle_asb_run                              SB/CUDA_GPU/m2_opt.cu:148-187: per step
 *       amplitude = s/(float)STEP (:158), UpdateTwice (:168), then cublasSgemv y = coeff1*J*x + y
 *       with coeff1 = DeltaT*xi (:148, :169). cuBLAS's summation order is not published; the field
 *       here is summed in index order (the order of the cuBLAS-free twin
 *       SB/CUDA_GPU/Bifurcation_m2.cu.c:93-95) and the kick is fmaf(coeff1, f, y).
 *   oracle_energy_i64 / oracle_energy_f64       SB/CUDA_GPU/m2_opt.cu:192-202 with
 *       s = x > 0 ? 1 : -1 and the reported value -E; h_i s_i terms follow the reference project's README.md:9-13.
 *   oracle_sb_update_f32 / oracle_sb_run        bSB / dSB of Goto et al., Sci. Adv. 7, eabe7953
 *       (2021) (no reference code exists for these): y += dt*(-(a0-a(t)) x + c0 (f + h)),
 *       x += dt*a0*y, |x| > 1 -> x = sign(x), y = 0, with f = J x (bSB) or J sign(x) (dSB). The
 *       operation order and roundings are the ones the CUDA kernels use, so the FP32 dSB trajectory
 *       is bitwise equal to the device's.
 *
 * Parity pins: the reference ships no test vectors for this path (its only per-step data,
 * SB/CUDA_GPU/plot_figure/plot_energy_decrease/*_stats.csv, is for an instance that is not
 * shipped). The pins are (a) tests/golden/ trajectories produced by the reference's own kernels
 * (prepare_points, UpdateTwice) compiled from its sources plus cuBLAS SGEMV, and (b) the energy
 * distribution of those CSVs used as a statistical band.
 *
 * Build: -O2 -ffp-contract=off (no fused multiply-add except the explicit fmaf calls).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- initial state ---------------- */

uint32_t oracle_xorshift32(uint32_t *state) {
  uint32_t v = *state;
  v ^= v << 13;
  v ^= v >> 17;
  v ^= v << 5;
  *state = v;
  return v;
}

/* prepare_points value: ((u / (float)MAX) / 10.0). (float)4294967295.0 rounds to 2^32, so the float
 * division is an exact scaling; the "/ 10.0" is a double division rounded back to float. */
static float ref_unit(uint32_t u) {
  float q = (float)u / 4294967296.0f;
  return (float)((double)q / 10.0);
}

void oracle_init_reference(int n, int replicas, float *x, float *y) {
  for (int i = 0; i < n; ++i) {
    uint32_t st = (uint32_t)i;
    for (int r = 0; r < replicas; ++r) {
      uint32_t ux = oracle_xorshift32(&st);
      uint32_t uy = oracle_xorshift32(&st);
      x[(size_t)r * n + i] = ref_unit(ux);
      y[(size_t)r * n + i] = ref_unit(uy);
    }
  }
}

static uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return z;
}

/* Uniform [-0.1, 0.1): element index e = 2*(r*n + i) + {0: x, 1: y}. */
float oracle_uniform_value(uint64_t seed, uint64_t e) {
  uint64_t z = mix64(seed + 0x9E3779B97F4A7C15ULL * (e + 1));
  uint32_t u = (uint32_t)(z >> 40);
  float f = (float)u * 5.9604644775390625e-08f; /* 2^-24 */
  float t = f * 2.0f - 1.0f;                    /* exact */
  return t * 0.1f;
}

void oracle_init_uniform(int n, int replicas, uint64_t seed, float *x, float *y) {
  for (int r = 0; r < replicas; ++r)
    for (int i = 0; i < n; ++i) {
      uint64_t e = 2 * ((uint64_t)r * (uint64_t)n + (uint64_t)i);
      x[(size_t)r * n + i] = oracle_uniform_value(seed, e);
      y[(size_t)r * n + i] = oracle_uniform_value(seed, e + 1);
    }
}

/* ---------------- schedule and coefficients ---------------- */

float oracle_pump(float a0, int t, int steps) {
  float a = (float)((double)a0 * (double)t / (double)steps);
  return a0 - a;
}

double oracle_coupling_std(int n, const float *J) {
  if (n < 2) return 0.0;
  double s = 0.0, s2 = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (i == j) continue;
      double v = (double)J[(size_t)i * n + j];
      s += v;
      s2 += v * v;
    }
  double cnt = (double)n * (double)(n - 1);
  double mean = s / cnt;
  double var = s2 / cnt - mean * mean;
  return var > 0.0 ? sqrt(var) : 0.0;
}

float oracle_default_c0(int n, const float *J) {
  double sd = oracle_coupling_std(n, J);
  if (!(sd > 0.0)) sd = 1.0;
  return (float)(0.5 / (sqrt((double)n) * sd));
}

/* ---------------- fields ---------------- */

/* f[r][i] = sum_j J[i][j] * v[r][j], FP32, index order */
void oracle_field_f32(int n, int replicas, const float *J, const float *v, float *f) {
  for (int r = 0; r < replicas; ++r) {
    const float *vr = v + (size_t)r * n;
    for (int i = 0; i < n; ++i) {
      const float *Ji = J + (size_t)i * n;
      float acc = 0.0f;
      for (int j = 0; j < n; ++j) acc = acc + Ji[j] * vr[j];
      f[(size_t)r * n + i] = acc;
    }
  }
}

void oracle_field_f64(int n, int replicas, const float *J, const double *v, double *f) {
  for (int r = 0; r < replicas; ++r) {
    const double *vr = v + (size_t)r * n;
    for (int i = 0; i < n; ++i) {
      const float *Ji = J + (size_t)i * n;
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc = acc + (double)Ji[j] * vr[j];
      f[(size_t)r * n + i] = acc;
    }
  }
}

void oracle_signs_f32(size_t count, const float *x, float *s) {
  for (size_t k = 0; k < count; ++k) s[k] = x[k] > 0.0f ? 1.0f : -1.0f;
}

/* ---------------- bSB / dSB ---------------- */

void oracle_sb_update_f32(int n, int replicas, const float *f, const float *h, float *x, float *y,
                          float pump, float c0, float dt, float dta0) {
  for (int r = 0; r < replicas; ++r)
    for (int i = 0; i < n; ++i) {
      size_t k = (size_t)r * n + i;
      float fv = f[k];
      if (h) fv = fv + h[i];
      float g = c0 * fv;
      float force = fmaf(-pump, x[k], g);
      float yv = fmaf(dt, force, y[k]);
      float xv = fmaf(dta0, yv, x[k]);
      if (fabsf(xv) > 1.0f) {
        xv = copysignf(1.0f, xv);
        yv = 0.0f;
      }
      x[k] = xv;
      y[k] = yv;
    }
}

void oracle_sb_update_f64(int n, int replicas, const double *f, const float *h, double *x,
                          double *y, double pump, double c0, double dt, double a0) {
  for (int r = 0; r < replicas; ++r)
    for (int i = 0; i < n; ++i) {
      size_t k = (size_t)r * n + i;
      double fv = f[k] + (h ? (double)h[i] : 0.0);
      double yv = y[k] + dt * (-pump * x[k] + c0 * fv);
      double xv = x[k] + dt * a0 * yv;
      if (fabs(xv) > 1.0) {
        xv = xv > 0 ? 1.0 : -1.0;
        yv = 0.0;
      }
      x[k] = xv;
      y[k] = yv;
    }
}

/* energy of s = sign(x) for each replica, double */
static void energies_of_x_f32(int n, int replicas, const float *J, const float *h, const float *x,
                              double *e_out);

/* Full bSB/dSB run in FP32 (variant 1 = bSB, 2 = dSB). x, y hold the initial state and receive the
 * final one. trace (steps+1 doubles, may be NULL) gets the min-over-replicas energy of s(t) for
 * t = 0..steps; trace_all ((steps+1)*replicas, may be NULL) every replica's. */
void oracle_sb_run_f32(int variant, int n, int replicas, const float *J, const float *h, float *x,
                       float *y, int steps, float a0, float c0, float dt, double *trace,
                       double *trace_all) {
  size_t cnt = (size_t)n * replicas;
  float *v = (float *)malloc(cnt * sizeof(float));
  float *f = (float *)malloc(cnt * sizeof(float));
  double *e = (double *)malloc((size_t)replicas * sizeof(double));
  float dta0 = dt * a0;
  for (int t = 0; t <= steps; ++t) {
    if (trace || trace_all) {
      energies_of_x_f32(n, replicas, J, h, x, e);
      double m = e[0];
      for (int r = 0; r < replicas; ++r) {
        if (e[r] < m) m = e[r];
        if (trace_all) trace_all[(size_t)t * replicas + r] = e[r];
      }
      if (trace) trace[t] = m;
    }
    if (t == steps) break;
    if (variant == 2)
      oracle_signs_f32(cnt, x, v);
    else
      memcpy(v, x, cnt * sizeof(float));
    oracle_field_f32(n, replicas, J, v, f);
    oracle_sb_update_f32(n, replicas, f, h, x, y, oracle_pump(a0, t, steps), c0, dt, dta0);
  }
  free(v);
  free(f);
  free(e);
}

/* The same in FP64 from the same FP32 initial state (x0, y0); results in xd, yd. */
void oracle_sb_run_f64(int variant, int n, int replicas, const float *J, const float *h,
                       const float *x0, const float *y0, double *xd, double *yd, int steps,
                       double a0, double c0, double dt) {
  size_t cnt = (size_t)n * replicas;
  double *v = (double *)malloc(cnt * sizeof(double));
  double *f = (double *)malloc(cnt * sizeof(double));
  for (size_t k = 0; k < cnt; ++k) {
    xd[k] = x0[k];
    yd[k] = y0[k];
  }
  for (int t = 0; t < steps; ++t) {
    for (size_t k = 0; k < cnt; ++k)
      v[k] = (variant == 2) ? (xd[k] > 0.0 ? 1.0 : -1.0) : xd[k];
    oracle_field_f64(n, replicas, J, v, f);
    double pump = a0 - a0 * (double)t / (double)steps;
    oracle_sb_update_f64(n, replicas, f, h, xd, yd, pump, c0, dt, a0);
  }
  free(v);
  free(f);
}

/* ---------------- aSB (the reference algorithm) ---------------- */

void oracle_asb_local(size_t count, float *x, float *y, float amp, int m, float mts_dt,
                      float detune, float kerr) {
  double dd = detune, dk = kerr, dh = mts_dt, da = amp;
  for (size_t k = 0; k < count; ++k) {
    float lx = x[k], ly = y[k];
    for (int s = 0; s < m; ++s) {
      lx = (float)((double)lx + dd * (double)ly * dh);
      double x3 = dk * (double)lx * (double)lx * (double)lx;
      ly = (float)((double)ly - dh * (x3 + (dd - da) * (double)lx));
    }
    x[k] = lx;
    y[k] = ly;
  }
}

/* coeff1 = DeltaT * xi rounded to float (m2_opt.cu:148) */
float oracle_asb_coeff(float coupling_dt, float xi) {
  return (float)((double)coupling_dt * (double)xi);
}

float oracle_asb_amplitude(int s, int steps) { return (float)s / (float)steps; }

void oracle_asb_kick(int n, int replicas, const float *f, float coeff, float *y) {
  size_t cnt = (size_t)n * replicas;
  for (size_t k = 0; k < cnt; ++k) y[k] = fmaf(coeff, f[k], y[k]);
}

/* Full aSB run; x_trace (may be NULL) receives x after every step: steps * replicas * n floats. */
void oracle_asb_run(int n, int replicas, const float *J, float *x, float *y, int steps, int m,
                    float mts_dt, float coupling_dt, float xi, float detune, float kerr,
                    float *x_trace, float *y_trace) {
  size_t cnt = (size_t)n * replicas;
  float *f = (float *)malloc(cnt * sizeof(float));
  float coeff = oracle_asb_coeff(coupling_dt, xi);
  for (int s = 0; s < steps; ++s) {
    float amp = oracle_asb_amplitude(s, steps);
    oracle_asb_local(cnt, x, y, amp, m, mts_dt, detune, kerr);
    oracle_field_f32(n, replicas, J, x, f);
    oracle_asb_kick(n, replicas, f, coeff, y);
    if (x_trace) memcpy(x_trace + (size_t)s * cnt, x, cnt * sizeof(float));
    if (y_trace) memcpy(y_trace + (size_t)s * cnt, y, cnt * sizeof(float));
  }
  free(f);
}

/* ---------------- energies ---------------- */

/* returns 0 on success, 1 if a coupling or field is not an integer */
int oracle_energy_i64(int n, const float *J, const float *h, const int8_t *s, int64_t *out) {
  int64_t e = 0;
  for (int i = 0; i < n; ++i) {
    const float *Ji = J + (size_t)i * n;
    int64_t row = 0;
    for (int j = i + 1; j < n; ++j) {
      float w = Ji[j];
      if (w != floorf(w)) return 1;
      row += (int64_t)w * (int64_t)s[j];
    }
    e -= row * (int64_t)s[i];
    if (h) {
      if (h[i] != floorf(h[i])) return 1;
      e -= (int64_t)h[i] * (int64_t)s[i];
    }
  }
  *out = e;
  return 0;
}

double oracle_energy_f64(int n, const float *J, const float *h, const int8_t *s) {
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    const float *Ji = J + (size_t)i * n;
    double row = 0.0;
    for (int j = i + 1; j < n; ++j) row += (double)Ji[j] * (double)s[j];
    e -= row * (double)s[i];
    if (h) e -= (double)h[i] * (double)s[i];
  }
  return e;
}

static void energies_of_x_f32(int n, int replicas, const float *J, const float *h, const float *x,
                              double *e_out) {
  int8_t *s = (int8_t *)malloc((size_t)n);
  for (int r = 0; r < replicas; ++r) {
    for (int i = 0; i < n; ++i) s[i] = x[(size_t)r * n + i] > 0.0f ? 1 : -1;
    e_out[r] = oracle_energy_f64(n, J, h, s);
  }
  free(s);
}

void oracle_energies_of_x(int n, int replicas, const float *J, const float *h, const float *x,
                          double *e_out) {
  energies_of_x_f32(n, replicas, J, h, x, e_out);
}
