/*
 * Multithreaded FP32 CPU port of the SB step loop — the timed CPU baseline. TEST / BENCH
 * INFRASTRUCTURE ONLY: bench.py's CPU-baseline leg and `bench.py --impl reference` time it; the
 * solver never calls it.
 *
 * The reference has no CPU implementation of this path; this is a C port of its step loop:
 *   aSB: UpdateTwice (SB/CUDA_GPU/m2_opt.cu:58-75) on every spin, then the dense matrix-vector
 *        coupling kick y += DeltaT*xi*J*x (m2_opt.cu:169), amplitude s/STEP (m2_opt.cu:158);
 *   bSB / dSB: the same loop with the Goto et al. (2021) update (see sb_oracle.c), field J*x or
 *        J*sign(x).
 * Replicas are independent trajectories (the reference's TIMES trials, m2_opt.cu:152).
 *
 * Parallelism: POSIX threads; each step has three phases separated by a barrier:
 * (1) per replica: the vector the field multiplies (x, sign(x), or x after the aSB local update);
 * (2) the field F = V * J^T as a blocked FP32 product over 64x64 (replica, spin) tiles with 4x4
 *     register micro-tiles (GCC vector extensions, portable to x86-64 and aarch64);
 * (3) per replica: the state update.
 * Build: -O3 -ffp-contract=fast (this file is a timed baseline, not a bit-exact restatement).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef float v4 __attribute__((vector_size(16)));

typedef struct {
  int variant, n, np, replicas, steps, m, nthreads;
  const float *J; /* np-pitched, zero padded */
  const float *h;
  float *x, *y;   /* replicas * n (caller layout) */
  float *v, *f;   /* replicas * np */
  float a0, c0, dt, mts_dt, coeff, detune, kerr;
  pthread_barrier_t bar;
} job_t;

typedef struct {
  job_t *job;
  int tid;
} arg_t;

static void field_tile(const job_t *jb, int r0, int r1, int i0, int i1) {
  const int np = jb->np;
  for (int r = r0; r < r1; r += 4) {
    int rc = r1 - r < 4 ? r1 - r : 4;
    for (int i = i0; i < i1; i += 4) {
      int ic = i1 - i < 4 ? i1 - i : 4;
      v4 acc[4][4];
      memset(acc, 0, sizeof(acc));
      const float *vr[4], *Ji[4];
      for (int a = 0; a < 4; ++a) vr[a] = jb->v + (size_t)(r + (a < rc ? a : 0)) * np;
      for (int b = 0; b < 4; ++b) Ji[b] = jb->J + (size_t)(i + (b < ic ? b : 0)) * np;
      for (int k = 0; k < np; k += 4) {
        v4 va[4], jbv[4];
        for (int a = 0; a < 4; ++a) memcpy(&va[a], vr[a] + k, 16);
        for (int b = 0; b < 4; ++b) memcpy(&jbv[b], Ji[b] + k, 16);
        for (int a = 0; a < 4; ++a)
          for (int b = 0; b < 4; ++b) acc[a][b] += va[a] * jbv[b];
      }
      for (int a = 0; a < rc; ++a)
        for (int b = 0; b < ic; ++b) {
          v4 s = acc[a][b];
          jb->f[(size_t)(r + a) * np + i + b] = (s[0] + s[1]) + (s[2] + s[3]);
        }
    }
  }
}

static void *worker(void *p) {
  arg_t *ag = (arg_t *)p;
  job_t *jb = ag->job;
  const int T = jb->nthreads, tid = ag->tid, n = jb->n, np = jb->np, R = jb->replicas;
  const int TB = 64;
  const int nrb = (R + TB - 1) / TB, nib = (n + TB - 1) / TB;
  const float dta0 = jb->dt * jb->a0;
  for (int t = 0; t < jb->steps; ++t) {
    /* phase 1: the multiplied vector */
    for (int r = tid; r < R; r += T) {
      float *xr = jb->x + (size_t)r * n, *yr = jb->y + (size_t)r * n;
      float *vr = jb->v + (size_t)r * np;
      if (jb->variant == 0) {
        float amp = (float)t / (float)jb->steps;
        double dd = jb->detune, dk = jb->kerr, dh = jb->mts_dt;
        for (int i = 0; i < n; ++i) {
          float lx = xr[i], ly = yr[i];
          for (int s = 0; s < jb->m; ++s) {
            lx = (float)((double)lx + dd * (double)ly * dh);
            ly = (float)((double)ly - dh * (dk * lx * lx * lx + (dd - (double)amp) * lx));
          }
          xr[i] = lx;
          yr[i] = ly;
          vr[i] = lx;
        }
      } else if (jb->variant == 2) {
        for (int i = 0; i < n; ++i) vr[i] = xr[i] > 0.0f ? 1.0f : -1.0f;
      } else {
        memcpy(vr, xr, (size_t)n * sizeof(float));
      }
    }
    pthread_barrier_wait(&jb->bar);
    /* phase 2: field */
    for (int tile = tid; tile < nrb * nib; tile += T) {
      int rb = tile / nib, ib = tile % nib;
      int r0 = rb * TB, r1 = r0 + TB < R ? r0 + TB : R;
      int i0 = ib * TB, i1 = i0 + TB < n ? i0 + TB : n;
      field_tile(jb, r0, r1, i0, i1);
    }
    pthread_barrier_wait(&jb->bar);
    /* phase 3: update */
    float a = (float)((double)jb->a0 * (double)t / (double)jb->steps);
    float pump = jb->a0 - a;
    for (int r = tid; r < R; r += T) {
      float *xr = jb->x + (size_t)r * n, *yr = jb->y + (size_t)r * n;
      const float *fr = jb->f + (size_t)r * np;
      if (jb->variant == 0) {
        for (int i = 0; i < n; ++i) yr[i] = fmaf(jb->coeff, fr[i], yr[i]);
      } else {
        for (int i = 0; i < n; ++i) {
          float fv = fr[i] + (jb->h ? jb->h[i] : 0.0f);
          float yv = fmaf(jb->dt, fmaf(-pump, xr[i], jb->c0 * fv), yr[i]);
          float xv = fmaf(dta0, yv, xr[i]);
          if (fabsf(xv) > 1.0f) {
            xv = copysignf(1.0f, xv);
            yv = 0.0f;
          }
          xr[i] = xv;
          yr[i] = yv;
        }
      }
    }
    pthread_barrier_wait(&jb->bar);
  }
  return NULL;
}

/* Runs `steps` steps on (x, y) in place. variant 0 = aSB, 1 = bSB, 2 = dSB. Returns 0 on success. */
int oracle_cpu_run(int variant, int n, int replicas, const float *J, const float *h, float *x,
                   float *y, int steps, float a0, float c0, float dt, int m, float mts_dt,
                   float coupling_dt, float xi, float detune, float kerr, int nthreads) {
  if (n <= 0 || replicas <= 0 || steps < 0 || nthreads <= 0) return 1;
  job_t jb;
  memset(&jb, 0, sizeof(jb));
  jb.variant = variant;
  jb.n = n;
  jb.np = (n + 3) & ~3;
  jb.replicas = replicas;
  jb.steps = steps;
  jb.m = m;
  jb.nthreads = nthreads;
  jb.h = h;
  jb.x = x;
  jb.y = y;
  jb.a0 = a0;
  jb.c0 = c0;
  jb.dt = dt;
  jb.mts_dt = mts_dt;
  jb.coeff = (float)((double)coupling_dt * (double)xi);
  jb.detune = detune;
  jb.kerr = kerr;
  size_t jsz = (size_t)n * jb.np, vsz = (size_t)replicas * jb.np;
  float *Jp = (float *)aligned_alloc(64, ((jsz * 4 + 63) / 64) * 64);
  jb.v = (float *)aligned_alloc(64, ((vsz * 4 + 63) / 64) * 64);
  jb.f = (float *)aligned_alloc(64, ((vsz * 4 + 63) / 64) * 64);
  if (!Jp || !jb.v || !jb.f) {
    free(Jp);
    free(jb.v);
    free(jb.f);
    return 2;
  }
  memset(Jp, 0, jsz * 4);
  memset(jb.v, 0, vsz * 4);
  for (int i = 0; i < n; ++i) memcpy(Jp + (size_t)i * jb.np, J + (size_t)i * n, (size_t)n * 4);
  jb.J = Jp;
  pthread_barrier_init(&jb.bar, NULL, (unsigned)nthreads);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
  arg_t *args = (arg_t *)malloc(sizeof(arg_t) * (size_t)nthreads);
  for (int k = 0; k < nthreads; ++k) {
    args[k].job = &jb;
    args[k].tid = k;
    if (k > 0) pthread_create(&th[k], NULL, worker, &args[k]);
  }
  worker(&args[0]);
  for (int k = 1; k < nthreads; ++k) pthread_join(th[k], NULL);
  pthread_barrier_destroy(&jb.bar);
  free(th);
  free(args);
  free(Jp);
  free(jb.v);
  free(jb.f);
  return 0;
}
