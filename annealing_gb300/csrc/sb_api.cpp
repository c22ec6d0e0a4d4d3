// C ABI implementation: contexts, plans (device-resident solves) and sb_solve.
//
// A solve is the reference's trial loop turned sideways (SB/CUDA_GPU/m2_opt.cu:152-203): the
// TIMES trials become R replicas that advance together, the per-step UpdateTwice + cublasSgemv
// pair (m2_opt.cu:168-169) becomes one fused step kernel (plain FP32) or one tensor-core step
// kernel, and the host O(N^2) energy loop (m2_opt.cu:192-202) becomes a device reduction whose
// result for the returned spin vector is re-checked on the host in exact int64.
// The step loop is captured once per plan into a CUDA graph and replayed.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "sb.h"
#include "sb_host.h"
#include "sb_internal.h"
#include "sb_ctx.h"
#include "sb_serve.h"

namespace {
thread_local std::string g_thread_error;
}

void sbh::set_thread_error(const std::string &e) { g_thread_error = e; }
const char *sbh::thread_error() { return g_thread_error.c_str(); }

struct PlanKey {
  int n, R, steps, variant, mode, dtype, init, trace, trace_all, has_h;
  float c0, coeff, dt, a0, mts_dt, detune, kerr;
  int m;
  bool operator==(const PlanKey &o) const { return memcmp(this, &o, sizeof(PlanKey)) == 0; }
};

struct sb_plan {
  sb_ctx *ctx = nullptr;
  const sb_problem *prob = nullptr;  // host problem (kept alive by the caller)
  sb_params prm{};
  PlanKey key{};
  int n = 0, R = 0, jp = 0, xp = 0;
  int mode = SB_FIELD_FP32, dtype = 0;
  bool integral = false;
  bool split_exact = false;  // integer couplings held exactly by BF16 hi + lo (|J| < 2^16)
  float c0 = 0, coeff = 0, dta0 = 0;
  float *dJ = nullptr, *dh = nullptr, *dx[2] = {nullptr, nullptr}, *dy = nullptr;
  double *denergy = nullptr;
  uint32_t *dstatus = nullptr;
  float *dpump = nullptr;  // [steps] a0 - a(t), the schedule every kernel reads
  // plain FP32 SB that fits one cooperative launch: the exchange lines of PlainPersist
  unsigned long long *dwords = nullptr;
  size_t words_bytes = 0;
  float *dxk = nullptr;    // [kTopK][xp] rows of the best candidates (real-valued J)
  double *dek = nullptr;   // [kTopK] their FP64 energies
  // compact copy of integer couplings for the host re-check, built on a background thread while
  // the device solves (it reads the caller's problem: reset before that may go away)
  std::unique_ptr<sbh::CouplingCopies> copies;
  sbk::TcEngine *tc = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int64_t launches_in_loop = 0;
};

namespace {

constexpr int kTopK = 8;  // replicas whose energy is recomputed in FP64 for real-valued couplings

#define SB_CUDA(call)                                                                       \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      err = std::string(#call) + ": " + cudaGetErrorString(_e);                             \
      return _e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;                    \
    }                                                                                       \
  } while (0)

sb_status check_params(const sb_problem *p, const sb_params *prm, std::string &err) {
  if (!p || !p->J || p->n <= 0) {
    err = "problem is empty";
    return SB_ERR_INVALID_ARG;
  }
  if (p->n > 65536) {
    err = "n above 65536";
    return SB_ERR_INVALID_ARG;
  }
  if (!prm || prm->steps < 0 || prm->steps > (1 << 24) || prm->replicas <= 0 ||
      prm->replicas > 65536) {
    err = "steps must be in [0, 2^24] and replicas in [1, 65536]";
    return SB_ERR_INVALID_ARG;
  }
  if (prm->variant < SB_ASB || prm->variant > SB_DSB || prm->field_mode < SB_FIELD_AUTO ||
      prm->field_mode > SB_FIELD_TC || prm->init_mode < 0 || prm->init_mode > 1) {
    err = "unknown variant, field mode or init mode";
    return SB_ERR_INVALID_ARG;
  }
  if (prm->variant == SB_ASB && (prm->mts_m < 0 || prm->mts_m > 64)) {
    err = "mts_m must be in [0, 64]";
    return SB_ERR_INVALID_ARG;
  }
  if ((size_t)p->n * (size_t)prm->replicas > ((size_t)1 << 31)) {
    err = "n * replicas above 2^31";
    return SB_ERR_INVALID_ARG;
  }
  return SB_OK;
}

// Field mode and operand dtype for (problem, params).
sb_status resolve_mode(const sb_problem *p, const sb_params *prm, int &mode, int &dtype,
                       std::string &err) {
  mode = prm->field_mode;
  if (mode == SB_FIELD_AUTO)
    mode = (prm->variant != SB_ASB && prm->replicas >= 32) ? SB_FIELD_TC : SB_FIELD_FP32;
  dtype = 0;
  if (mode == SB_FIELD_FP32) return SB_OK;
  if (prm->variant == SB_ASB) {
    err = "aSB runs on the plain FP32 path only";
    return SB_ERR_UNSUPPORTED;
  }
  const int want = prm->operand_dtype;
  if (want < SB_OPERAND_AUTO || want > SB_OPERAND_FP6) {
    err = "unknown operand_dtype";
    return SB_ERR_INVALID_ARG;
  }
  if (want == SB_OPERAND_FP6) {
    err = "E2M3 operands run on the grouped path (sb_batch_*, serving)";
    return SB_ERR_UNSUPPORTED;
  }
  if (prm->variant == SB_DSB) {
    const bool fp4 = p->integer_valued && p->max_abs_j <= 4 && sbk::tc_fp4_fits(p->n, prm->replicas);
    if (want == SB_OPERAND_AUTO) {
      if (fp4)
        dtype = sbk::kTcFp4;
      else if (p->integer_valued && p->max_abs_j <= 16)
        dtype = sbk::kTcFp8;
      else if (p->integer_valued && p->max_abs_j <= 256)
        dtype = sbk::kTcBf16;
      else
        dtype = sbk::kTcBf16Split;
    } else {
      const bool exact = want == SB_OPERAND_FP4    ? fp4
                         : want == SB_OPERAND_FP8  ? (p->integer_valued && p->max_abs_j <= 16)
                         : want == SB_OPERAND_BF16 ? (p->integer_valued && p->max_abs_j <= 256)
                                                   : true;
      if (!exact) {
        err = "the requested operand_dtype is not exact for these couplings (or, for FP4, this size)";
        return SB_ERR_UNSUPPORTED;
      }
      dtype = want;  // sb_operand_dtype and TcDtype share their codes
    }
  } else {
    if (want != SB_OPERAND_AUTO && want != SB_OPERAND_BF16X2 && want != SB_OPERAND_FP16X2) {
      err = "bSB on tensor cores runs split operands only (BF16 or FP16 hi + lo)";
      return SB_ERR_UNSUPPORTED;
    }
    dtype = want == SB_OPERAND_FP16X2 ? sbk::kTcFp16Split : sbk::kTcBf16Split;
    if (prm->trace || prm->trace_all) {
      err = "per-step energy traces of bSB are produced by the plain FP32 path only";
      return SB_ERR_UNSUPPORTED;
    }
  }
  return SB_OK;
}

PlanKey make_key(const sb_problem *p, const sb_params *prm, int mode, int dtype, float c0,
                 float coeff) {
  PlanKey k;
  memset(&k, 0, sizeof(k));
  k.n = p->n;
  k.R = prm->replicas;
  k.steps = prm->steps;
  k.variant = prm->variant;
  k.mode = mode;
  k.dtype = dtype;
  k.init = prm->init_mode;
  k.trace = prm->trace;
  k.trace_all = prm->trace_all;
  k.has_h = p->h != nullptr;
  k.c0 = c0;
  k.coeff = coeff;
  k.dt = prm->dt;
  k.a0 = prm->a0;
  k.mts_dt = prm->mts_dt;
  k.detune = prm->detune;
  k.kerr = prm->kerr;
  k.m = prm->mts_m;
  return k;
}

void plan_free_device(sb_plan *pl) {
  if (pl->graph) cudaGraphExecDestroy(pl->graph);
  if (pl->tc) sbk::tc_destroy(pl->tc);
  cudaFree(pl->dJ);
  cudaFree(pl->dh);
  cudaFree(pl->dx[0]);
  cudaFree(pl->dx[1]);
  cudaFree(pl->dy);
  cudaFree(pl->denergy);
  cudaFree(pl->dstatus);
  cudaFree(pl->dpump);
  cudaFree(pl->dxk);
  cudaFree(pl->dek);
  cudaFree(pl->dwords);
  pl->dwords = nullptr;
  pl->dpump = nullptr;
  pl->dxk = nullptr;
  pl->dek = nullptr;
  if (pl->ev0) cudaEventDestroy(pl->ev0);
  if (pl->ev1) cudaEventDestroy(pl->ev1);
  pl->graph = nullptr;
  pl->tc = nullptr;
  pl->dJ = pl->dh = pl->dx[0] = pl->dx[1] = pl->dy = nullptr;
  pl->denergy = nullptr;
  pl->dstatus = nullptr;
  pl->ev0 = pl->ev1 = nullptr;
}

bool needs_trace(const sb_params &p) { return p.trace || p.trace_all; }

size_t energy_slots(const sb_params &p) { return needs_trace(p) ? (size_t)p.steps + 1 : 1; }

// Upload the problem's couplings and field into an existing plan (shapes already match).
sb_status upload_problem(sb_plan *pl, const sb_problem *p, std::string &err) {
  cudaStream_t st = pl->ctx->stream;
  const int n = pl->n;
  SB_CUDA(cudaMemsetAsync(pl->dJ, 0, (size_t)n * pl->jp * sizeof(float), st));
  SB_CUDA(cudaMemcpy2DAsync(pl->dJ, (size_t)pl->jp * sizeof(float), p->J, (size_t)n * sizeof(float),
                            (size_t)n * sizeof(float), (size_t)n, cudaMemcpyHostToDevice, st));
  if (p->h) SB_CUDA(cudaMemcpyAsync(pl->dh, p->h, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
  if (pl->mode == SB_FIELD_TC) {
    if (pl->tc) {
      // same shapes: re-convert the new couplings into the engine's operand buffers
      SB_CUDA(sbk::tc_reload(pl->tc, pl->dJ, pl->jp, st));
    } else {
      sbk::TcSetup s{pl->prm.variant, pl->dtype, n, pl->R, pl->xp};
      sb_status ts = sbk::tc_create(&pl->tc, s, pl->dJ, pl->jp, err, st);
      if (ts != SB_OK) return ts;
    }
  }
  pl->copies.reset();
  pl->prob = p;
  if (p->integer_valued) pl->copies.reset(new sbh::CouplingCopies({p}));
  return SB_OK;
}

sb_status plan_create(sb_ctx *ctx, const sb_problem *p, const sb_params *prm, sb_plan **out,
                      std::string &err) {
  sb_status s = check_params(p, prm, err);
  if (s != SB_OK) return s;
  int mode, dtype;
  s = resolve_mode(p, prm, mode, dtype, err);
  if (s != SB_OK) return s;
  sb_plan *pl = new sb_plan();
  pl->ctx = ctx;
  pl->prm = *prm;
  pl->n = p->n;
  pl->R = prm->replicas;
  pl->jp = sbk::pitch_for(p->n, 4);
  pl->xp = pl->jp;
  pl->mode = mode;
  pl->dtype = dtype;
  pl->integral = p->integer_valued != 0;
  pl->split_exact = pl->integral && p->max_abs_j < 65536;
  pl->c0 = prm->c0 > 0.0f ? prm->c0 : sb_default_c0(p);
  const float xi = prm->xi > 0.0f ? prm->xi : (float)(0.7 * (double)prm->detune / sqrt((double)p->n));
  pl->coeff = (float)((double)prm->coupling_dt * (double)xi);
  pl->dta0 = prm->dt * prm->a0;
  pl->key = make_key(p, prm, mode, dtype, pl->c0, pl->coeff);
  const size_t xs = (size_t)pl->R * pl->xp * sizeof(float);
  auto fail = [&](sb_status st) {
    plan_free_device(pl);
    delete pl;
    return st;
  };
  cudaError_t e;
#define PLAN_ALLOC(ptr, bytes)                                                \
  e = cudaMalloc((void **)&(ptr), (bytes));                                   \
  if (e != cudaSuccess) {                                                     \
    err = std::string("cudaMalloc: ") + cudaGetErrorString(e);                \
    return fail(e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA);   \
  }
  PLAN_ALLOC(pl->dJ, (size_t)pl->n * pl->jp * sizeof(float));
  if (p->h) {
    PLAN_ALLOC(pl->dh, (size_t)pl->n * sizeof(float));
  }
  PLAN_ALLOC(pl->dx[0], xs);
  if (mode == SB_FIELD_FP32) {
    PLAN_ALLOC(pl->dx[1], xs);
  }
  PLAN_ALLOC(pl->dy, xs);
  PLAN_ALLOC(pl->denergy, energy_slots(*prm) * (size_t)pl->R * sizeof(double));
  PLAN_ALLOC(pl->dstatus, sizeof(uint32_t));
  PLAN_ALLOC(pl->dpump, (size_t)(prm->steps > 0 ? prm->steps : 1) * sizeof(float));
  // plain FP32 solves whose rows fit one co-resident grid run every step in one launch (N=2000,
  // 1000 steps: dSB 5.7 -> 1.6 ms, its signs one tagged word per CTA; bSB 6.3 -> 1.5 ms and aSB
  // 7.4 -> 2.6 ms, x as sixteen tagged words per CTA read by sixteen threads together, aSB's FP64
  // sub-steps for a CTA's 16 rows in one warp); SB_PLAIN_PERSIST=0 keeps one launch per step
  if (mode == SB_FIELD_FP32 && !needs_trace(*prm) && prm->steps > 0) {
    const char *env = getenv("SB_PLAIN_PERSIST");
    const bool want = !(env && env[0] == '0');
    const int ctas = want ? sbk::plain_persist_ctas(pl->n, pl->R, pl->jp) : 0;
    if (ctas > 0) {
      pl->words_bytes = (size_t)2 * ctas * 128;  // one 128-byte line per CTA's word
      PLAN_ALLOC(pl->dwords, pl->words_bytes);
    }
  }
#undef PLAN_ALLOC
  {
    std::vector<float> pumps((size_t)(prm->steps > 0 ? prm->steps : 1), 0.0f);
    for (int t = 0; t < prm->steps; ++t) pumps[t] = sb_pump(prm->a0, t, prm->steps);
    if (cudaMemcpy(pl->dpump, pumps.data(), pumps.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
      err = "uploading the pump schedule failed";
      return fail(SB_ERR_CUDA);
    }
  }
  // padding columns of the state stay zero for the life of the plan
  if (cudaMemsetAsync(pl->dx[0], 0, xs, ctx->stream) != cudaSuccess ||
      (pl->dx[1] && cudaMemsetAsync(pl->dx[1], 0, xs, ctx->stream) != cudaSuccess) ||
      cudaMemsetAsync(pl->dy, 0, xs, ctx->stream) != cudaSuccess ||
      cudaEventCreate(&pl->ev0) != cudaSuccess || cudaEventCreate(&pl->ev1) != cudaSuccess) {
    err = "plan setup failed";
    return fail(SB_ERR_CUDA);
  }
  s = upload_problem(pl, p, err);
  if (s != SB_OK) return fail(s);
  *out = pl;
  return SB_OK;
}

// Energy pass over state x into slot (R doubles). FP32 fields (exact for integer J), FP64 on
// request; rows: replicas in x (x has R rows unless given).
cudaError_t enqueue_energy(sb_plan *pl, const float *x, double *slot, cudaStream_t st, int t, bool fp64 = false,
                           int rows = -1) {
  if (pl->tc && !sbk::tc_split(pl->dtype) && pl->prm.variant == SB_DSB && t >= 0)
    return sbk::tc_energy(pl->tc, t, x, pl->dh, slot, pl->dstatus, st);
  // split couplings (bSB, real-valued dSB): the final pass on the tensor cores too (FP32 sums of the
  // hi and lo products: exact for integer couplings, and for real ones it ranks the replicas whose
  // best kTopK are recomputed in FP64 below); FP64 passes stay on the plain kernel
  if (pl->tc && sbk::tc_split(pl->dtype) && t >= 0 && !fp64 && (pl->split_exact || !pl->integral))
    return sbk::tc_energy_signs(pl->tc, x, pl->dh, slot, pl->dstatus, st);
  sbk::PlainEnergy a;
  const int R = rows > 0 ? rows : pl->R;
  a.n = pl->n;
  a.R = R;
  a.jp = pl->jp;
  a.xp = pl->xp;
  a.rb = R < 8 ? R : 8;
  a.J = pl->dJ;
  a.h = pl->dh;
  a.x = x;
  a.energy = slot;
  a.status = pl->dstatus;
  return sbk::launch_plain_energy(a, fp64, st);
}

// Everything between the initial state and the final energy. Plain path: steps x (step kernel
// [+ trace energy pass]), captured into a graph. Tensor-core path: one persistent launch.
// With `evs`, an event pair brackets each step-kernel launch (profiling).
cudaError_t enqueue_loop(sb_plan *pl, cudaStream_t st, std::vector<cudaEvent_t> *evs,
                         int64_t *launches) {
  const sb_params &p = pl->prm;
  const bool tr = needs_trace(p);
  const int R = pl->R;
  int64_t nl = 0;
  if (pl->mode == SB_FIELD_TC) {
    if (p.steps > 0) {
      sbk::tc_set_waits(pl->tc, (long long)pl->ctx->wait_cycles, pl->ctx->debug_skip_step);
      pl->ctx->debug_skip_step = -1;
      if (evs) cudaEventRecord((*evs)[0], st);
      cudaError_t e = sbk::tc_run(pl->tc, p.steps, pl->dpump, pl->dx[0], pl->dy, pl->dh, pl->c0, p.dt,
                                  pl->dta0, tr ? pl->denergy : nullptr, pl->dstatus, st);
      if (e != cudaSuccess) return e;
      if (evs) cudaEventRecord((*evs)[1], st);
      nl = 1;
    }
    if (launches) *launches = nl;
    return cudaSuccess;
  }
  if (pl->dwords) {
    // plain FP32 SB in one cooperative launch (same fields and updates as the per-step kernel)
    if (p.steps > 0) {
      cudaError_t e = cudaMemsetAsync(pl->dwords, 0, pl->words_bytes, st);
      if (e != cudaSuccess) return e;
      sbk::PlainPersist a;
      memset(&a, 0, sizeof(a));
      a.variant = p.variant;
      a.n = pl->n;
      a.R = R;
      a.jp = pl->jp;
      a.xp = pl->xp;
      a.J = pl->dJ;
      a.h = pl->dh;
      a.x_in = pl->dx[0];
      a.x_out = pl->dx[p.steps & 1];
      a.y = pl->dy;
      a.pumps = pl->dpump;
      a.c0 = pl->c0;
      a.dt = p.dt;
      a.dta0 = pl->dta0;
      a.coeff = pl->coeff;
      a.mts_dt = p.mts_dt;
      a.detune = p.detune;
      a.kerr = p.kerr;
      a.m = p.mts_m;
      a.steps = p.steps;
      a.words = pl->dwords;
      a.status = pl->dstatus;
      if (evs) cudaEventRecord((*evs)[0], st);
      if ((e = sbk::launch_plain_persist(a, st)) != cudaSuccess) return e;
      if (evs) cudaEventRecord((*evs)[1], st);
      nl = 1;
    }
    if (launches) *launches = nl;
    return cudaSuccess;
  }
  for (int t = 0; t < p.steps; ++t) {
    cudaError_t e;
    // aSB: the pass before step t records the state after reference step t (slot t + 1); the
    // final pass records slot `steps`, so the last step needs none here.
    if (tr && p.variant != SB_DSB && !(p.variant == SB_ASB && t + 1 == p.steps)) {
      const int slot = p.variant == SB_ASB ? t + 1 : t;
      e = enqueue_energy(pl, pl->dx[t & 1], pl->denergy + (size_t)slot * R, st, -1);
      if (e != cudaSuccess) return e;
      ++nl;
    }
    double *eslot = (tr && p.variant == SB_DSB) ? pl->denergy + (size_t)t * R : nullptr;
    if (evs) cudaEventRecord((*evs)[2 * t], st);
    sbk::PlainStep a;
    memset(&a, 0, sizeof(a));
    a.variant = p.variant;
    a.n = pl->n;
    a.R = R;
    a.jp = pl->jp;
    a.xp = pl->xp;
    a.rb = R < 8 ? R : 8;
    a.J = pl->dJ;
    a.h = pl->dh;
    a.x_in = pl->dx[t & 1];
    a.x_out = pl->dx[(t + 1) & 1];
    a.y = pl->dy;
    a.pump = sb_pump(p.a0, t, p.steps);
    a.c0 = pl->c0;
    a.dt = p.dt;
    a.dta0 = pl->dta0;
    a.coeff = pl->coeff;
    a.amp_next = (float)(t + 1) / (float)p.steps;
    a.mts_dt = p.mts_dt;
    a.detune = p.detune;
    a.kerr = p.kerr;
    a.m = p.mts_m;
    a.do_local = (t + 1 < p.steps) ? 1 : 0;
    a.energy = eslot;
    a.status = pl->dstatus;
    // consecutive steps overlap (J is never written inside the loop); profiled runs time each
    // launch alone between its events
    a.overlap = evs ? 0 : 1;
    e = sbk::launch_plain_step(a, st);
    if (e != cudaSuccess) return e;
    if (evs) cudaEventRecord((*evs)[2 * t + 1], st);
    ++nl;
  }
  if (launches) *launches = nl;
  return cudaSuccess;
}

const float *final_x(const sb_plan *pl) {
  if (pl->mode == SB_FIELD_TC) return pl->dx[0];
  return pl->dx[pl->prm.steps & 1];
}

sb_status plan_run(sb_plan *pl, uint64_t seed, sb_result *res, std::string &err) {
  sb_ctx *ctx = pl->ctx;
  cudaStream_t st = ctx->stream;
  const sb_params &p = pl->prm;
  const int n = pl->n, R = pl->R;
  const bool tr = needs_trace(p);
  const auto t_start = std::chrono::steady_clock::now();
  int64_t launches = 0;
  SB_CUDA(cudaMemsetAsync(pl->dstatus, 0, sizeof(uint32_t), st));
  SB_CUDA(cudaMemsetAsync(pl->denergy, 0, energy_slots(p) * (size_t)R * sizeof(double), st));
  SB_CUDA(cudaEventRecord(pl->ev0, st));
  if (p.init_mode == SB_INIT_REFERENCE)
    SB_CUDA(sbk::launch_init_reference(pl->dx[0], pl->dy, n, R, pl->xp, st));
  else
    SB_CUDA(sbk::launch_init_uniform(pl->dx[0], pl->dy, n, R, pl->xp, seed, st));
  ++launches;
  if (p.variant == SB_ASB) {
    if (tr) {
      SB_CUDA(enqueue_energy(pl, pl->dx[0], pl->denergy, st, -1));
      ++launches;
    }
    if (p.steps > 0) {
      SB_CUDA(sbk::launch_asb_local(pl->dx[0], pl->dy, n, R, pl->xp, 0.0f, p.mts_m, p.mts_dt,
                                    p.detune, p.kerr, st));
      ++launches;
    }
  }
  if (pl->tc) {
    SB_CUDA(sbk::tc_prepare(pl->tc, pl->dx[0], st));
    ++launches;
  }
  double kernel_ms = 0.0;
  if (p.profile) {
    const int nmeas = (pl->mode == SB_FIELD_TC || pl->dwords) ? (p.steps > 0 ? 1 : 0) : p.steps;
    std::vector<cudaEvent_t> evs((size_t)2 * (nmeas > 0 ? nmeas : 1));
    for (auto &ev : evs) SB_CUDA(cudaEventCreate(&ev));
    int64_t nl = 0;
    cudaError_t e = enqueue_loop(pl, st, &evs, &nl);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (int t = 0; t < nmeas && e == cudaSuccess; ++t) {
      float ms = 0.0f;
      e = cudaEventElapsedTime(&ms, evs[2 * t], evs[2 * t + 1]);
      kernel_ms += ms;
    }
    for (auto &ev : evs) cudaEventDestroy(ev);
    if (e != cudaSuccess) {
      err = std::string("profiled step loop: ") + cudaGetErrorString(e);
      return SB_ERR_CUDA;
    }
    if (nmeas > 0) kernel_ms /= nmeas;
    launches += nl;
  } else if (p.steps > 0 && (pl->mode == SB_FIELD_TC || pl->dwords)) {
    int64_t nl = 0;
    SB_CUDA(enqueue_loop(pl, st, nullptr, &nl));
    launches += nl;
  } else if (p.steps > 0) {
    if (!pl->graph) {
      cudaGraph_t g = nullptr;
      SB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      int64_t nl = 0;
      cudaError_t e = enqueue_loop(pl, st, nullptr, &nl);
      cudaError_t e2 = cudaStreamEndCapture(st, &g);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        err = std::string("capturing the step loop: ") +
              cudaGetErrorString(e != cudaSuccess ? e : e2);
        return SB_ERR_CUDA;
      }
      e = cudaGraphInstantiate(&pl->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        pl->graph = nullptr;
        err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e);
        return SB_ERR_CUDA;
      }
      pl->launches_in_loop = nl;
    }
    SB_CUDA(cudaGraphLaunch(pl->graph, st));
    launches += pl->launches_in_loop;
  }
  double *final_slot = pl->denergy + (tr ? (size_t)p.steps * R : 0);
  // Integer couplings: the FP32 field is exact. Real couplings: FP32 energies rank the replicas
  // and the best kTopK are recomputed in FP64 (FP64 on every replica would cost more than the
  // solve on this part).
  const bool refine = !pl->integral;
  SB_CUDA(enqueue_energy(pl, final_x(pl), final_slot, st, p.steps, refine && R <= kTopK));
  ++launches;
  std::vector<double> e_final((size_t)R);
  uint32_t status = 0;
  SB_CUDA(cudaMemcpyAsync(e_final.data(), final_slot, (size_t)R * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  SB_CUDA(cudaMemcpyAsync(&status, pl->dstatus, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SB_CUDA(cudaStreamSynchronize(st));
  bool refined = false;
  int order_best = 0;
  if (refine && R > kTopK && status == 0) {
    std::vector<int> order((size_t)R);
    for (int r = 0; r < R; ++r) order[r] = r;
    std::partial_sort(order.begin(), order.begin() + kTopK, order.end(),
                      [&](int a, int b) { return e_final[a] < e_final[b]; });
    if (!pl->dxk) {
      SB_CUDA(cudaMalloc(&pl->dxk, (size_t)kTopK * pl->xp * sizeof(float)));
      SB_CUDA(cudaMalloc(&pl->dek, (size_t)kTopK * sizeof(double)));
    }
    for (int q = 0; q < kTopK; ++q)
      SB_CUDA(cudaMemcpyAsync(pl->dxk + (size_t)q * pl->xp, final_x(pl) + (size_t)order[q] * pl->xp,
                              (size_t)pl->xp * sizeof(float), cudaMemcpyDeviceToDevice, st));
    SB_CUDA(cudaMemsetAsync(pl->dek, 0, (size_t)kTopK * sizeof(double), st));
    SB_CUDA(enqueue_energy(pl, pl->dxk, pl->dek, st, -1, true, kTopK));
    ++launches;
    double ek[kTopK];
    SB_CUDA(cudaMemcpyAsync(ek, pl->dek, sizeof(ek), cudaMemcpyDeviceToHost, st));
    SB_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < kTopK; ++q) e_final[order[q]] = ek[q];
    refined = true;
    order_best = order[0];
    for (int q = 1; q < kTopK; ++q)
      if (e_final[order[q]] < e_final[order_best]) order_best = order[q];
  }
  SB_CUDA(cudaEventRecord(pl->ev1, st));
  if (status != 0) {
    err = sbh::device_status_text(status);
    return (status & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
  }
  // after a refinement the best replica is chosen among the FP64-refined candidates: a replica in
  // the same state as one of them but outside the top kTopK keeps its FP32 energy, which may sit a
  // rounding below the exact one
  int best = refined ? order_best : 0;
  if (!refined)
    for (int r = 1; r < R; ++r)
      if (e_final[r] < e_final[best]) best = r;
  SB_CUDA(cudaEventSynchronize(pl->ev1));
  std::vector<float> xb((size_t)n);
  SB_CUDA(cudaMemcpyAsync(xb.data(), final_x(pl) + (size_t)best * pl->xp, (size_t)n * sizeof(float),
                          cudaMemcpyDeviceToHost, st));
  if (res->final_x)
    SB_CUDA(cudaMemcpy2DAsync(res->final_x, (size_t)n * sizeof(float), final_x(pl),
                              (size_t)pl->xp * sizeof(float), (size_t)n * sizeof(float), (size_t)R,
                              cudaMemcpyDeviceToHost, st));
  if (res->final_y)
    SB_CUDA(cudaMemcpy2DAsync(res->final_y, (size_t)n * sizeof(float), pl->dy,
                              (size_t)pl->xp * sizeof(float), (size_t)n * sizeof(float), (size_t)R,
                              cudaMemcpyDeviceToHost, st));
  std::vector<double> tr_all;
  if (tr && (res->energy_trace || res->energy_trace_all)) {
    tr_all.resize(energy_slots(p) * (size_t)R);
    SB_CUDA(cudaMemcpyAsync(tr_all.data(), pl->denergy, tr_all.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  }
  SB_CUDA(cudaStreamSynchronize(st));
  float dev_ms = 0.0f;
  SB_CUDA(cudaEventElapsedTime(&dev_ms, pl->ev0, pl->ev1));
  std::vector<int8_t> spins((size_t)n);
  for (int i = 0; i < n; ++i) spins[i] = xb[i] > 0.0f ? 1 : -1;
  if (res->best_spins) memcpy(res->best_spins, spins.data(), (size_t)n);
  if (res->replica_energies) memcpy(res->replica_energies, e_final.data(), (size_t)R * sizeof(double));
  if (!tr_all.empty()) {
    if (res->energy_trace_all) memcpy(res->energy_trace_all, tr_all.data(), tr_all.size() * sizeof(double));
    if (res->energy_trace)
      for (int t = 0; t <= p.steps; ++t) {
        double m = tr_all[(size_t)t * R];
        for (int r = 1; r < R; ++r) m = fmin(m, tr_all[(size_t)t * R + r]);
        res->energy_trace[t] = m;
      }
  }
  res->best_replica = best;
  res->best_energy = e_final[best];
  res->field_mode_used = pl->mode;
  res->field_dtype_used = pl->dtype;
  res->energy_check_ok = 0;
  res->best_energy_i64 = 0;
  if (pl->prob) {
    if (pl->integral) {
      int64_t ei = 0;
      const sb_status es = pl->copies ? pl->copies->energy(0, spins.data(), &ei, 0)
                                      : sb_energy_i64(pl->prob, spins.data(), &ei);
      if (es == SB_OK) {
        res->best_energy_i64 = ei;
        res->energy_check_ok = ((double)ei == e_final[best]) ? 1 : 0;
      }
    } else {
      const double ef = sb_energy_f64(pl->prob, spins.data());
      res->energy_check_ok = fabs(ef - e_final[best]) <= 1e-9 * (1.0 + fabs(ef)) ? 1 : 0;
    }
  }
  res->device_ms = dev_ms;
  res->kernel_ms_avg = kernel_ms;
  res->steps_per_launch = (pl->mode == SB_FIELD_TC || pl->dwords) ? p.steps : 1;
  res->kernel_launches = launches;
  res->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  res->spin_updates_per_s =
      dev_ms > 0 ? (double)n * (double)R * (double)p.steps / ((double)dev_ms * 1e-3) : 0.0;
  return SB_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
extern "C" {

sb_status sb_create(sb_ctx **out, const sb_device_opts *opts) {
  if (!out) return SB_ERR_INVALID_ARG;
  *out = nullptr;
  int dev = opts ? opts->device : 0;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    sbh::set_thread_error("no CUDA device");
    return SB_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= count) {
    sbh::set_thread_error("device ordinal out of range");
    return SB_ERR_INVALID_ARG;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return SB_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) {
    sbh::set_thread_error(std::string("kernels are built for sm_103a; device is ") + prop.name);
    return SB_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(dev) != cudaSuccess) return SB_ERR_CUDA;
  sbk::init_kernel_attributes();
  sb_ctx *c = new sb_ctx();
  c->device = dev;
  if (opts && opts->stream) {
    c->stream = (cudaStream_t)opts->stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return SB_ERR_CUDA;
    }
    c->own_stream = true;
  }
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->hbm_budget = (opts && opts->hbm_budget_bytes > 0) ? opts->hbm_budget_bytes : (int64_t)(0.8 * (double)fr);
  c->max_inflight = (opts && opts->max_inflight > 0) ? opts->max_inflight : 64;
  *out = c;
  return SB_OK;
}

sb_status sb_destroy(sb_ctx *ctx) {
  if (!ctx) return SB_ERR_INVALID_ARG;
  if (ctx->server) {
    sbs::server_destroy(ctx->server);
    ctx->server = nullptr;
  }
  cudaSetDevice(ctx->device);
  if (ctx->cached) {
    plan_free_device(ctx->cached);
    delete ctx->cached;
  }
  sbh::nmfa_cache_free(ctx->nmfa);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SB_OK;
}

sb_status sb_set_wait_limit(sb_ctx *ctx, int64_t cycles) {
  if (!ctx || cycles < 0) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->wait_cycles = cycles;
  return SB_OK;
}

sb_status sb_debug_skip_publish(sb_ctx *ctx, int32_t step) {
  if (!ctx || step < 0) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->debug_skip_step = step;
  return SB_OK;
}

const char *sb_last_error(sb_ctx *ctx) {
  if (!ctx) return sbh::thread_error();
  return ctx->last_error.c_str();
}

sb_status sb_plan_create(sb_ctx *ctx, const sb_problem *p, const sb_params *params, sb_plan **out) {
  if (!ctx || !out) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  std::string err;
  sb_status s = plan_create(ctx, p, params, out, err);
  ctx->last_error = err;
  return s;
}

sb_status sb_plan_run(sb_plan *plan, uint64_t seed, sb_result *res) {
  if (!plan || !res) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(plan->ctx->mu);
  cudaSetDevice(plan->ctx->device);
  std::string err;
  sb_status s = plan_run(plan, seed, res, err);
  plan->ctx->last_error = err;
  return s;
}

sb_status sb_plan_destroy(sb_plan *plan) {
  if (!plan) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(plan->ctx->mu);
  cudaSetDevice(plan->ctx->device);
  plan_free_device(plan);
  delete plan;
  return SB_OK;
}

int64_t sb_plan_footprint(const sb_problem *p, const sb_params *prm) {
  if (!p || !prm || p->n <= 0 || prm->replicas <= 0) return -1;
  std::string err;
  int mode, dtype;
  if (resolve_mode(p, prm, mode, dtype, err) != SB_OK) return -1;
  const int64_t jp = sbk::pitch_for(p->n, 4);
  int64_t b = (int64_t)p->n * jp * 4 + (p->h ? (int64_t)p->n * 4 : 0);
  const int64_t xs = (int64_t)prm->replicas * jp * 4;
  b += xs * (mode == SB_FIELD_FP32 ? 3 : 2);
  b += (int64_t)energy_slots(*prm) * prm->replicas * 8 + 4;
  if (mode == SB_FIELD_TC) {
    sbk::TcSetup s{prm->variant, dtype, p->n, prm->replicas, (int)jp};
    b += sbk::tc_footprint(s);
  }
  return b;
}

sb_status sb_solve(sb_ctx *ctx, const sb_problem *p, const sb_params *params, sb_result *res) {
  if (!ctx || !res) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  std::string err;
  const auto t0 = std::chrono::steady_clock::now();
  sb_status s = check_params(p, params, err);
  int mode = 0, dtype = 0;
  if (s == SB_OK) s = resolve_mode(p, params, mode, dtype, err);
  if (s != SB_OK) {
    ctx->last_error = err;
    return s;
  }
  const float c0 = params->c0 > 0.0f ? params->c0 : sb_default_c0(p);
  const float xi = params->xi > 0.0f ? params->xi : (float)(0.7 * (double)params->detune / sqrt((double)p->n));
  const PlanKey key = make_key(p, params, mode, dtype, c0, (float)((double)params->coupling_dt * (double)xi));
  sb_plan *pl = ctx->cached;
  if (pl && pl->key == key) {
    s = upload_problem(pl, p, err);
  } else {
    if (pl) {
      plan_free_device(pl);
      delete pl;
      ctx->cached = nullptr;
    }
    s = plan_create(ctx, p, params, &pl, err);
    if (s == SB_OK) ctx->cached = pl;
  }
  if (s == SB_OK) {
    pl->prm.profile = params->profile;
    s = plan_run(pl, params->seed, res, err);
  }
  // the cached plan outlives this call, the caller's problem need not
  if (pl && ctx->cached == pl) pl->copies.reset();
  if (s == SB_OK)
    res->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  ctx->last_error = err;
  return s;
}

// ---- serving entry points: forwarded to the server (sb_serve.cpp) ----

sb_status sb_submit(sb_ctx *ctx, const sb_problem *p, const sb_params *params, uint64_t *ticket) {
  if (!ctx || !p || !params || !ticket) return SB_ERR_INVALID_ARG;
  std::string err;
  sb_status s = check_params(p, params, err);
  if (s != SB_OK) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error = err;
    return s;
  }
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->server) {
      sb_status cs = sbs::server_create(&ctx->server, ctx->device, ctx->hbm_budget, ctx->max_inflight, err);
      if (cs != SB_OK) {
        ctx->last_error = err;
        return cs;
      }
    }
  }
  return sbs::server_submit(ctx->server, p, params, ticket);
}

sb_status sb_poll(sb_ctx *ctx, uint64_t ticket, sb_result *res, int32_t wait_ms) {
  if (!ctx || !res) return SB_ERR_INVALID_ARG;
  if (!ctx->server) return SB_ERR_NOT_FOUND;
  std::string err;
  const sb_status s = sbs::server_poll(ctx->server, ticket, res, wait_ms, err);
  if (s != SB_OK && s != SB_ERR_PENDING) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->last_error = err;
  }
  return s;
}

sb_status sb_cancel(sb_ctx *ctx, uint64_t ticket) {
  if (!ctx) return SB_ERR_INVALID_ARG;
  if (!ctx->server) return SB_ERR_NOT_FOUND;
  return sbs::server_cancel(ctx->server, ticket);
}

sb_status sb_serving_stats_get(sb_ctx *ctx, sb_serving_stats *out) {
  if (!ctx || !out) return SB_ERR_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  if (!ctx->server) return SB_OK;
  return sbs::server_stats(ctx->server, out);
}

}  // extern "C"
