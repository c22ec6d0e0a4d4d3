// NMFA (noisy mean-field annealing) on the GPU: the host side of sb_nmfa_solve / sb_gpu_nmfa.
//
// Replaces gpu_nmfa (NMFA/CUDA_GPU/src/nmfa.cu:142-199: copy J and the betas, one launch of
// gpu_nmfa_kernel with one CTA per sample, copy the samples back, return the kernel's event time).
// Here the samples are replicas. J is padded to [n][jp] once and every (sample, spin) gets its
// XORWOW words from one seeding launch; then either
//   * FP32 (the plain fused kernel's layout, sb_plain.cu): when the rows fit one co-resident grid
//     (few samples: the reference program's single sample), every sweep runs in one cooperative
//     launch of the plain solve's persistent kernel (J rows in registers, the states exchanged as
//     tagged words through L2, the same summation order and bits); otherwise each of a stage's two
//     sweeps is one fused launch (field + noise + tanh update), issued back to back so that
//     consecutive launches overlap (programmatic dependent launch); the last sweep writes the +-1
//     samples and one energy pass gives every sample's energy; or
//   * tensor cores (sb_tc_kernel.cuh, variant 3): all sweeps in one persistent tcgen05 launch, the
//     states as BF16 hi + lo against exact BF16 couplings, then one launch writes the samples and
//     the dSB energy contraction on the same couplings gives the energies.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "sb.h"
#include "sb_ctx.h"
#include "sb_host.h"
#include "sb_internal.h"

namespace {

sb_status fail(sb_ctx *ctx, sb_status s, const std::string &msg) {
  ctx->last_error = msg;
  return s;
}

}  // namespace

// Device buffers of the last NMFA shape a context ran (sb_nmfa_solve / sb_gpu_nmfa keep them between
// calls, as sb_solve keeps its plan): a call with the same n and sample count uploads J and runs.
struct NmfaCache {
  int n = 0, R = 0, jp = 0, xp = 0;
  sbk::TcEngine *te = nullptr;  // built on the first tensor-core call for this shape
  float *dJ = nullptr, *dnorm = nullptr, *ds = nullptr, *dz1 = nullptr, *dbetas = nullptr;
  size_t betas_cap = 0;
  uint32_t *drng = nullptr, *dstatus = nullptr;
  int32_t *dsamp = nullptr;
  double *den = nullptr;
  unsigned long long *dwords = nullptr;  // the one-launch FP32 solve's exchange lines
  size_t words_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace sbh {
void nmfa_cache_free(NmfaCache *c) {
  if (!c) return;
  sbk::tc_destroy(c->te);
  cudaFree(c->dJ);
  cudaFree(c->dnorm);
  cudaFree(c->ds);
  cudaFree(c->dz1);
  cudaFree(c->dbetas);
  cudaFree(c->drng);
  cudaFree(c->dstatus);
  cudaFree(c->dsamp);
  cudaFree(c->den);
  cudaFree(c->dwords);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  delete c;
}
}  // namespace sbh

namespace {

// Everything sb_nmfa_solve and sb_gpu_nmfa share; samples32 (when set) receives int32 +-1.
sb_status nmfa_run(sb_ctx *ctx, const sb_problem *prob, const sb_nmfa_params *prm, sb_nmfa_result *res,
                   int32_t *samples32, const char *who) {
  const auto t0 = std::chrono::steady_clock::now();
  const int n = prob->n, R = prm->samples, stages = prm->stages;
  if (n < 1 || R < 1 || stages < 1 || !(prm->noise >= 0.0f) || !(prm->recombination >= 0.0f) ||
      !(prm->recombination <= 1.0f))
    return fail(ctx, SB_ERR_INVALID_ARG, std::string(who) + ": needs n >= 1, samples >= 1, stages >= 1, "
                                                            "noise >= 0 and recombination in [0, 1]");
  if ((int64_t)n * R > ((int64_t)1 << 31) / 8)
    return fail(ctx, SB_ERR_UNSUPPORTED, std::string(who) + ": n x samples too large");
  if (prob->h)
    for (int i = 0; i < n; ++i)
      if (prob->h[i] != 0.0f)
        return fail(ctx, SB_ERR_UNSUPPORTED, std::string(who) + ": fields are not supported (the reference has none)");
  std::vector<float> betas((size_t)stages);
  if (prm->betas)
    memcpy(betas.data(), prm->betas, (size_t)stages * sizeof(float));
  else
    sb_nmfa_schedule(stages, betas.data());
  const bool exact = prob->integer_valued && (double)prob->max_abs_j * n < 16777216.0;
  const bool tc_ok = exact && prob->max_abs_j <= 256;
  if (prm->field_mode == SB_FIELD_TC && !tc_ok)
    return fail(ctx, SB_ERR_UNSUPPORTED, std::string(who) + ": the tensor-core field needs integer couplings "
                                                            "with |J| <= 256");
  bool use_tc = prm->field_mode == SB_FIELD_TC || (prm->field_mode == SB_FIELD_AUTO && tc_ok && R >= 32);
  int persist_ctas = 0;  // FP32 field: CTAs of the one-launch solve, 0 when it does not fit
  std::vector<float> sweep_betas((size_t)2 * stages);
  for (int t = 0; t < 2 * stages; ++t) sweep_betas[t] = betas[t / 2];
  cudaSetDevice(ctx->device);
  const int jp = (n + 3) & ~3, xp = jp;
  const int rb = R < 8 ? R : 8;
  const size_t plane = (size_t)R * xp;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  uint32_t hstatus = 0;
  float dev_ms = 0.0f;
  // the samples go straight into the caller's int32 buffer when there is one
  std::vector<int32_t> hsamp(samples32 ? 0 : (size_t)R * n);
  int32_t *samp = samples32 ? samples32 : hsamp.data();
  std::vector<double> hen((size_t)R);
  std::string where;
  sb_status out = SB_OK;
  int64_t launches = 0;
  NmfaCache *c = ctx->nmfa;
#define NM_CUDA(call)                \
  if ((e = (call)) != cudaSuccess) { \
    where = #call;                   \
    goto cleanup;                    \
  }
  sbk::init_kernel_attributes();
  if (c && (c->n != n || c->R != R)) {
    sbh::nmfa_cache_free(c);
    c = ctx->nmfa = nullptr;
  }
  if (!c) {
    c = ctx->nmfa = new NmfaCache();
    c->n = n;
    c->R = R;
    c->jp = jp;
    c->xp = xp;
    NM_CUDA(cudaEventCreate(&c->ev0));
    NM_CUDA(cudaEventCreate(&c->ev1));
    NM_CUDA(cudaMalloc((void **)&c->dJ, (size_t)n * jp * sizeof(float)));
    NM_CUDA(cudaMalloc((void **)&c->dnorm, (size_t)n * sizeof(float)));
    NM_CUDA(cudaMalloc((void **)&c->ds, 2 * plane * sizeof(float)));
    NM_CUDA(cudaMalloc((void **)&c->dz1, plane * sizeof(float)));
    NM_CUDA(cudaMalloc((void **)&c->drng, 5 * plane * sizeof(uint32_t)));
    NM_CUDA(cudaMalloc((void **)&c->dsamp, (size_t)R * n * sizeof(int32_t)));
    NM_CUDA(cudaMalloc((void **)&c->den, (size_t)R * sizeof(double)));
    NM_CUDA(cudaMalloc((void **)&c->dstatus, sizeof(uint32_t)));
    // the padding columns of J (and of the states) are never written afterwards
    if (jp != n) NM_CUDA(cudaMemsetAsync(c->dJ, 0, (size_t)n * jp * sizeof(float), st));
  }
  if (c->betas_cap < sweep_betas.size()) {
    cudaFree(c->dbetas);
    c->dbetas = nullptr;
    c->betas_cap = 0;
    NM_CUDA(cudaMalloc((void **)&c->dbetas, sweep_betas.size() * sizeof(float)));
    c->betas_cap = sweep_betas.size();
  }
  NM_CUDA(cudaMemcpy2DAsync(c->dJ, (size_t)jp * sizeof(float), prob->J, (size_t)n * sizeof(float),
                            (size_t)n * sizeof(float), (size_t)n, cudaMemcpyHostToDevice, st));
  // norm_i = -1 / sqrt(sum_j |J_ij|) (nmfa.cu:88-93), on the device from the uploaded couplings
  NM_CUDA(sbk::launch_nmfa_norms(c->dJ, n, jp, c->dnorm,
                                  prob->integer_valued && (double)prob->max_abs_j * n < 9.0e15, st));
  NM_CUDA(cudaMemcpyAsync(c->dbetas, sweep_betas.data(), sweep_betas.size() * sizeof(float), cudaMemcpyHostToDevice,
                          st));
  NM_CUDA(cudaMemsetAsync(c->ds, 0, 2 * plane * sizeof(float), st));
  NM_CUDA(cudaMemsetAsync(c->den, 0, (size_t)R * sizeof(double), st));
  NM_CUDA(cudaMemsetAsync(c->dstatus, 0, sizeof(uint32_t), st));
  if (use_tc) {
    if (c->te) {
      NM_CUDA(sbk::tc_reload(c->te, c->dJ, jp, st));
    } else {
      std::string terr;
      sbk::TcSetup ts;
      ts.variant = 3;
      ts.dtype = sbk::kTcBf16;
      ts.n = n;
      ts.R = R;
      ts.xp = xp;
      const sb_status tst = sbk::tc_create(&c->te, ts, c->dJ, jp, terr, st);
      if (tst != SB_OK) {
        c->te = nullptr;
        if (prm->field_mode == SB_FIELD_TC) {
          out = tst;
          ctx->last_error = std::string(who) + ": " + terr;
          goto cleanup_noerr;
        }
        use_tc = false;  // auto: the FP32 path runs every shape
      }
    }
  }
  if (!use_tc) {
    // SB_PLAIN_PERSIST=0 keeps one launch per sweep
    const char *env = getenv("SB_PLAIN_PERSIST");
    persist_ctas = (env && env[0] == '0') ? 0 : sbk::plain_persist_ctas(n, R, jp);
    const size_t need = (size_t)2 * persist_ctas * 128;  // one 128-byte line per CTA and parity
    if (persist_ctas > 0 && c->words_bytes < need) {
      cudaFree(c->dwords);
      c->dwords = nullptr;
      c->words_bytes = 0;
      NM_CUDA(cudaMalloc((void **)&c->dwords, need));
      c->words_bytes = need;
    }
  }
  NM_CUDA(cudaEventRecord(c->ev0, st));
  NM_CUDA(sbk::launch_nmfa_seed(c->drng, n, R, xp, prm->seed, st));
  ++launches;
  if (use_tc) {
    NM_CUDA(sbk::tc_prepare(c->te, c->ds, st));
    NM_CUDA(sbk::tc_run_nmfa(c->te, 2 * stages, c->dbetas, c->ds, c->dz1, c->dnorm, c->drng, prm->noise,
                             (float)(1.0 - (double)prm->recombination), prm->recombination, c->dstatus, st));
    NM_CUDA(sbk::launch_nmfa_signs(c->ds, n, R, xp, c->dsamp, st));
    NM_CUDA(sbk::tc_energy_signs(c->te, c->ds, nullptr, c->den, c->dstatus, st));
    launches += 5;
  } else if (persist_ctas > 0) {
    // every sweep in one cooperative launch: J rows in registers, states exchanged as tagged words
    // (the plain solve's one-launch kernel with the NMFA update; the same bits as one launch per
    // sweep)
    NM_CUDA(cudaMemsetAsync(c->dwords, 0, c->words_bytes, st));
    sbk::PlainPersist a;
    memset(&a, 0, sizeof(a));
    a.variant = 3;
    a.n = n;
    a.R = R;
    a.jp = jp;
    a.xp = xp;
    a.J = c->dJ;
    a.x_in = c->ds;
    a.x_out = c->ds;
    a.pumps = c->dbetas;
    a.steps = 2 * stages;
    a.words = c->dwords;
    a.status = c->dstatus;
    a.norm = c->dnorm;
    a.rng = c->drng;
    a.samples = c->dsamp;
    a.noise = prm->noise;
    a.keep = (float)(1.0 - (double)prm->recombination);  // nmfa.cu:95, 1.0 - recombination
    a.mix = prm->recombination;
    NM_CUDA(sbk::launch_plain_persist(a, st));
    ++launches;
    sbk::PlainEnergy pe;
    memset(&pe, 0, sizeof(pe));
    pe.n = n;
    pe.R = R;
    pe.jp = jp;
    pe.xp = xp;
    pe.rb = rb;
    pe.J = c->dJ;
    pe.h = nullptr;
    pe.x = c->ds;
    pe.energy = c->den;
    pe.status = c->dstatus;
    NM_CUDA(sbk::launch_plain_energy(pe, !exact, st));
    ++launches;
  } else {
    sbk::NmfaSweep a;
    memset(&a, 0, sizeof(a));
    a.n = n;
    a.R = R;
    a.jp = jp;
    a.xp = xp;
    a.rb = rb;
    a.J = c->dJ;
    a.norm = c->dnorm;
    a.rng = c->drng;
    a.z1 = c->dz1;
    a.noise = prm->noise;
    a.keep = (float)(1.0 - (double)prm->recombination);  // nmfa.cu:95, 1.0 - recombination
    a.mix = prm->recombination;
    a.status = c->dstatus;
    a.overlap = 1;
    int cur = 0;
    for (int t = 0; t < stages; ++t)
      for (int k = 0; k < 2; ++k) {
        a.s_in = c->ds + (size_t)cur * plane;
        a.s_out = c->ds + (size_t)(cur ^ 1) * plane;
        a.beta = betas[t];
        a.first = k == 0 ? 1 : 0;
        a.samples = (t + 1 == stages && k == 1) ? c->dsamp : nullptr;
        NM_CUDA(sbk::launch_nmfa_sweep(a, st));
        ++launches;
        cur ^= 1;
      }
    // an even number of sweeps: the final states are back in buffer 0
    sbk::PlainEnergy pe;
    memset(&pe, 0, sizeof(pe));
    pe.n = n;
    pe.R = R;
    pe.jp = jp;
    pe.xp = xp;
    pe.rb = rb;
    pe.J = c->dJ;
    pe.h = nullptr;
    pe.x = c->ds;
    pe.energy = c->den;
    pe.status = c->dstatus;
    NM_CUDA(sbk::launch_plain_energy(pe, !exact, st));
    ++launches;
  }
  NM_CUDA(cudaEventRecord(c->ev1, st));
  NM_CUDA(cudaMemcpyAsync(samp, c->dsamp, (size_t)R * n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaMemcpyAsync(hen.data(), c->den, hen.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (res && res->states)
    NM_CUDA(cudaMemcpy2DAsync(res->states, (size_t)n * sizeof(float), c->ds, (size_t)xp * sizeof(float),
                              (size_t)n * sizeof(float), (size_t)R, cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaMemcpyAsync(&hstatus, c->dstatus, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaStreamSynchronize(st));
  if (hstatus) {
    out = (hstatus & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
    ctx->last_error = std::string(who) + ": " + sbh::device_status_text(hstatus);
    sbh::nmfa_cache_free(c);
    ctx->nmfa = nullptr;
    goto cleanup_noerr;
  }
  NM_CUDA(cudaEventElapsedTime(&dev_ms, c->ev0, c->ev1));
  if (res) {
    // the energy pass gives H = -1/2 s J s (fields are 0): NMFA's E is -H
    int best = 0;
    for (int r = 0; r < R; ++r) {
      hen[r] = -hen[r];
      if (hen[r] < hen[best]) best = r;
    }
    std::vector<int8_t> sp((size_t)n);
    for (int i = 0; i < n; ++i) sp[i] = (int8_t)samp[(size_t)best * n + i];
    if (res->samples)
      for (size_t k = 0; k < (size_t)R * n; ++k) res->samples[k] = (int8_t)samp[k];
    if (res->energies) memcpy(res->energies, hen.data(), (size_t)R * sizeof(double));
    if (res->best_spins) memcpy(res->best_spins, sp.data(), (size_t)n);
    double check;
    int64_t ei = 0;
    if (prob->integer_valued && sbh::energy_i64(prob, sp.data(), &ei, 0) == SB_OK)
      check = -(double)ei;
    else
      check = -sb_energy_f64(prob, sp.data());
    res->energy_check_ok = exact ? (check == hen[best]) : (fabs(check - hen[best]) <= 1e-9 * (1.0 + fabs(check)));
    res->best_energy = check;
    res->best_sample = best;
    res->device_ms = dev_ms;
    res->kernel_launches = launches;
    res->field_mode_used = use_tc ? SB_FIELD_TC : SB_FIELD_FP32;
    const double updates = (double)n * R * 2.0 * stages;
    res->spin_updates_per_s = dev_ms > 0 ? updates / ((double)dev_ms * 1e-3) : 0.0;
  }
  goto cleanup_noerr;
cleanup:
  out = e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  ctx->last_error = std::string(who) + ": " + where + ": " + cudaGetErrorString(e);
  cudaStreamSynchronize(st);
  sbh::nmfa_cache_free(ctx->nmfa);  // a failed call leaves nothing behind
  ctx->nmfa = nullptr;
cleanup_noerr:
#undef NM_CUDA
  if (out == SB_OK && res)
    res->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return out;
}

}  // namespace

extern "C" sb_status sb_nmfa_params_default(sb_nmfa_params *p) {
  if (!p) return SB_ERR_INVALID_ARG;
  memset(p, 0, sizeof(*p));
  p->samples = 1;          // Ising.cpp:8
  p->stages = 100;         // Ising.cpp:10
  p->betas = nullptr;
  p->noise = 0.15f;        // Ising.cpp:12
  p->recombination = 0.15f;  // Ising.cpp:11
  p->seed = 1234u;         // Ising.cpp:13
  p->field_mode = SB_FIELD_AUTO;
  return SB_OK;
}

// Ising.cpp:37-43
extern "C" sb_status sb_nmfa_schedule(int32_t stages, float *betas) {
  if (stages < 1 || !betas) return SB_ERR_INVALID_ARG;
  const float increase = (8 - 1 / (float)16) / (float)stages;
  float beta = 1 / (float)16;
  for (int i = 0; i < stages; ++i) {
    betas[i] = beta;
    beta += increase;
  }
  return SB_OK;
}

extern "C" sb_status sb_nmfa_solve(sb_ctx *ctx, const sb_problem *p, const sb_nmfa_params *prm,
                                   sb_nmfa_result *res) {
  if (!ctx || !p || !prm || !res || !p->J) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return nmfa_run(ctx, p, prm, res, nullptr, "sb_nmfa_solve");
}

extern "C" sb_status sb_gpu_nmfa(sb_ctx *ctx, int32_t n, const float *J, const float *betas, int32_t num_betas,
                                 int32_t num_samples, int32_t *samples, float noise, float recombination,
                                 uint32_t seed, float *elapsed_ms) {
  if (!ctx || !J || !betas || !samples || n < 1 || num_betas < 1 || num_samples < 1) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  sb_problem p;
  sb_status s = sb_problem_wrap(&p, n, const_cast<float *>(J), nullptr);
  if (s != SB_OK) return fail(ctx, s, "sb_gpu_nmfa: bad couplings");
  sb_nmfa_params prm;
  sb_nmfa_params_default(&prm);
  prm.samples = num_samples;
  prm.stages = num_betas;
  prm.betas = betas;
  prm.noise = noise;
  prm.recombination = recombination;
  prm.seed = seed;
  sb_nmfa_result r;
  memset(&r, 0, sizeof(r));
  s = nmfa_run(ctx, &p, &prm, &r, samples, "sb_gpu_nmfa");
  if (s == SB_OK && elapsed_ms) *elapsed_ms = (float)r.device_ms;
  return s;
}
