// NMFA (noisy mean-field annealing) on the GPU: the host side of sb_nmfa_solve / sb_gpu_nmfa.
//
// Replaces gpu_nmfa (NMFA/CUDA_GPU/src/nmfa.cu:142-199: copy J and the betas, one launch of
// gpu_nmfa_kernel with one CTA per sample, copy the samples back, return the kernel's event time).
// Here the samples are replicas. J is padded to [n][jp] once and every (sample, spin) gets its
// XORWOW words from one seeding launch; then either
//   * FP32 (the plain fused kernel's layout, sb_plain.cu): each of a stage's two sweeps is one fused
//     launch (field + noise + tanh update), issued back to back so that consecutive launches overlap
//     (programmatic dependent launch); the last sweep writes the +-1 samples and one energy pass
//     gives every sample's energy; or
//   * tensor cores (sb_tc_kernel.cuh, variant 3): all sweeps in one persistent tcgen05 launch, the
//     states as BF16 hi + lo against exact BF16 couplings, then one launch writes the samples and
//     the dSB energy contraction on the same couplings gives the energies.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
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

// norm_i = -1 / sqrt(sum_j |J_ij|) (nmfa.cu:88-93), the sum in double over j in index order (exact
// for integer couplings); 0 for a row without couplings, whose field is then 0.
void row_norms(const sb_problem *p, std::vector<float> &norm) {
  const int n = p->n;
  norm.assign((size_t)n, 0.0f);
  for (int i = 0; i < n; ++i) {
    double a = 0.0;
    const float *row = p->J + (size_t)i * n;
    for (int j = 0; j < n; ++j) a += fabs((double)row[j]);
    norm[i] = a > 0.0 ? (float)(-1.0 / sqrt(a)) : 0.0f;
  }
}

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
  std::vector<float> norm;
  row_norms(prob, norm);
  cudaSetDevice(ctx->device);
  const int jp = (n + 3) & ~3, xp = jp;
  const int rb = R < 8 ? R : 8;
  const size_t plane = (size_t)R * xp;
  const bool exact = prob->integer_valued && (double)prob->max_abs_j * n < 16777216.0;
  const bool tc_ok = exact && prob->max_abs_j <= 256;
  if (prm->field_mode == SB_FIELD_TC && !tc_ok)
    return fail(ctx, SB_ERR_UNSUPPORTED, std::string(who) + ": the tensor-core field needs integer couplings "
                                                            "with |J| <= 256");
  bool use_tc = prm->field_mode == SB_FIELD_TC || (prm->field_mode == SB_FIELD_AUTO && tc_ok && R >= 32);
  sbk::TcEngine *te = nullptr;
  std::vector<float> sweep_betas((size_t)2 * stages);
  for (int t = 0; t < 2 * stages; ++t) sweep_betas[t] = betas[t / 2];
  float *dbetas = nullptr;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  float *dJ = nullptr, *dnorm = nullptr, *ds = nullptr, *dz1 = nullptr;
  uint32_t *drng = nullptr, *dstatus = nullptr;
  int32_t *dsamp = nullptr;
  double *den = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t hstatus = 0;
  float dev_ms = 0.0f;
  std::vector<int32_t> hsamp((size_t)R * n);
  std::vector<double> hen((size_t)R);
  std::string where;
  sb_status out = SB_OK;
  int64_t launches = 0;
#define NM_CUDA(call)                \
  if ((e = (call)) != cudaSuccess) { \
    where = #call;                   \
    goto cleanup;                    \
  }
  sbk::init_kernel_attributes();
  NM_CUDA(cudaEventCreate(&ev0));
  NM_CUDA(cudaEventCreate(&ev1));
  NM_CUDA(cudaMallocAsync((void **)&dJ, (size_t)n * jp * sizeof(float), st));
  NM_CUDA(cudaMallocAsync((void **)&dnorm, (size_t)n * sizeof(float), st));
  NM_CUDA(cudaMallocAsync((void **)&ds, 2 * plane * sizeof(float), st));
  NM_CUDA(cudaMallocAsync((void **)&dz1, plane * sizeof(float), st));
  NM_CUDA(cudaMallocAsync((void **)&drng, 5 * plane * sizeof(uint32_t), st));
  NM_CUDA(cudaMallocAsync((void **)&dsamp, (size_t)R * n * sizeof(int32_t), st));
  NM_CUDA(cudaMallocAsync((void **)&den, (size_t)R * sizeof(double), st));
  NM_CUDA(cudaMallocAsync((void **)&dstatus, sizeof(uint32_t), st));
  if (jp != n) NM_CUDA(cudaMemsetAsync(dJ, 0, (size_t)n * jp * sizeof(float), st));
  NM_CUDA(cudaMemcpy2DAsync(dJ, (size_t)jp * sizeof(float), prob->J, (size_t)n * sizeof(float),
                            (size_t)n * sizeof(float), (size_t)n, cudaMemcpyHostToDevice, st));
  NM_CUDA(cudaMemcpyAsync(dnorm, norm.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
  NM_CUDA(cudaMemsetAsync(ds, 0, 2 * plane * sizeof(float), st));
  NM_CUDA(cudaMemsetAsync(den, 0, (size_t)R * sizeof(double), st));
  NM_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(uint32_t), st));
  if (use_tc) {
    std::string terr;
    sbk::TcSetup ts;
    ts.variant = 3;
    ts.dtype = sbk::kTcBf16;
    ts.n = n;
    ts.R = R;
    ts.xp = xp;
    const sb_status tst = sbk::tc_create(&te, ts, dJ, jp, terr, st);
    if (tst != SB_OK) {
      if (prm->field_mode == SB_FIELD_TC) {
        out = tst;
        ctx->last_error = std::string(who) + ": " + terr;
        goto cleanup_noerr;
      }
      use_tc = false;  // auto: the FP32 path runs every shape
    } else {
      NM_CUDA(cudaMallocAsync((void **)&dbetas, sweep_betas.size() * sizeof(float), st));
      NM_CUDA(cudaMemcpyAsync(dbetas, sweep_betas.data(), sweep_betas.size() * sizeof(float), cudaMemcpyHostToDevice,
                              st));
    }
  }
  NM_CUDA(cudaEventRecord(ev0, st));
  NM_CUDA(sbk::launch_nmfa_seed(drng, n, R, xp, prm->seed, st));
  ++launches;
  if (use_tc) {
    NM_CUDA(sbk::tc_prepare(te, ds, st));
    NM_CUDA(sbk::tc_run_nmfa(te, 2 * stages, dbetas, ds, dz1, dnorm, drng, prm->noise,
                             (float)(1.0 - (double)prm->recombination), prm->recombination, dstatus, st));
    NM_CUDA(sbk::launch_nmfa_signs(ds, n, R, xp, dsamp, st));
    NM_CUDA(sbk::tc_nmfa_energy(te, ds, den, dstatus, st));
    launches += 5;
  } else {
    sbk::NmfaSweep a;
    memset(&a, 0, sizeof(a));
    a.n = n;
    a.R = R;
    a.jp = jp;
    a.xp = xp;
    a.rb = rb;
    a.J = dJ;
    a.norm = dnorm;
    a.rng = drng;
    a.z1 = dz1;
    a.noise = prm->noise;
    a.keep = (float)(1.0 - (double)prm->recombination);  // nmfa.cu:95, 1.0 - recombination
    a.mix = prm->recombination;
    a.status = dstatus;
    a.overlap = 1;
    int cur = 0;
    for (int t = 0; t < stages; ++t)
      for (int k = 0; k < 2; ++k) {
        a.s_in = ds + (size_t)cur * plane;
        a.s_out = ds + (size_t)(cur ^ 1) * plane;
        a.beta = betas[t];
        a.first = k == 0 ? 1 : 0;
        a.samples = (t + 1 == stages && k == 1) ? dsamp : nullptr;
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
    pe.J = dJ;
    pe.h = nullptr;
    pe.x = ds;
    pe.energy = den;
    pe.status = dstatus;
    NM_CUDA(sbk::launch_plain_energy(pe, !exact, st));
    ++launches;
  }
  NM_CUDA(cudaEventRecord(ev1, st));
  NM_CUDA(cudaMemcpyAsync(hsamp.data(), dsamp, hsamp.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaMemcpyAsync(hen.data(), den, hen.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (res && res->states)
    NM_CUDA(cudaMemcpy2DAsync(res->states, (size_t)n * sizeof(float), ds, (size_t)xp * sizeof(float),
                              (size_t)n * sizeof(float), (size_t)R, cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaMemcpyAsync(&hstatus, dstatus, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  NM_CUDA(cudaStreamSynchronize(st));
  if (hstatus) {
    out = (hstatus & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
    ctx->last_error = std::string(who) + ": device status " + std::to_string(hstatus);
    goto cleanup_noerr;
  }
  NM_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
  if (samples32) memcpy(samples32, hsamp.data(), hsamp.size() * sizeof(int32_t));
  if (res) {
    // the energy pass gives H = -1/2 s J s (fields are 0): NMFA's E is -H
    int best = 0;
    for (int r = 0; r < R; ++r) {
      hen[r] = -hen[r];
      if (hen[r] < hen[best]) best = r;
    }
    std::vector<int8_t> sp((size_t)n);
    for (int i = 0; i < n; ++i) sp[i] = (int8_t)hsamp[(size_t)best * n + i];
    if (res->samples)
      for (size_t k = 0; k < hsamp.size(); ++k) res->samples[k] = (int8_t)hsamp[k];
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
    res->field_used = use_tc ? SB_FIELD_TC : SB_FIELD_FP32;
    const double updates = (double)n * R * 2.0 * stages;
    res->spin_updates_per_s = dev_ms > 0 ? updates / ((double)dev_ms * 1e-3) : 0.0;
  }
  goto cleanup_noerr;
cleanup:
  out = e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  ctx->last_error = std::string(who) + ": " + where + ": " + cudaGetErrorString(e);
cleanup_noerr:
  cudaFreeAsync(dJ, st);
  cudaFreeAsync(dnorm, st);
  cudaFreeAsync(ds, st);
  cudaFreeAsync(dz1, st);
  cudaFreeAsync(drng, st);
  cudaFreeAsync(dsamp, st);
  cudaFreeAsync(den, st);
  cudaFreeAsync(dstatus, st);
  if (dbetas) cudaFreeAsync(dbetas, st);
  cudaStreamSynchronize(st);
  sbk::tc_destroy(te);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
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
