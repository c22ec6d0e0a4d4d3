// sb_batch_*: many instances of uneven size solved together by the grouped tensor-core kernel.
//
// The reference solves one instance per program run and its trials one after another
// (SB/CUDA_GPU/m2_opt.cu:152); a batch here advances every instance and every replica of it in
// one grouped launch per SB step, the step loop replayed from a CUDA graph. Per instance the
// outputs are those of sb_solve (best spins, per-replica energies, host int64 re-check).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sb.h"
#include "sb_ctx.h"
#include "sb_grouped.h"
#include "sb_host.h"
#include "sb_internal.h"

struct sb_batch {
  sb_ctx *ctx = nullptr;
  std::vector<const sb_problem *> probs;
  sb_params prm{};
  sbk::Grouped *g = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // compact copies of the couplings for the host re-check, built in the background (the first
  // runs' device time hides them)
  std::unique_ptr<sbh::CouplingCopies> copies;
};

namespace {

std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune_cache;

sb_status init_all(sb_batch *b, uint64_t seed, std::string &err) {
  for (size_t k = 0; k < b->g->insts.size(); ++k) {
    sb_status s = b->g->init_state(b->g->insts[k], seed + k, err);
    if (s != SB_OK) return s;
  }
  return SB_OK;
}

// Times a few steps of each (replica tile, item order) candidate on the batch itself and keeps the
// fastest; the choice is cached by (replica count, total work bucket, batch size bucket).
sb_status autotune(sb_batch *b, std::string &err) {
  sbk::Grouped &g = *b->g;
  const std::string key = g.tune_key();
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      sb_status s = g.retile(it->second.first, err);
      g.set_order(it->second.second);
      return s;
    }
  }
  const auto cands = sbk::Grouped::candidates(b->prm.replicas);
  std::pair<int, int> best = cands.front();
  float best_ms = 1e30f;
  if (cands.size() > 1 && b->prm.steps >= 4) {
    cudaStream_t st = b->ctx->stream;
    for (const auto &c : cands) {
      sb_status s = g.retile(c.first, err);
      if (s != SB_OK) return s;
      g.set_order(c.second);
      if ((s = g.sync_tables(err)) != SB_OK) return s;
      if ((s = init_all(b, b->prm.seed, err)) != SB_OK) return s;
      if (g.run_steps(0, 1, false) != cudaSuccess) continue;
      cudaEventRecord(b->ev0, st);
      if (g.run_steps(1, 3, false) != cudaSuccess) continue;
      cudaEventRecord(b->ev1, st);
      if (cudaEventSynchronize(b->ev1) != cudaSuccess) continue;
      float ms = 0;
      cudaEventElapsedTime(&ms, b->ev0, b->ev1);
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
  }
  sb_status s = g.retile(best.first, err);
  g.set_order(best.second);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return s;
}

void destroy(sb_batch *b) {
  if (!b) return;
  delete b->g;
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  delete b;
}

sb_status create(sb_ctx *ctx, const sb_problem *problems, int32_t count, const sb_params *prm, sb_batch **out,
                 std::string &err) {
  if (!problems || count <= 0 || !prm || !out) {
    err = "need at least one problem";
    return SB_ERR_INVALID_ARG;
  }
  if (prm->steps < 0 || prm->replicas <= 0) {
    err = "steps >= 0 and replicas >= 1";
    return SB_ERR_INVALID_ARG;
  }
  for (int k = 0; k < count; ++k) {
    if (!problems[k].J || problems[k].n <= 0) {
      err = "problem " + std::to_string(k) + " is empty";
      return SB_ERR_INVALID_ARG;
    }
    if (!sbk::grouped_supports(&problems[k], prm)) {
      err = "problem " + std::to_string(k) +
            ": the grouped path runs dSB with integer couplings |J| <= 16 (exact FP8 operands)";
      return SB_ERR_UNSUPPORTED;
    }
  }
  // operands: packed E2M1 when every instance's couplings allow it (|J| <= 4), else FP8 E4M3
  bool fp4 = true;
  for (int k = 0; k < count; ++k) fp4 = fp4 && sbk::grouped_fp4_exact(&problems[k]);
  if (prm->operand_dtype == SB_OPERAND_FP8) {
    fp4 = false;
  } else if (prm->operand_dtype == SB_OPERAND_FP4) {
    if (!fp4) {
      err = "E2M1 operands need integer couplings |J| <= 4 in every problem of the batch";
      return SB_ERR_UNSUPPORTED;
    }
  } else if (prm->operand_dtype != SB_OPERAND_AUTO) {
    err = "the grouped path runs E2M1 or FP8 operands";
    return SB_ERR_UNSUPPORTED;
  }
  sb_batch *b = new sb_batch();
  b->ctx = ctx;
  b->prm = *prm;
  b->probs.resize(count);
  const int R = prm->replicas;
  b->g = new sbk::Grouped(ctx->stream, R <= 32 ? 32 : (R <= 64 ? 64 : 128), 0, fp4);
  if (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
    destroy(b);
    err = "cudaEventCreate";
    return SB_ERR_CUDA;
  }
  // Instances are prepared (packed on the host, uploaded, seeded) by several threads, each with its
  // own stream and pinned staging buffer, then made resident in order.
  std::vector<sbk::GHost> hosts(count);
  std::vector<sb_status> sts(count, SB_OK);
  const int nw = std::min(count, 8);
  std::vector<std::string> errs(nw);
  std::atomic<int> next{0};
  std::atomic<bool> failed{false};
  const int nr = b->g->nr;
  auto worker = [&](int w) {
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
      errs[w] = "cudaSetDevice";
      failed = true;
      return;
    }
    cudaStream_t ps = nullptr;
    if (cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking) != cudaSuccess) {
      errs[w] = "cudaStreamCreate";
      failed = true;
      return;
    }
    {
      sbk::Staging stg;
      for (int k; !failed.load() && (k = next.fetch_add(1)) < count;) {
        const sb_status st = sbk::Grouped::prepare(hosts[k], &problems[k], prm, prm->seed + k, k, nr, ps, stg, errs[w], fp4);
        if (st != SB_OK) {
          sts[k] = st;
          failed = true;
        }
      }
      cudaStreamSynchronize(ps);  // before the staging buffer is freed
    }
    cudaStreamDestroy(ps);
  };
  std::vector<std::thread> th;
  for (int w = 0; w < nw; ++w) th.emplace_back(worker, w);
  for (auto &t : th) t.join();
  if (failed.load()) {
    sb_status first = SB_ERR_CUDA;
    for (int k = 0; k < count; ++k)
      if (sts[k] != SB_OK) {
        first = sts[k];
        break;
      }
    for (int w = 0; w < nw; ++w)
      if (!errs[w].empty()) {
        err = errs[w];
        break;
      }
    for (auto &h : hosts) sbk::Grouped::release(h, ctx->stream);
    destroy(b);
    return first;
  }
  for (int k = 0; k < count; ++k) {
    b->probs[k] = &problems[k];
    b->g->attach(hosts[k], 0);
  }
  sb_status s = autotune(b, err);
  if (s == SB_OK) s = b->g->sync_tables(err);
  if (s != SB_OK) {
    destroy(b);
    return s;
  }
  b->copies.reset(new sbh::CouplingCopies(
      b->probs, (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2))));
  *out = b;
  return SB_OK;
}

sb_status run(sb_batch *b, uint64_t seed, sb_result *res, std::string &err) {
  sbk::Grouped &g = *b->g;
  cudaStream_t st = b->ctx->stream;
  const int steps = b->prm.steps;
  const auto t_start = std::chrono::steady_clock::now();
  sb_status s = g.sync_tables(err);
  if (s != SB_OK) return s;
  if (cudaMemsetAsync(g.d_status, 0, sizeof(uint32_t), st) != cudaSuccess) return SB_ERR_CUDA;
  const int64_t l0 = g.launches;
  cudaEventRecord(b->ev0, st);
  if ((s = init_all(b, seed, err)) != SB_OK) return s;
  cudaError_t e = cudaSuccess;
  double kernel_ms = 0.0;
  if (b->prm.profile && steps > 0) {
    std::vector<cudaEvent_t> evs(2 * (size_t)steps);
    for (auto &ev : evs) cudaEventCreate(&ev);
    for (int t = 0; t < steps && e == cudaSuccess; ++t) {
      cudaEventRecord(evs[2 * t], st);
      e = g.run_steps(t, 1, false);
      cudaEventRecord(evs[2 * t + 1], st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (int t = 0; t < steps && e == cudaSuccess; ++t) {
      float ms = 0;
      cudaEventElapsedTime(&ms, evs[2 * t], evs[2 * t + 1]);
      kernel_ms += ms;
    }
    for (auto &ev : evs) cudaEventDestroy(ev);
    kernel_ms /= steps;
  } else {
    e = g.run_steps(0, steps, true);
  }
  if (e == cudaSuccess) e = g.energy_pass(steps);
  cudaEventRecord(b->ev1, st);
  const size_t count = g.insts.size();
  std::vector<std::vector<double>> energies(count);
  uint32_t status = 0;
  for (size_t k = 0; k < count && e == cudaSuccess; ++k) {
    energies[k].resize(g.insts[k].R);
    e = cudaMemcpyAsync(energies[k].data(), g.insts[k].energy, (size_t)g.insts[k].R * sizeof(double),
                        cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, g.d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("batch run: ") + cudaGetErrorString(e);
    return SB_ERR_CUDA;
  }
  if (status) {
    err = sbh::device_status_text(status);
    return (status & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
  }
  float dev_ms = 0;
  cudaEventElapsedTime(&dev_ms, b->ev0, b->ev1);
  // best replica of each instance, its spins, optional full state
  std::vector<int> best(count, 0);
  std::vector<std::vector<float>> xb(count);
  for (size_t k = 0; k < count; ++k) {
    const auto &gi = g.insts[k];
    for (int r = 1; r < gi.R; ++r)
      if (energies[k][r] < energies[k][best[k]]) best[k] = r;
    xb[k].resize(gi.n);
    e = cudaMemcpyAsync(xb[k].data(), gi.x + (size_t)best[k] * gi.xp, (size_t)gi.n * sizeof(float),
                        cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && res[k].final_x)
      e = cudaMemcpy2DAsync(res[k].final_x, (size_t)gi.n * 4, gi.x, (size_t)gi.xp * 4, (size_t)gi.n * 4, (size_t)gi.R,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && res[k].final_y)
      e = cudaMemcpy2DAsync(res[k].final_y, (size_t)gi.n * 4, gi.y, (size_t)gi.xp * 4, (size_t)gi.n * 4, (size_t)gi.R,
                            cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) break;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("batch results: ") + cudaGetErrorString(e);
    return SB_ERR_CUDA;
  }
  // exact host re-check of every returned spin vector, spread over the host cores
  std::vector<int64_t> e64(count, 0);
  std::vector<int> okv(count, 0);
  std::vector<std::vector<int8_t>> spins(count);
  const unsigned nth = std::max(1u, std::min(std::thread::hardware_concurrency(), (unsigned)count));
  std::vector<std::thread> th;
  for (unsigned w = 0; w < nth; ++w)
    th.emplace_back([&, w] {
      for (size_t k = w; k < count; k += nth) {
        const auto &gi = g.insts[k];
        spins[k].resize(gi.n);
        for (int i = 0; i < gi.n; ++i) spins[k][i] = xb[k][i] > 0.0f ? 1 : -1;
        if (b->copies->energy(k, spins[k].data(), &e64[k], 1) == SB_OK)
          okv[k] = (double)e64[k] == energies[k][best[k]] ? 1 : 0;
      }
    });
  for (auto &t : th) t.join();
  const double total_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  double updates = 0;
  for (size_t k = 0; k < count; ++k) updates += (double)g.insts[k].n * g.insts[k].R * steps;
  for (size_t k = 0; k < count; ++k) {
    sb_result &r = res[k];
    if (r.best_spins) memcpy(r.best_spins, spins[k].data(), spins[k].size());
    if (r.replica_energies) memcpy(r.replica_energies, energies[k].data(), energies[k].size() * sizeof(double));
    r.best_energy = energies[k][best[k]];
    r.best_energy_i64 = e64[k];
    r.best_replica = best[k];
    r.field_mode_used = SB_FIELD_TC;
    r.field_dtype_used = g.fp4 ? SB_OPERAND_FP4 : SB_OPERAND_FP8;
    r.energy_check_ok = okv[k];
    r.device_ms = dev_ms;
    r.kernel_ms_avg = kernel_ms;
    r.steps_per_launch = 1;
    r.kernel_launches = g.launches - l0 + 2 * (int64_t)count;  // + init and sign kernels per instance
    r.total_ms = total_ms;
    r.spin_updates_per_s = dev_ms > 0 ? updates / (dev_ms * 1e-3) : 0.0;
  }
  return SB_OK;
}

}  // namespace

extern "C" {

sb_status sb_batch_create(sb_ctx *ctx, const sb_problem *problems, int32_t count, const sb_params *params,
                          sb_batch **out) {
  if (!ctx || !out) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  std::string err;
  sb_status s = create(ctx, problems, count, params, out, err);
  ctx->last_error = err;
  return s;
}

sb_status sb_batch_run(sb_batch *b, uint64_t seed, sb_result *results) {
  if (!b || !results) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(b->ctx->mu);
  cudaSetDevice(b->ctx->device);
  std::string err;
  sb_status s = run(b, seed, results, err);
  b->ctx->last_error = err;
  return s;
}

sb_status sb_batch_destroy(sb_batch *b) {
  if (!b) return SB_ERR_INVALID_ARG;
  sb_ctx *ctx = b->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  destroy(b);
  return SB_OK;
}

sb_status sb_solve_batch(sb_ctx *ctx, const sb_problem *problems, int32_t count, const sb_params *params,
                         sb_result *results) {
  sb_batch *b = nullptr;
  sb_status s = sb_batch_create(ctx, problems, count, params, &b);
  if (s != SB_OK) return s;
  s = sb_batch_run(b, params->seed, results);
  sb_batch_destroy(b);
  return s;
}

}  // extern "C"
