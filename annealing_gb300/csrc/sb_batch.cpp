// sb_batch_*: many instances of uneven size solved together by the grouped tensor-core kernel.
//
// The reference solves one instance per program run and its trials one after another
// (SB/CUDA_GPU/m2_opt.cu:152); a batch here advances every instance and every replica of it in
// one grouped launch per SB step and operand bucket (packed E2M1 where the couplings allow it,
// packed E2M3 for the rest), the step loop replayed from a CUDA graph. Per instance the outputs are those
// of sb_solve (best spins, per-replica energies, host int64 re-check).
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

// One operand bucket of a batch: the instances whose couplings share an operand type (packed E2M1
// when every coupling is an integer |J| <= 4, else packed E2M3), advanced by their own grouped
// launch per step with their own autotuned replica tile and item order.
struct sb_bucket {
  sbk::Grouped *g = nullptr;
  std::vector<int> members;  // batch index of each resident instance, in residence order
};

struct sb_batch {
  sb_ctx *ctx = nullptr;
  std::vector<const sb_problem *> probs;
  sb_params prm{};
  std::vector<sb_bucket> buckets;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // compact copies of the couplings for the host re-check, built in the background (the first
  // runs' device time hides them)
  std::unique_ptr<sbh::CouplingCopies> copies;
};

namespace {

std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune_cache;

// instance k of the batch starts from seed + k, whichever bucket holds it
sb_status init_all(sb_bucket &bk, uint64_t seed, std::string &err) {
  for (size_t j = 0; j < bk.g->insts.size(); ++j) {
    sb_status s = bk.g->init_state(bk.g->insts[j], seed + (uint64_t)bk.members[j], err);
    if (s != SB_OK) return s;
  }
  return SB_OK;
}

// Times a few steps of each (replica tile, item order) candidate on the bucket itself and keeps the
// fastest; the choice is cached by (replica count, total work bucket, batch size bucket, operands).
sb_status autotune(sb_batch *b, sb_bucket &bk, std::string &err) {
  sbk::Grouped &g = *bk.g;
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
      if ((s = init_all(bk, b->prm.seed, err)) != SB_OK) return s;
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
  for (auto &bk : b->buckets) delete bk.g;
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
            ": the grouped path runs dSB with integer couplings |J| <= 16 (exact E2M1 / E2M3 / FP8 operands)";
      return SB_ERR_UNSUPPORTED;
    }
  }
  // operands per instance: packed E2M1 where its couplings allow it (integers |J| <= 4; half the
  // bytes of FP8), else packed E2M3 (six bits per coupling); SB_OPERAND_FP8 / SB_OPERAND_FP6 /
  // SB_OPERAND_FP4 force one type for the batch
  std::vector<int> op(count, sbk::kGopE2m3);
  bool all_fp4 = true;
  for (int k = 0; k < count; ++k) {
    if (sbk::grouped_fp4_exact(&problems[k])) op[k] = sbk::kGopE2m1;
    all_fp4 = all_fp4 && op[k] == sbk::kGopE2m1;
  }
  if (prm->operand_dtype == SB_OPERAND_FP8 || prm->operand_dtype == SB_OPERAND_FP6) {
    std::fill(op.begin(), op.end(), prm->operand_dtype == SB_OPERAND_FP8 ? sbk::kGopFp8 : sbk::kGopE2m3);
  } else if (prm->operand_dtype == SB_OPERAND_FP4) {
    if (!all_fp4) {
      err = "E2M1 operands need integer couplings |J| <= 4 in every problem of the batch";
      return SB_ERR_UNSUPPORTED;
    }
  } else if (prm->operand_dtype != SB_OPERAND_AUTO) {
    err = "the grouped path runs E2M1, E2M3 or FP8 operands";
    return SB_ERR_UNSUPPORTED;
  }
  sb_batch *b = new sb_batch();
  b->ctx = ctx;
  b->prm = *prm;
  b->probs.resize(count);
  const int R = prm->replicas;
  const int nr = R <= 32 ? 32 : (R <= 64 ? 64 : 128);  // the autotuner may retile each bucket
  for (int o : {sbk::kGopE2m1, sbk::kGopE2m3, sbk::kGopFp8}) {
    sb_bucket bk;
    for (int k = 0; k < count; ++k)
      if (op[k] == o) bk.members.push_back(k);
    if (bk.members.empty()) continue;
    bk.g = new sbk::Grouped(ctx->stream, nr, 0, o);
    b->buckets.push_back(std::move(bk));
  }
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
        const sb_status st =
            sbk::Grouped::prepare(hosts[k], &problems[k], prm, prm->seed + k, k, nr, ps, stg, errs[w], op[k]);
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
  for (int k = 0; k < count; ++k) b->probs[k] = &problems[k];
  for (auto &bk : b->buckets)
    for (int k : bk.members) bk.g->attach(hosts[k], 0);
  for (auto &bk : b->buckets) {
    sb_status s = autotune(b, bk, err);
    if (s == SB_OK) s = bk.g->sync_tables(err);
    if (s != SB_OK) {
      destroy(b);
      return s;
    }
  }
  b->copies.reset(new sbh::CouplingCopies(
      b->probs, (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2))));
  *out = b;
  return SB_OK;
}

sb_status run(sb_batch *b, uint64_t seed, sb_result *res, std::string &err) {
  cudaStream_t st = b->ctx->stream;
  const int steps = b->prm.steps;
  const auto t_start = std::chrono::steady_clock::now();
  int64_t l0 = 0;
  for (auto &bk : b->buckets) {
    sb_status s = bk.g->sync_tables(err);
    if (s != SB_OK) return s;
    if (cudaMemsetAsync(bk.g->d_status, 0, sizeof(uint32_t), st) != cudaSuccess) return SB_ERR_CUDA;
    l0 += bk.g->launches;
  }
  cudaEventRecord(b->ev0, st);
  for (auto &bk : b->buckets) {
    sb_status s = init_all(bk, seed, err);
    if (s != SB_OK) return s;
  }
  cudaError_t e = cudaSuccess;
  double kernel_ms = 0.0;  // profile: device time of one SB step, all buckets' launches
  for (auto &bk : b->buckets) {
    sbk::Grouped &g = *bk.g;
    if (b->prm.profile && steps > 0) {
      std::vector<cudaEvent_t> evs(2 * (size_t)steps);
      for (auto &ev : evs) cudaEventCreate(&ev);
      for (int t = 0; t < steps && e == cudaSuccess; ++t) {
        cudaEventRecord(evs[2 * t], st);
        e = g.run_steps(t, 1, false);
        cudaEventRecord(evs[2 * t + 1], st);
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      double ms_sum = 0.0;
      for (int t = 0; t < steps && e == cudaSuccess; ++t) {
        float ms = 0;
        cudaEventElapsedTime(&ms, evs[2 * t], evs[2 * t + 1]);
        ms_sum += ms;
      }
      for (auto &ev : evs) cudaEventDestroy(ev);
      kernel_ms += ms_sum / steps;
    } else if (e == cudaSuccess) {
      e = g.run_steps(0, steps, true);
    }
    if (e == cudaSuccess) e = g.energy_pass(steps);
  }
  cudaEventRecord(b->ev1, st);
  const size_t count = b->probs.size();
  // (bucket, position) of every batch index
  std::vector<const sbk::GHost *> inst(count, nullptr);
  std::vector<int> inst_op(count, sbk::kGopFp8);
  for (auto &bk : b->buckets)
    for (size_t j = 0; j < bk.members.size(); ++j) {
      inst[bk.members[j]] = &bk.g->insts[j];
      inst_op[bk.members[j]] = bk.g->op;
    }
  std::vector<std::vector<double>> energies(count);
  std::vector<uint32_t> status(b->buckets.size(), 0);
  for (size_t k = 0; k < count && e == cudaSuccess; ++k) {
    energies[k].resize(inst[k]->R);
    e = cudaMemcpyAsync(energies[k].data(), inst[k]->energy, (size_t)inst[k]->R * sizeof(double),
                        cudaMemcpyDeviceToHost, st);
  }
  for (size_t i = 0; i < b->buckets.size() && e == cudaSuccess; ++i)
    e = cudaMemcpyAsync(&status[i], b->buckets[i].g->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("batch run: ") + cudaGetErrorString(e);
    return SB_ERR_CUDA;
  }
  uint32_t any = 0;
  for (uint32_t v : status) any |= v;
  if (any) {
    err = sbh::device_status_text(any);
    return (any & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
  }
  float dev_ms = 0;
  cudaEventElapsedTime(&dev_ms, b->ev0, b->ev1);
  // best replica of each instance, its spins, optional full state
  std::vector<int> best(count, 0);
  std::vector<std::vector<float>> xb(count);
  for (size_t k = 0; k < count; ++k) {
    const auto &gi = *inst[k];
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
        const auto &gi = *inst[k];
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
  int64_t launches = -l0;
  for (size_t k = 0; k < count; ++k) updates += (double)inst[k]->n * inst[k]->R * steps;
  for (auto &bk : b->buckets) launches += bk.g->launches;
  for (size_t k = 0; k < count; ++k) {
    sb_result &r = res[k];
    if (r.best_spins) memcpy(r.best_spins, spins[k].data(), spins[k].size());
    if (r.replica_energies) memcpy(r.replica_energies, energies[k].data(), energies[k].size() * sizeof(double));
    r.best_energy = energies[k][best[k]];
    r.best_energy_i64 = e64[k];
    r.best_replica = best[k];
    r.field_mode_used = SB_FIELD_TC;
    r.field_dtype_used = inst_op[k] == sbk::kGopE2m1 ? SB_OPERAND_FP4
                         : inst_op[k] == sbk::kGopE2m3 ? SB_OPERAND_FP6 : SB_OPERAND_FP8;
    r.energy_check_ok = okv[k];
    r.device_ms = dev_ms;
    r.kernel_ms_avg = kernel_ms;
    r.steps_per_launch = 1;
    r.kernel_launches = launches + 2 * (int64_t)count;  // + init and sign kernels per instance
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
