// Continuous-batching request server behind sb_submit / sb_poll / sb_cancel.
//
// The reference has no service: one instance per program run, trials one after another
// (SB/CUDA_GPU/m2_opt.cu:152). Here a worker thread owns a stream and a set of grouped engines
// (one per replica tile). Requests queue in arrival order; the worker admits them while the
// in-flight limit and the HBM budget allow (the budget counts each resident request's device
// bytes), so requests that arrive while others run join the running set at the next tick and
// their steps overlap on the device with everyone else's: one grouped launch per tick advances
// every resident request by one SB step, each on its own schedule. A request retires at its own
// step budget (energy pass, best spins back to the host, exact int64 re-check) and its memory is
// freed for the next. Requests the grouped engine does not cover (bSB, aSB, real couplings,
// |J| > 16) are solved one at a time on the worker's stream between ticks.
#include "sb_serve.h"

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sb_grouped.h"
#include "sb_host.h"
#include "sb_internal.h"

namespace sbs {

namespace {
using Clock = std::chrono::steady_clock;

// Couplings of grouped requests (integers |J| <= 16) are held as packed E2M3, six bits per coupling:
// the step's HBM traffic is mostly couplings, and this is a quarter less than FP8 for the same
// exact products.
constexpr int kServeOperand = sbk::kGopE2m3;

enum State { kQueued = 0, kResident = 1, kDone = 2, kCancelled = 3, kFailed = 4 };

struct Req {
  uint64_t ticket = 0;
  const sb_problem *prob = nullptr;
  sb_params prm{};
  Clock::time_point submitted, admitted, done;
  int state = kQueued;
  std::atomic<bool> cancel{false};
  int mode = 0, dtype = 0;
  int nr = 0;
  int64_t bytes = 0;
  int ticks = 0;
  sb_status status = SB_OK;
  std::string err;
  std::vector<int8_t> spins;
  std::vector<double> energies;
  double best = 0;
  int64_t e64 = 0;
  int best_r = 0, ok = 0;
};

int tile_for(int R) { return R <= 32 ? 32 : (R <= 64 ? 64 : 128); }
}  // namespace

struct Server {
  int device = 0;
  cudaStream_t st = nullptr;
  int64_t budget = 0, used = 0;
  int max_inflight = 64;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::deque<Req *> queue;
  std::unordered_map<uint64_t, Req *> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
  std::map<int, sbk::Grouped *> groups;
  std::vector<Req *> resident;
  // admission runs on its own thread and stream: requests are prepared (allocated, uploaded,
  // seeded) while the worker keeps stepping the resident ones, then attached at a tick boundary
  static constexpr int kPreparers = 4;
  std::thread preparer[kPreparers];
  cudaStream_t pst[kPreparers] = {};
  sbk::Staging stg[kPreparers];
  std::vector<std::pair<Req *, sbk::GHost>> ready;
  int preparing = 0;
  void prepare_loop(int w);
  void attach_ready();
  int tick = 0;
  sb_serving_stats stats{};
  sb_ctx *solo = nullptr;  // requests outside the grouped engine
  Clock::time_point t_start = Clock::now();
  // exact host re-checks run on their own threads so the device loop never waits for them
  std::vector<std::thread> energy_threads;
  std::deque<std::pair<Req *, sb_status>> check_q;
  std::condition_variable check_cv;
  bool check_stop = false;
  void check_loop();

  void run();

  void retire(int at_tick);
  void finish(Req *r, sb_status s, const std::string &err);
  void solve_alone(Req *r);
};

void Server::finish(Req *r, sb_status s, const std::string &err) {
  std::lock_guard<std::mutex> lk(mu);
  r->status = s;
  r->err = err;
  r->done = Clock::now();
  r->state = s == SB_OK ? kDone : (s == SB_ERR_CANCELLED ? kCancelled : kFailed);
  if (s == SB_ERR_CANCELLED) ++stats.cancelled;
  else ++stats.finished;
  done_cv.notify_all();
}

void Server::solve_alone(Req *r) {
  sb_result res;
  memset(&res, 0, sizeof(res));
  r->spins.assign(r->prob->n, 0);
  r->energies.assign(r->prm.replicas, 0.0);
  res.best_spins = r->spins.data();
  res.replica_energies = r->energies.data();
  sb_params p = r->prm;
  p.trace = p.trace_all = 0;
  sb_status s = SB_ERR_NO_DEVICE;
  if (solo) s = sb_solve(solo, r->prob, &p, &res);
  r->best = res.best_energy;
  r->mode = res.field_mode_used;
  r->dtype = res.field_dtype_used;
  r->e64 = res.best_energy_i64;
  r->best_r = res.best_replica;
  r->ok = res.energy_check_ok;
  r->ticks = p.steps;
  finish(r, s, s == SB_OK ? "" : std::string(sb_last_error(solo)));
}

// Admission thread: takes requests in arrival order while the in-flight limit and the HBM budget
// allow (a request that does not fit waits, and so does everything behind it), prepares each on
// its own stream, and hands it to the worker.
void Server::prepare_loop(int w) {
  cudaSetDevice(device);
  for (;;) {
    Req *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      for (;;) {
        if (stop) return;
        while (!queue.empty() && queue.front()->cancel) {
          Req *c = queue.front();
          queue.pop_front();
          c->state = kCancelled;
          c->status = SB_ERR_CANCELLED;
          c->done = Clock::now();
          ++stats.cancelled;
          done_cv.notify_all();
        }
        if (!queue.empty()) {
          Req *f = queue.front();
          const int inflight = (int)resident.size() + (int)ready.size() + preparing;
          const bool fits = used + f->bytes <= budget || inflight == 0;
          if (inflight < max_inflight && fits) {
            queue.pop_front();
            used += f->bytes;
            ++preparing;
            r = f;
            break;
          }
        }
        cv.wait_for(lk, std::chrono::milliseconds(20));
      }
    }
    r->admitted = Clock::now();
    const auto tp = Clock::now();
    if (r->nr == 0) {
      solve_alone(r);
      std::lock_guard<std::mutex> lk(mu);
      used -= r->bytes;
      --preparing;
      cv.notify_all();
      continue;
    }
    sbk::GHost g;
    std::string err;
    const sb_status s =
        sbk::Grouped::prepare(g, r->prob, &r->prm, r->prm.seed, (int)r->ticket, r->nr, pst[w], stg[w], err, kServeOperand);
    if (s != SB_OK) {
      {
        std::lock_guard<std::mutex> lk(mu);
        used -= r->bytes;
        --preparing;
      }
      finish(r, s, err);
      continue;
    }
    std::lock_guard<std::mutex> lk(mu);
    --preparing;
    stats.admit_ms += std::chrono::duration<double, std::milli>(Clock::now() - tp).count();
    ready.push_back({r, g});
    cv.notify_all();
  }
}

// Worker: makes prepared requests resident; they take their first step at the current tick.
void Server::attach_ready() {
  std::vector<std::pair<Req *, sbk::GHost>> take;
  {
    std::lock_guard<std::mutex> lk(mu);
    take.swap(ready);
  }
  for (auto &rg : take) {
    Req *r = rg.first;
    sbk::Grouped *&g = groups[r->nr];
    if (!g) g = new sbk::Grouped(st, r->nr, 0, kServeOperand);
    g->attach(rg.second, tick);
    std::lock_guard<std::mutex> lk(mu);
    r->state = kResident;
    resident.push_back(r);
    stats.peak_inflight = std::max<int64_t>(stats.peak_inflight, (int64_t)resident.size());
  }
}

// Retires every resident request whose step budget ends at `at_tick`, and drops cancelled ones.
void Server::retire(int at_tick) {
  std::vector<Req *> fin, gone;
  for (Req *r : resident) {
    if (r->cancel) gone.push_back(r);
    else if (r->ticks >= r->prm.steps) fin.push_back(r);
  }
  if (fin.empty() && gone.empty()) return;
  // energies of the finishing requests, per engine
  std::map<int, std::vector<int>> by_group;
  for (Req *r : fin) by_group[r->nr].push_back(groups[r->nr]->find((int)r->ticket));
  for (auto &kv : by_group) {
    cudaError_t e = groups[kv.first]->energy_pass_for(kv.second, at_tick);
    if (e != cudaSuccess)
      for (Req *r : fin)
        if (r->nr == kv.first) {
          r->status = SB_ERR_CUDA;
          r->err = std::string("energy pass: ") + cudaGetErrorString(e);
        }
  }
  uint32_t status = 0;
  for (auto &kv : groups)
    if (kv.second->d_status) cudaMemcpyAsync(&status, kv.second->d_status, 4, cudaMemcpyDeviceToHost, st);
  for (Req *r : fin) {
    sbk::Grouped *g = groups[r->nr];
    const sbk::GHost &gi = g->insts[g->find((int)r->ticket)];
    r->energies.resize(gi.R);
    cudaMemcpyAsync(r->energies.data(), gi.energy, (size_t)gi.R * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  cudaStreamSynchronize(st);
  std::vector<std::vector<float>> xbs(fin.size());
  for (size_t q = 0; q < fin.size(); ++q) {
    Req *r = fin[q];
    sbk::Grouped *g = groups[r->nr];
    const sbk::GHost &gi = g->insts[g->find((int)r->ticket)];
    int b = 0;
    for (int k = 1; k < gi.R; ++k)
      if (r->energies[k] < r->energies[b]) b = k;
    r->best_r = b;
    r->best = r->energies[b];
    xbs[q].resize(gi.n);
    cudaMemcpyAsync(xbs[q].data(), gi.x + (size_t)b * gi.xp, (size_t)gi.n * sizeof(float), cudaMemcpyDeviceToHost, st);
  }
  cudaStreamSynchronize(st);
  for (size_t q = 0; q < fin.size(); ++q) {
    Req *r = fin[q];
    r->spins.resize(xbs[q].size());
    for (size_t i = 0; i < xbs[q].size(); ++i) r->spins[i] = xbs[q][i] > 0.0f ? 1 : -1;
  }
  // free the finished and the cancelled
  std::vector<Req *> out = fin;
  out.insert(out.end(), gone.begin(), gone.end());
  for (Req *r : out) {
    sbk::Grouped *g = groups[r->nr];
    g->remove(g->find((int)r->ticket));
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    for (Req *r : out) {
      used -= r->bytes;
      resident.erase(std::find(resident.begin(), resident.end(), r));
    }
  }
  cv.notify_all();  // room for the next admission
  {
    std::lock_guard<std::mutex> lk(mu);
    for (Req *r : fin)
      check_q.push_back({r, (status & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : r->status});
  }
  check_cv.notify_all();
  for (Req *r : gone) finish(r, SB_ERR_CANCELLED, "cancelled");
}

void Server::run() {
  cudaSetDevice(device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      if (stop) break;
      if (ready.empty() && resident.empty()) {
        cv.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    attach_ready();
    if (resident.empty()) continue;
    const auto t0 = Clock::now();
    std::string err;
    for (auto &kv : groups)
      if (kv.second->sync_tables(err) != SB_OK) {
        // fail everything resident in this engine
        std::vector<Req *> bad;
        for (Req *r : resident)
          if (r->nr == kv.first) bad.push_back(r);
        for (Req *r : bad) r->cancel = true;
      }
    // run ticks up to the next retirement (at most 32, to take in new arrivals)
    int nt = 32;
    for (Req *r : resident) nt = std::min(nt, r->prm.steps - r->ticks);
    if (nt < 0) nt = 0;
    for (int s = 0; s < nt; ++s) {
      for (auto &kv : groups)
        if (kv.second->n_items > 0) {
          const int64_t before = kv.second->launches;
          kv.second->run_steps(tick, 1, false);
          stats.grouped_launches += kv.second->launches - before;
        }
      ++tick;
    }
    for (Req *r : resident) r->ticks += nt;
    stats.ticks += nt;
    cudaStreamSynchronize(st);
    retire(tick);
    stats.busy_ms += std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
  }
}

void Server::check_loop() {
  for (;;) {
    std::pair<Req *, sb_status> job;
    {
      std::unique_lock<std::mutex> lk(mu);
      check_cv.wait(lk, [&] { return check_stop || !check_q.empty(); });
      if (check_q.empty()) return;
      job = check_q.front();
      check_q.pop_front();
    }
    Req *r = job.first;
    if (job.second == SB_OK && sbh::energy_i64(r->prob, r->spins.data(), &r->e64, 1) == SB_OK)
      r->ok = (double)r->e64 == r->best ? 1 : 0;
    finish(r, job.second, job.second == SB_OK ? "" : (r->err.empty() ? std::string("device error") : r->err));
  }
}

sb_status server_create(Server **out, int device, int64_t hbm_budget, int max_inflight, std::string &err) {
  Server *s = new Server();
  s->device = device;
  s->budget = hbm_budget;
  s->max_inflight = max_inflight;
  cudaSetDevice(device);
  bool streams_ok = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) == cudaSuccess;
  for (int w = 0; w < Server::kPreparers; ++w)
    streams_ok = streams_ok && cudaStreamCreateWithFlags(&s->pst[w], cudaStreamNonBlocking) == cudaSuccess;
  if (!streams_ok) {
    delete s;
    err = "cudaStreamCreate";
    return SB_ERR_CUDA;
  }
  // keep freed blocks in the stream-ordered pool instead of returning them at every sync
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = (uint64_t)(hbm_budget > 0 ? hbm_budget : 0);
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  sb_device_opts o;
  memset(&o, 0, sizeof(o));
  o.device = device;
  o.stream = s->pst[0];  // solo solves run on an admission thread
  if (sb_create(&s->solo, &o) != SB_OK) s->solo = nullptr;
  s->worker = std::thread([s] { s->run(); });
  for (int w = 0; w < Server::kPreparers; ++w) s->preparer[w] = std::thread([s, w] { s->prepare_loop(w); });
  const unsigned nc = std::max(2u, std::min(8u, std::thread::hardware_concurrency() / 2));
  for (unsigned k = 0; k < nc; ++k) s->energy_threads.emplace_back([s] { s->check_loop(); });
  *out = s;
  return SB_OK;
}

void server_destroy(Server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto &t : s->preparer)
    if (t.joinable()) t.join();
  for (auto &rg : s->ready) sbk::Grouped::release(rg.second, s->pst[0]);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->check_stop = true;
  }
  s->check_cv.notify_all();
  for (auto &t : s->energy_threads) t.join();
  cudaSetDevice(s->device);
  for (auto &kv : s->groups) delete kv.second;
  for (auto &kv : s->reqs) delete kv.second;
  if (s->solo) sb_destroy(s->solo);
  for (auto ps : s->pst) cudaStreamSynchronize(ps);
  cudaStreamDestroy(s->st);
  for (auto ps : s->pst) cudaStreamDestroy(ps);
  delete s;
}

sb_status server_submit(Server *s, const sb_problem *p, const sb_params *prm, uint64_t *ticket) {
  Req *r = new Req();
  r->prob = p;
  r->prm = *prm;
  r->submitted = Clock::now();
  const bool grouped = sbk::grouped_supports(p, prm) && prm->trace == 0 && prm->trace_all == 0;
  r->nr = grouped ? tile_for(prm->replicas) : 0;
  r->bytes = grouped ? sbk::grouped_instance_bytes(p->n, prm->replicas, prm->steps, r->nr, kServeOperand)
                     : sb_plan_footprint(p, prm);
  std::lock_guard<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  s->reqs[r->ticket] = r;
  s->queue.push_back(r);
  ++s->stats.submitted;
  *ticket = r->ticket;
  s->cv.notify_all();
  return SB_OK;
}

sb_status server_poll(Server *s, uint64_t ticket, sb_result *res, int32_t wait_ms, std::string &err) {
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return SB_ERR_NOT_FOUND;
  Req *r = it->second;
  auto finished = [&] { return r->state >= kDone; };
  if (!finished()) {
    if (wait_ms == 0) return SB_ERR_PENDING;
    if (wait_ms < 0)
      s->done_cv.wait(lk, finished);
    else if (!s->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), finished))
      return SB_ERR_PENDING;
  }
  const sb_status st = r->status;
  if (st != SB_OK) err = r->err;
  if (st == SB_OK) {
    if (res->best_spins) memcpy(res->best_spins, r->spins.data(), r->spins.size());
    if (res->replica_energies) memcpy(res->replica_energies, r->energies.data(), r->energies.size() * sizeof(double));
    res->best_energy = r->best;
    res->best_energy_i64 = r->e64;
    res->best_replica = r->best_r;
    res->energy_check_ok = r->ok;
    res->field_mode_used = r->nr ? SB_FIELD_TC : r->mode;
    res->field_dtype_used = r->nr ? SB_OPERAND_FP6 : r->dtype;
    res->device_ms = std::chrono::duration<double, std::milli>(r->done - r->admitted).count();
    res->total_ms = std::chrono::duration<double, std::milli>(r->done - r->submitted).count();
    res->kernel_launches = r->ticks;
    res->steps_per_launch = 1;
    res->spin_updates_per_s =
        res->device_ms > 0 ? (double)r->prob->n * r->prm.replicas * r->prm.steps / (res->device_ms * 1e-3) : 0.0;
  }
  s->reqs.erase(it);
  delete r;
  return st;
}

sb_status server_cancel(Server *s, uint64_t ticket) {
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return SB_ERR_NOT_FOUND;
  if (it->second->state >= kDone) return SB_OK;
  it->second->cancel = true;
  s->cv.notify_all();
  return SB_OK;
}

sb_status server_stats(Server *s, sb_serving_stats *out) {
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->inflight = (int64_t)s->resident.size();
  out->queued = (int64_t)s->queue.size();
  return SB_OK;
}

}  // namespace sbs
