// Host-side problem handling: graph reader, coefficients, schedule, exact energy evaluators.
// No CUDA here; everything in this file works without a GPU.
#include <math.h>
#include <algorithm>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <pthread.h>

#include <condition_variable>
#include <deque>
#include <new>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sb.h"
#include "sb_host.h"
#include "sb_internal.h"

extern "C" {

const char *sb_status_string(sb_status s) {
  switch (s) {
    case SB_OK: return "ok";
    case SB_ERR_INVALID_ARG: return "invalid argument";
    case SB_ERR_IO: return "i/o error";
    case SB_ERR_PARSE: return "parse error";
    case SB_ERR_CUDA: return "cuda error";
    case SB_ERR_OOM: return "out of memory";
    case SB_ERR_UNSUPPORTED: return "unsupported";
    case SB_ERR_TIMEOUT: return "device wait timed out";
    case SB_ERR_BUSY: return "busy";
    case SB_ERR_NOT_FOUND: return "not found";
    case SB_ERR_CANCELLED: return "cancelled";
    case SB_ERR_NO_DEVICE: return "no usable device";
    case SB_ERR_PENDING: return "pending";
  }
  return "unknown status";
}

int32_t sb_abi_version(void) { return SB_ABI_VERSION; }

void sb_params_default(sb_params *p, int32_t variant) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->variant = variant;
  p->field_mode = SB_FIELD_AUTO;
  p->init_mode = variant == SB_ASB ? SB_INIT_REFERENCE : SB_INIT_UNIFORM;
  p->steps = variant == SB_ASB ? 100 : 1000;  // aSB: STEP of m2_opt.cu:22
  p->replicas = 1;
  p->seed = 1234;
  p->dt = 1.25f;
  p->a0 = 1.0f;
  p->c0 = 0.0f;
  p->mts_m = 2;          // m2_opt.cu:21
  p->mts_dt = 0.5f;      // m2_opt.cu:19
  p->coupling_dt = 1.0f; // m2_opt.cu:20
  p->xi = 0.01565f;      // m2_opt.cu:18 (<= 0 selects 0.7 * detune / sqrt(N))
  p->detune = 1.0f;      // m2_opt.cu:17
  p->kerr = 1.0f;        // m2_opt.cu:16
}

void sb_graph_opts_default(sb_graph_opts *o) {
  if (!o) return;
  o->index_base = -1;
  o->n_override = 0;
  o->strict = 0;
}

float sb_pump(float a0, int32_t t, int32_t steps) {
  float a = (float)((double)a0 * (double)t / (double)steps);
  return a0 - a;
}

double sb_coupling_std(const sb_problem *p) { return sbh::coupling_std(p, 0); }

float sb_default_c0(const sb_problem *p) { return sbh::default_c0(p, 0); }

}  // extern "C"

namespace {
int auto_threads(int n, int threads) { return threads > 0 ? threads : sbh::host_threads(n); }
}  // namespace

float sbh::default_c0(const sb_problem *p, int threads) {
  double sd = sbh::coupling_std(p, threads);
  if (!(sd > 0.0)) sd = 1.0;
  return (float)(0.5 / (sqrt((double)(p ? p->n : 1)) * sd));
}

static double std_from_sums(int n, double s, double s2) {
  const double cnt = (double)n * (double)(n - 1);
  const double mean = s / cnt;
  const double var = s2 / cnt - mean * mean;
  return var > 0.0 ? sqrt(var) : 0.0;
}

float sbh::c0_from_sums(int n, int64_t s, int64_t s2) {
  double sd = n >= 2 ? std_from_sums(n, (double)s, (double)s2) : 0.0;
  if (!(sd > 0.0)) sd = 1.0;
  return (float)(0.5 / (sqrt((double)n) * sd));
}

double sbh::coupling_std(const sb_problem *p, int threads) {
  if (!p || !p->J || p->n < 2) return 0.0;
  const int n = p->n;
  // the scan's exact sums: the same doubles the integer pass below would produce
  if (p->stats_valid && p->integer_valued) return std_from_sums(n, (double)p->sum_j, (double)p->sum_j2);
  double s = 0.0, s2 = 0.0;
  const double maxj = (double)p->max_abs_j;
  if (p->integer_valued && p->max_abs_j < 2000000000 && (double)n * n * maxj * maxj < 9.0e15) {
    // Integer couplings whose sums stay below 2^53: the sequential double sums below are exact, so
    // exact int64 sums (vectorised, rows dealt round-robin to host threads) give the same doubles.
    const int nt = auto_threads(n, threads);
    std::vector<int64_t> ps((size_t)nt, 0), ps2((size_t)nt, 0);
    auto rows = [&](int t) {
      int64_t a = 0, a2 = 0;
      for (int i = t; i < n; i += nt) {
        const float *Ji = p->J + (size_t)i * n;
        int64_t r = 0, r2 = 0;
        for (int j = 0; j < n; ++j) {
          const int64_t v = (int64_t)(int32_t)Ji[j];
          r += v;
          r2 += v * v;
        }
        const int64_t d = (int64_t)(int32_t)Ji[i];  // the diagonal does not count
        a += r - d;
        a2 += r2 - d * d;
      }
      ps[t] = a;
      ps2[t] = a2;
    };
    sbh::parallel_run(nt, rows);
    int64_t a = 0, a2 = 0;
    for (int t = 0; t < nt; ++t) {
      a += ps[t];
      a2 += ps2[t];
    }
    s = (double)a;
    s2 = (double)a2;
  } else {
    for (int i = 0; i < n; ++i) {
      const float *Ji = p->J + (size_t)i * n;
      for (int j = 0; j < n; ++j) {
        if (i == j) continue;
        double v = (double)Ji[j];
        s += v;
        s2 += v * v;
      }
    }
  }
  return std_from_sums(n, s, s2);
}

extern "C" {

sb_status sb_energy_i64(const sb_problem *p, const int8_t *spins, int64_t *out) {
  return sbh::energy_i64(p, spins, out, 0);
}

}  // extern "C"

sb_status sbh::energy_i64(const sb_problem *p, const int8_t *spins, int64_t *out, int threads) {
  if (!p || !p->J || !spins || !out || p->n <= 0) return SB_ERR_INVALID_ARG;
  const int n = p->n;
  if (p->h)
    for (int i = 0; i < n; ++i)
      if (p->h[i] != floorf(p->h[i]) || !(fabsf(p->h[i]) < 9.0e18f)) return SB_ERR_UNSUPPORTED;
  // A problem scanned on creation (sb_problem_init / wrap / load / random) carries its
  // integrality and max |J|: the couplings need no per-element test, and when n * max|J| stays
  // below 2^31 every row sum is exact in int32, which the compiler vectorises. Otherwise each
  // coupling is tested and the products are summed in int64.
  const bool scanned = p->integer_valued != 0;
  const bool row32 = scanned && p->max_abs_j < 2000000000 && (double)p->max_abs_j * (double)n < 2147483647.0;
  // rows [i0, i1) step `stride` of the upper triangle; false on a non-integral coupling
  auto rows = [&](int i0, int stride, int64_t &sum) -> bool {
    int64_t e = 0;
    for (int i = i0; i < n; i += stride) {
      const float *Ji = p->J + (size_t)i * n;
      int64_t row = 0;
      if (row32) {
        int32_t acc = 0;
        for (int j = i + 1; j < n; ++j) {
          const int32_t w = (int32_t)Ji[j];
          const int32_t m = (int32_t)spins[j] >> 1;  // 0 for +1, -1 for -1
          acc += (w ^ m) - m;
        }
        row = acc;
      } else {
        for (int j = i + 1; j < n; ++j) {
          const float w = Ji[j];
          if (w != floorf(w) || !(fabsf(w) < 9.0e18f)) return false;
          row += (int64_t)w * (int64_t)spins[j];
        }
      }
      e -= row * (int64_t)spins[i];
      if (p->h) e -= (int64_t)p->h[i] * (int64_t)spins[i];
    }
    sum = e;
    return true;
  };
  // large problems: rows dealt round-robin to host threads (the triangle stays balanced); the
  // integer sum does not depend on the split
  const int nt = auto_threads(n, threads);
  std::vector<int64_t> part((size_t)nt, 0);
  std::vector<char> ok((size_t)nt, 1);
  sbh::parallel_run(nt, [&](int t) { ok[t] = rows(t, nt, part[t]); });
  int64_t e = 0;
  for (int t = 0; t < nt; ++t) {
    if (!ok[t]) return SB_ERR_UNSUPPORTED;
    e += part[t];
  }
  *out = e;
  return SB_OK;
}

// ---------------------------------------------------------------------------------------------
// Compact coupling copies for the int64 re-check.

bool sbh::CouplingCopy::build(const sb_problem *p, const std::atomic<bool> *cancel) {
  mode = kNone;
  nz.clear();
  neg.clear();
  upper.clear();
  j8.clear();
  h.clear();
  if (!p || !p->J || p->n <= 0) return false;
  const int nn = p->n;
  auto stop = [&] { return cancel && cancel->load(std::memory_order_relaxed); };
  std::vector<int64_t> hv;
  if (p->h) {
    hv.resize((size_t)nn);
    for (int i = 0; i < nn; ++i) {
      const float v = p->h[i];
      if (v != floorf(v) || !(fabsf(v) < 9.0e18f)) return false;
      hv[(size_t)i] = (int64_t)v;
    }
  }
  // the scan on creation (sb_problem_init / wrap / load / random) vouches for integral couplings
  // and their largest magnitude, which picks the form
  if (!p->integer_valued || p->max_abs_j > 127) return false;
  const int amax = p->max_abs_j;
  n = nn;
  if (amax <= 1) {
    words = (nn + 63) / 64;
    nz.assign((size_t)nn * words, 0);
    neg.assign((size_t)nn * words, 0);
    for (int i = 0; i < nn; ++i) {
      if ((i & 63) == 0 && stop()) return false;
      const float *Ji = p->J + (size_t)i * nn;
      uint64_t *zi = nz.data() + (size_t)i * words, *gi = neg.data() + (size_t)i * words;
      for (int w = 0; w < words; ++w) {
        const int j0 = 64 * w, j1 = std::min(nn, j0 + 64);
        uint64_t z = 0, g = 0;
        if (j1 - j0 == 64) {
          // eight bytes of eight bits each
          for (int q = 0; q < 8; ++q) {
            const float *v = Ji + j0 + 8 * q;
            uint32_t zb = 0, gb = 0;
            for (int b = 0; b < 8; ++b) {
              zb |= (uint32_t)(v[b] != 0.0f) << b;
              gb |= (uint32_t)(v[b] < 0.0f) << b;
            }
            z |= (uint64_t)zb << (8 * q);
            g |= (uint64_t)gb << (8 * q);
          }
        } else {
          for (int j = j0; j < j1; ++j) {
            z |= (uint64_t)(Ji[j] != 0.0f) << (j - j0);
            g |= (uint64_t)(Ji[j] < 0.0f) << (j - j0);
          }
        }
        zi[w] = z;
        gi[w] = g;
      }
    }
    upper.assign((size_t)nn, 0);
    for (int i = 0; i + 1 < nn; ++i) {
      const uint64_t *zi = nz.data() + (size_t)i * words;
      const int w0 = (i + 1) >> 6;
      int32_t c = 0;
      for (int w = w0; w < words; ++w) c += __builtin_popcountll(zi[w] & (w == w0 ? ~0ull << ((i + 1) & 63) : ~0ull));
      upper[(size_t)i] = c;
    }
    mode = kBits;
  } else {
    j8.resize((size_t)nn * nn);
    for (int i = 0; i < nn; ++i) {
      if ((i & 63) == 0 && stop()) return false;
      const float *Ji = p->J + (size_t)i * nn;
      int8_t *di = j8.data() + (size_t)i * nn;
      for (int j = 0; j < nn; ++j) di[j] = (int8_t)Ji[j];
    }
    mode = kInt8;
  }
  h.swap(hv);
  return true;
}

int64_t sbh::CouplingCopy::energy(const int8_t *spins, int threads) const {
  // E = -sum_{i<j} J_ij s_i s_j - sum_i h_i s_i, rows i dealt round-robin to host threads
  std::vector<uint64_t> sn;
  if (mode == kBits) {
    sn.assign((size_t)words, 0);
    for (int j = 0; j < n; ++j) sn[(size_t)(j >> 6)] |= (uint64_t)(spins[j] < 0) << (j & 63);
  }
  auto rows = [&](int i0, int stride) -> int64_t {
    int64_t e = 0;
    for (int i = i0; i < n; i += stride) {
      int64_t row = 0;
      if (mode == kBits) {
        // sum_{j>i} J_ij s_j = (nonzero couplings) - 2 (those whose product is -1)
        const int j0 = i + 1;
        if (j0 < n) {
          const uint64_t *zi = nz.data() + (size_t)i * words, *gi = neg.data() + (size_t)i * words;
          const int w0 = j0 >> 6;
          int64_t minus = __builtin_popcountll(zi[w0] & (gi[w0] ^ sn[(size_t)w0]) & (~0ull << (j0 & 63)));
          for (int w = w0 + 1; w < words; ++w) minus += __builtin_popcountll(zi[w] & (gi[w] ^ sn[(size_t)w]));
          row = (int64_t)upper[(size_t)i] - 2 * minus;
        }
      } else {
        const int8_t *Ji = j8.data() + (size_t)i * n;
        int32_t acc = 0;  // |acc| <= 127 n
        for (int j = i + 1; j < n; ++j) acc += (int32_t)Ji[j] * (int32_t)spins[j];
        row = acc;
      }
      e -= row * (int64_t)spins[i];
      if (!h.empty()) e -= h[(size_t)i] * (int64_t)spins[i];
    }
    return e;
  };
  const int nt = threads > 0 ? threads : (mode == kInt8 && n >= 4096 ? auto_threads(n, 0) : 1);
  if (nt <= 1) return rows(0, 1);
  std::vector<int64_t> part((size_t)nt, 0);
  sbh::parallel_run(nt, [&](int t) { part[(size_t)t] = rows(t, nt); });
  int64_t e = 0;
  for (int64_t v : part) e += v;
  return e;
}

sbh::CouplingCopies::CouplingCopies(std::vector<const sb_problem *> probs, int threads)
    : probs_(std::move(probs)), copies_(probs_.size()), ready_(new std::atomic<int>[probs_.size()]) {
  for (size_t k = 0; k < probs_.size(); ++k) ready_[k].store(0);
  const size_t nt = std::max<size_t>(1, std::min<size_t>((size_t)std::max(1, threads), probs_.size()));
  for (size_t t = 0; t < nt; ++t)
    th_.emplace_back([this, t, nt] {
      for (size_t k = t; k < probs_.size() && !cancel_.load(std::memory_order_relaxed); k += nt)
        if (copies_[k].build(probs_[k], &cancel_)) ready_[k].store(1, std::memory_order_release);
    });
}

sbh::CouplingCopies::~CouplingCopies() {
  cancel_.store(true);
  for (auto &t : th_)
    if (t.joinable()) t.join();
}

bool sbh::CouplingCopies::ready(size_t k) const {
  return k < probs_.size() && ready_[k].load(std::memory_order_acquire) != 0;
}

sb_status sbh::CouplingCopies::energy(size_t k, const int8_t *spins, int64_t *out, int threads) const {
  if (k >= probs_.size() || !spins || !out) return SB_ERR_INVALID_ARG;
  if (ready(k)) {
    *out = copies_[k].energy(spins, threads);
    return SB_OK;
  }
  return sbh::energy_i64(probs_[k], spins, out, threads);
}

extern "C" sb_status sb_energies_i64(const sb_problem *p, const int8_t *spins, int32_t count, int64_t *out) {
  if (!p || !p->J || p->n <= 0 || !spins || !out || count < 0) return SB_ERR_INVALID_ARG;
  const size_t n = (size_t)p->n;
  sbh::CouplingCopy c;
  if (count < 2 || !c.build(p)) {
    // one vector, or couplings without a compact copy: the FP32 evaluator per vector
    for (int32_t v = 0; v < count; ++v) {
      const sb_status s = sbh::energy_i64(p, spins + (size_t)v * n, out + v, 0);
      if (s != SB_OK) return s;
    }
    return SB_OK;
  }
  const int nt = std::max(1, std::min<int>(count, (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency()))));
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t)
    th.emplace_back([&, t] {
      for (int32_t v = t; v < count; v += nt) out[v] = c.energy(spins + (size_t)v * n, 1);
    });
  for (int32_t v = 0; v < count; v += nt) out[v] = c.energy(spins + (size_t)v * n, 1);
  for (auto &x : th) x.join();
  return SB_OK;
}

extern "C" double sb_energy_f64(const sb_problem *p, const int8_t *spins) {
  if (!p || !p->J || !spins || p->n <= 0) return 0.0;
  const int n = p->n;
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    const float *Ji = p->J + (size_t)i * n;
    double row = 0.0;
    for (int j = i + 1; j < n; ++j) row += (double)Ji[j] * (double)spins[j];
    e -= row * (double)spins[i];
    if (p->h) e -= (double)p->h[i] * (double)spins[i];
  }
  return e;
}

// ---------------------------------------------------------------------------------------------
// Problem bookkeeping.

std::string sbh::device_status_text(uint32_t status) {
  std::string t = "device status " + std::to_string(status);
  if (status & sbk::kErrWaitTimeout) t += " (a bounded wait timed out)";
  if (status & sbk::kErrBadShape) t += " (a launch shape did not match its arguments)";
  if (status & sbk::kErrTmemAlloc) t += " (TMEM allocation failed)";
  if (status & sbk::kErrBounds) t += " (a device bounds check failed)";
  return t;
}

// Integrality, max |J| and the edge count of the couplings: branch-free row loops (vectorised), rows
// dealt round-robin to host threads for large n; none of the three depends on the order.
namespace {
// The process-wide worker pool behind sbh::parallel_run: a queue of (loop, index) tasks.
class HostPool;
HostPool *g_pool = nullptr;  // never destroyed: its threads outlive static teardown
std::mutex g_pool_mu;

// A child process made by fork() has none of the parent's worker threads (and may have inherited a
// lock held at the fork): it starts a pool of its own on first use.
void pool_after_fork_child() {
  new (&g_pool_mu) std::mutex();
  g_pool = nullptr;
}

class HostPool {
 public:
  static HostPool &get() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool) {
      static const int registered = pthread_atfork(nullptr, nullptr, pool_after_fork_child);
      (void)registered;
      g_pool = new HostPool();
    }
    return *g_pool;
  }
  int size() const { return (int)workers_.size() + 1; }
  void run(int nt, const std::function<void(int)> &fn) {
    if (nt <= 1 || workers_.empty()) {
      for (int t = 0; t < nt; ++t) fn(t);
      return;
    }
    Loop loop{&fn, nt - 1};
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (int t = 1; t < nt; ++t) queue_.push_back(Task{&loop, t});
    }
    cv_.notify_all();
    fn(0);
    // help with queued tasks (this loop's or another caller's) until this loop's are all done
    for (;;) {
      Task task{nullptr, 0};
      {
        std::unique_lock<std::mutex> lk(mu_);
        if (loop.left == 0) return;
        if (queue_.empty()) {
          done_cv_.wait(lk, [&] { return loop.left == 0 || !queue_.empty(); });
          if (loop.left == 0) return;
          continue;
        }
        task = queue_.front();
        queue_.pop_front();
      }
      execute(task);
    }
  }

 private:
  struct Loop {
    const std::function<void(int)> *fn;
    int left;  // tasks not yet finished (guarded by mu_)
  };
  struct Task {
    Loop *loop;
    int t;
  };
  HostPool() {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned n = std::min(hw, 16u) - 1;
    for (unsigned i = 0; i < n; ++i) workers_.emplace_back([this] { work(); });
  }
  void execute(const Task &task) {
    (*task.loop->fn)(task.t);
    std::lock_guard<std::mutex> lk(mu_);
    if (--task.loop->left == 0) done_cv_.notify_all();
  }
  void work() {
    for (;;) {
      Task task{nullptr, 0};
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !queue_.empty(); });
        task = queue_.front();
        queue_.pop_front();
      }
      execute(task);
    }
  }
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Task> queue_;
  std::vector<std::thread> workers_;
};
}  // namespace

void sbh::parallel_run(int nt, const std::function<void(int)> &fn) { HostPool::get().run(nt, fn); }

int sbh::host_threads(int n) { return n >= 1024 ? HostPool::get().size() : 1; }

void sbh::problem_scan(sb_problem *p) {
  const int n = p->n;
  const int nt = host_threads(n);
  std::vector<int> nonint((size_t)nt, 0);
  std::vector<float> mx((size_t)nt, 0.0f);
  std::vector<int64_t> ed((size_t)nt, 0);
  std::vector<double> sj((size_t)nt, 0.0), sj2((size_t)nt, 0.0);
  auto rows = [&](int t) {
    int bad = 0;
    float m = 0.0f;
    int64_t e = 0;
    int64_t a1 = 0, a2 = 0;
    for (int i = t; i < n; i += nt) {
      const float *Ji = p->J + (size_t)i * n;
      // one pass over the row for integrality, the largest |J| and the nonzero couplings right of
      // the diagonal, in a form the compiler vectorises: |w| < 2^23 is an integer exactly when
      // adding and subtracting 2^23 gives it back, larger floats all are, NaN is not; the maximum
      // runs on the bit patterns of |w| (monotonic for non-negative floats; NaN counts as 0)
      uint32_t rb = 0, rm = 0;
      int32_t re = 0;
      for (int j = 0; j < n; ++j) {
        const float w = Ji[j];
        const float a = fabsf(w);
        const float r = (a + 8388608.0f) - 8388608.0f;
        rb |= (uint32_t)((r != a) & (a < 8388608.0f)) | (uint32_t)(a != a);
        uint32_t u;
        memcpy(&u, &a, sizeof(u));
        u &= (a == a) ? 0xFFFFFFFFu : 0u;
        rm = u > rm ? u : rm;
        re += (int32_t)((j > i) & (w != 0.0f));
      }
      float rmax;
      memcpy(&rmax, &rm, sizeof(rmax));
      // the off-diagonal sums of J and J^2, kept only for integer couplings: exact integer sums
      // (a row sum of |J| < 2^15 stays below 2^31 for n <= 65536); the row is still in L1
      if (rb == 0 && (double)rmax * (double)rmax * (double)n < 2147483648.0) {
        // every partial sum of J^2 fits int32 too (the common case: small integer couplings)
        int32_t s1 = 0, s2 = 0;
        for (int j = 0; j < n; ++j) {
          const int32_t v = (int32_t)Ji[j];
          s1 += v;
          s2 += v * v;
        }
        const int64_t dg = (int64_t)Ji[i];  // the diagonal does not count
        a1 += (int64_t)s1 - dg;
        a2 += (int64_t)s2 - dg * dg;
      } else if (rb == 0 && rmax < 32768.0f) {
        int32_t s1 = 0;
        int64_t s2 = 0;
        for (int j = 0; j < n; ++j) {
          const int32_t v = (int32_t)Ji[j];
          s1 += v;
          s2 += (int64_t)(v * v);
        }
        const int64_t dg = (int64_t)Ji[i];  // the diagonal does not count
        a1 += (int64_t)s1 - dg;
        a2 += s2 - dg * dg;
      } else if (rb == 0 && rmax < 2147483648.0f) {
        for (int j = 0; j < n; ++j) {
          if (j == i) continue;
          const int64_t v = (int64_t)Ji[j];  // integral and below 2^31
          a1 += v;
          a2 += v * v;
        }
      }
      bad |= rb != 0 ? 1 : 0;
      m = rmax > m ? rmax : m;
      e += re;
    }
    nonint[t] = bad;
    mx[t] = m;
    ed[t] = e;
    sj[t] = (double)a1;
    sj2[t] = (double)a2;
  };
  parallel_run(nt, rows);
  bool integral = true;
  double maxabs = 0.0, s1 = 0.0, s2 = 0.0;
  int64_t edges = 0;
  for (int t = 0; t < nt; ++t) {
    integral = integral && !nonint[t];
    maxabs = (double)mx[t] > maxabs ? (double)mx[t] : maxabs;
    edges += ed[t];
    s1 += sj[t];
    s2 += sj2[t];
  }
  if (p->h)
    for (int i = 0; i < n; ++i)
      if (p->h[i] != floorf(p->h[i])) integral = false;
  p->integer_valued = integral ? 1 : 0;
  p->max_abs_j = (int32_t)ceil(maxabs > 2e9 ? 2e9 : maxabs);
  p->n_edges = edges;
  // integer couplings whose sums stay below 2^53 (every partial sum above is then exact): the
  // coupling statistics of the default c0, kept so that no solve reads J again for them
  const bool exact = integral && (double)n * n * maxabs * maxabs < 9.0e15;
  p->stats_valid = exact ? 1 : 0;
  p->sum_j = exact ? (int64_t)s1 : 0;
  p->sum_j2 = exact ? (int64_t)s2 : 0;
}

extern "C" sb_status sb_problem_init(sb_problem *p, int32_t n, const float *J, const float *h) {
  if (!p || !J || n <= 0) return SB_ERR_INVALID_ARG;
  memset(p, 0, sizeof(*p));
  const size_t nn = (size_t)n * (size_t)n;
  p->J = (float *)malloc(nn * sizeof(float));
  if (!p->J) return SB_ERR_OOM;
  memcpy(p->J, J, nn * sizeof(float));
  for (int i = 0; i < n; ++i) p->J[(size_t)i * n + i] = 0.0f;
  if (h) {
    p->h = (float *)malloc((size_t)n * sizeof(float));
    if (!p->h) {
      free(p->J);
      p->J = nullptr;
      return SB_ERR_OOM;
    }
    memcpy(p->h, h, (size_t)n * sizeof(float));
  }
  p->n = n;
  p->lib_owned = 1;
  sbh::problem_scan(p);
  return SB_OK;
}

extern "C" sb_status sb_problem_wrap(sb_problem *p, int32_t n, float *J, float *h) {
  if (!p || !J || n <= 0) return SB_ERR_INVALID_ARG;
  memset(p, 0, sizeof(*p));
  p->n = n;
  p->J = J;
  p->h = h;
  p->lib_owned = 0;
  sbh::problem_scan(p);
  return SB_OK;
}

extern "C" void sb_problem_free(sb_problem *p) {
  if (!p) return;
  if (p->lib_owned) {
    free(p->J);
    free(p->h);
  }
  memset(p, 0, sizeof(*p));
}

// ---------------------------------------------------------------------------------------------
// Graph reader. The reference reads "N" then "%d%d%d" triples until EOF (SB/CUDA_GPU/m2_opt.cu:
// 111-123) into a dense symmetric float matrix; a later line for the same pair wins. This reader
// keeps that, and adds: real weights, "i i h" field lines, an optional edge count in the header,
// 1-based indices, '#' comments, and errors instead of undefined behaviour for bad input.

namespace {

struct Cursor {
  const char *p, *end;
  int line = 1;
};

void skip_space(Cursor &c, bool stop_at_newline) {
  while (c.p < c.end) {
    const char ch = *c.p;
    if (ch == '#') {
      while (c.p < c.end && *c.p != '\n') ++c.p;
      continue;
    }
    if (ch == '\n') {
      if (stop_at_newline) return;
      ++c.line;
      ++c.p;
      continue;
    }
    if (ch == ' ' || ch == '\t' || ch == '\r' || ch == ',') {
      ++c.p;
      continue;
    }
    return;
  }
}

bool is_delim(char ch) {
  return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n' || ch == ',' || ch == '#';
}

bool parse_int(Cursor &c, long long &v) {
  const char *q = c.p;
  bool neg = false;
  if (q < c.end && (*q == '-' || *q == '+')) neg = (*q++ == '-');
  if (q >= c.end || *q < '0' || *q > '9') return false;
  long long acc = 0;
  while (q < c.end && *q >= '0' && *q <= '9') {
    acc = acc * 10 + (*q - '0');
    if (acc > (1LL << 40)) return false;
    ++q;
  }
  if (q < c.end && !is_delim(*q)) return false;
  v = neg ? -acc : acc;
  c.p = q;
  return true;
}

bool parse_num(Cursor &c, double &v) {
  long long iv;
  Cursor save = c;
  if (parse_int(c, iv)) {
    v = (double)iv;
    return true;
  }
  c = save;
  char buf[64];
  size_t len = 0;
  while (c.p + len < c.end && !is_delim(c.p[len]) && len < sizeof(buf) - 1) {
    buf[len] = c.p[len];
    ++len;
  }
  if (len == 0) return false;
  buf[len] = 0;
  char *e = nullptr;
  v = strtod(buf, &e);
  if (e != buf + len || !isfinite(v)) return false;
  c.p += len;
  return true;
}

// One edge line: indices clamped to int32 (anything outside [-1, 2^30] is out of range for every
// N <= 65536 either way; the true extremes are kept per chunk for the index-base rule), the weight
// as the float J stores, the chunk-local line number.
struct Triple {
  int32_t i, j;
  float w;
  int32_t line;
};
inline int32_t clamp_index(long long v) {
  return (int32_t)std::min<long long>(std::max<long long>(v, -1), 1 << 30);
}

}  // namespace

sb_status sbh::load_graph(const char *path, const sb_graph_opts *opts_in, sb_problem *out,
                          std::string &err) {
  if (!path || !out) return SB_ERR_INVALID_ARG;
  sb_graph_opts opts;
  sb_graph_opts_default(&opts);
  if (opts_in) opts = *opts_in;
  memset(out, 0, sizeof(*out));
  FILE *f = fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open ") + path;
    return SB_ERR_IO;
  }
  std::vector<char> buf;
  {
    // one read of the file's size, then whatever a growing file added
    if (fseek(f, 0, SEEK_END) == 0) {
      const long sz = ftell(f);
      if (sz > 0 && fseek(f, 0, SEEK_SET) == 0) {
        buf.resize((size_t)sz);
        buf.resize(fread(buf.data(), 1, (size_t)sz, f));
      } else {
        fseek(f, 0, SEEK_SET);
        buf.clear();
      }
    }
    char tmp[1 << 16];
    size_t got;
    while ((got = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
    const bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) {
      err = std::string("read error on ") + path;
      return SB_ERR_IO;
    }
  }
  Cursor c{buf.data(), buf.data() + buf.size()};
  skip_space(c, false);
  long long header[2] = {0, -1};
  int nh = 0;
  while (c.p < c.end && *c.p != '\n') {
    long long v;
    if (!parse_int(c, v)) {
      err = "line " + std::to_string(c.line) + ": header must be N or N E";
      return SB_ERR_PARSE;
    }
    if (nh < 2) header[nh] = v;
    ++nh;
    skip_space(c, true);
  }
  if (nh < 1 || nh > 2) {
    err = "header must be N or N E";
    return SB_ERR_PARSE;
  }
  long long n = opts.n_override > 0 ? opts.n_override : header[0];
  if (n <= 0 || n > 65536) {
    err = "N out of range (1..65536): " + std::to_string(n);
    return SB_ERR_PARSE;
  }
  // The edge lines, parsed in chunks that end at line ends (a triple never spans lines) on the host
  // pool. Each chunk keeps its triples in file order with chunk-local line numbers, its first parse
  // error and the newlines it consumed; the fill below walks the chunks in order, so duplicates,
  // conflicts, the index base and every error message are those of one pass over the file.
  struct Chunk {
    const char *b = nullptr, *e = nullptr;
    std::vector<Triple> tr;
    long long min_idx = (1LL << 40), max_idx = -1;
    int lines = 0;     // newlines consumed
    int err_line = 0;  // local line of the first parse error, with err_kind > 0
    int err_kind = 0;  // 1 expected an index, 2 expected 'i j w', 3 indices must be integers
    bool diag = false;  // a line i i h (a field)
  };
  const size_t rest = (size_t)(c.end - c.p);
  const int pool = host_threads(1 << 20);
  const int nchunks = (int)std::max<size_t>(1, std::min<size_t>((size_t)pool * 4, rest / (256 * 1024)));
  std::vector<Chunk> chunks((size_t)nchunks);
  {
    const char *at = c.p;
    for (int k = 0; k < nchunks; ++k) {
      chunks[k].b = at;
      const char *cut = k + 1 == nchunks ? c.end : c.p + rest / nchunks * (size_t)(k + 1);
      if (cut < at) cut = at;
      while (cut < c.end && cut[-1] != '\n') ++cut;  // the chunk ends just after a newline
      chunks[k].e = cut;
      at = cut;
    }
  }
  auto parse_chunk = [&](int k) {
    Chunk &ch = chunks[k];
    Cursor q{ch.b, ch.e, 0};
    for (;;) {
      skip_space(q, false);
      if (q.p >= q.end) break;
      Triple t;
      t.line = q.line;
      double wi, wj, wv;
      if (!parse_num(q, wi)) {
        ch.err_line = q.line;
        ch.err_kind = 1;
        return;
      }
      skip_space(q, true);
      if (q.p >= q.end || *q.p == '\n' || !parse_num(q, wj)) {
        ch.err_line = t.line;
        ch.err_kind = 2;
        return;
      }
      skip_space(q, true);
      if (q.p >= q.end || *q.p == '\n' || !parse_num(q, wv)) {
        ch.err_line = t.line;
        ch.err_kind = 2;
        return;
      }
      if (wi != floor(wi) || wj != floor(wj)) {
        ch.err_line = t.line;
        ch.err_kind = 3;
        return;
      }
      // bounded before the conversion (an index like 1e30 is out of range, not undefined)
      const double lim = (double)(1LL << 41);
      const long long ti = (long long)std::max(-lim, std::min(wi, lim));
      const long long tj = (long long)std::max(-lim, std::min(wj, lim));
      ch.min_idx = std::min(ch.min_idx, std::min(ti, tj));
      ch.max_idx = std::max(ch.max_idx, std::max(ti, tj));
      t.i = clamp_index(ti);
      t.j = clamp_index(tj);
      t.w = (float)wv;
      if (ti == tj) ch.diag = true;
      ch.tr.push_back(t);
    }
    ch.lines = q.line;
  };
  if (nchunks == 1)
    parse_chunk(0);
  else
    parallel_run(nchunks, parse_chunk);
  long long min_idx = (1LL << 40), max_idx = -1;
  bool any = false, diag = false;
  std::vector<int> line0((size_t)nchunks);  // the global line at each chunk's start
  {
    int ln = c.line;
    for (int k = 0; k < nchunks; ++k) {
      const Chunk &ch = chunks[k];
      line0[k] = ln;
      if (ch.err_kind) {
        static const char *const what[4] = {"", "expected an index", "expected 'i j w'",
                                            "indices must be integers"};
        err = "line " + std::to_string(ln + ch.err_line) + ": " + what[ch.err_kind];
        return SB_ERR_PARSE;
      }
      ln += ch.lines;
      if (!ch.tr.empty()) any = true;
      diag = diag || ch.diag;
      min_idx = std::min(min_idx, ch.min_idx);
      max_idx = std::max(max_idx, ch.max_idx);
    }
  }
  std::vector<char>().swap(buf);  // the text is parsed: release it before J is allocated
  int base = opts.index_base;
  if (base < 0) base = (any && max_idx == n && min_idx >= 1) ? 1 : 0;
  const size_t nn = (size_t)n * (size_t)n;
  float *J = (float *)calloc(nn, sizeof(float));
  if (!J) {
    err = "host allocation of J failed";
    return SB_ERR_OOM;
  }
  float *h = nullptr;
  if (diag) {
    h = (float *)calloc((size_t)n, sizeof(float));
    if (!h) {
      free(J);
      err = "host allocation of h failed";
      return SB_ERR_OOM;
    }
  }
  // The fill: thread w owns rows [n w / nt, n (w + 1) / nt) and walks every triple in file order,
  // writing only cells of its rows, so each cell sees its writes (and the strict check its earlier
  // value) in file order. A thread stops at its first error; the earliest line over the threads is
  // the error one pass in file order reports (an index out of range stops every thread there).
  struct FillErr {
    long long line = -1;
    int kind = 0;  // 1 index out of range, 2 conflicting field, 3 conflicting weight
    long long a = 0, b = 0;
  };
  const int nt = nchunks == 1 ? 1 : std::max(1, std::min(host_threads(1 << 20), (int)n));
  std::vector<FillErr> ferr((size_t)nt);
  auto fill = [&](int w) {
    const long long r0 = n * w / nt, r1 = n * (w + 1) / nt;
    FillErr &fe = ferr[w];
    for (int k = 0; k < nchunks; ++k) {
      for (const Triple &t : chunks[k].tr) {
        const long long i = (long long)t.i - base, j = (long long)t.j - base;
        if (i < 0 || j < 0 || i >= n || j >= n) {
          fe = {(long long)line0[k] + t.line, 1, 0, 0};
          return;
        }
        const bool own_i = i >= r0 && i < r1;
        if (i == j) {
          if (own_i) {
            if (opts.strict && h[i] != 0.0f && h[i] != t.w) {
              fe = {(long long)line0[k] + t.line, 2, i, 0};
              return;
            }
            h[i] = t.w;
          }
          continue;
        }
        if (own_i) {
          float &a = J[(size_t)i * n + j];
          if (opts.strict && a != 0.0f && a != t.w) {
            fe = {(long long)line0[k] + t.line, 3, i, j};
            return;
          }
          a = t.w;
        }
        if (j >= r0 && j < r1) J[(size_t)j * n + i] = t.w;
      }
    }
  };
  if (nt == 1)
    fill(0);
  else
    parallel_run(nt, fill);
  const FillErr *first = nullptr;
  for (const FillErr &fe : ferr)
    if (fe.kind && (!first || fe.line < first->line)) first = &fe;
  if (first) {
    free(J);
    free(h);
    const std::string at = "line " + std::to_string(first->line) + ": ";
    if (first->kind == 1)
      err = at + "index out of range for N=" + std::to_string(n);
    else if (first->kind == 2)
      err = at + "conflicting field for spin " + std::to_string(first->a);
    else
      err = at + "conflicting weight for edge " + std::to_string(first->a) + "-" + std::to_string(first->b);
    return SB_ERR_PARSE;
  }
  out->n = (int32_t)n;
  out->J = J;
  out->h = h;
  out->lib_owned = 1;
  problem_scan(out);
  return SB_OK;
}

extern "C" sb_status sb_load_graph_ex(const char *path, const sb_graph_opts *opts,
                                      sb_problem *out) {
  std::string err;
  sb_status s = sbh::load_graph(path, opts, out, err);
  if (s != SB_OK) sbh::set_thread_error(err);
  return s;
}

extern "C" sb_status sb_load_graph(const char *path, sb_problem *out) {
  return sb_load_graph_ex(path, nullptr, out);
}

// ---------------------------------------------------------------------------------------------
// Seeded random instances (Erdos-Renyi G(n, p) with integer or +-1 couplings), generated from a
// counter hash of (seed, i, j) so every row is independent: parallel over host threads and
// identical for any thread count.

namespace {
inline uint64_t mix(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return z;
}
}  // namespace

extern "C" sb_status sb_problem_random(sb_problem *p, int32_t n, double density, int32_t jmax,
                                       int32_t field_max, uint64_t seed) {
  if (!p || n <= 0 || n > 65536 || !(density >= 0.0 && density <= 1.0) || jmax < 1 || field_max < 0)
    return SB_ERR_INVALID_ARG;
  memset(p, 0, sizeof(*p));
  const size_t nn = (size_t)n * (size_t)n;
  p->J = (float *)malloc(nn * sizeof(float));
  if (!p->J) return SB_ERR_OOM;
  if (field_max > 0) {
    p->h = (float *)malloc((size_t)n * sizeof(float));
    if (!p->h) {
      free(p->J);
      p->J = nullptr;
      return SB_ERR_OOM;
    }
  }
  const uint64_t thr = density >= 1.0 ? ~0ULL : (uint64_t)(density * 18446744073709551616.0);
  const unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  std::vector<std::thread> th;
  for (unsigned w = 0; w < nt; ++w)
    th.emplace_back([=] {
      for (int i = (int)w; i < n; i += (int)nt) {
        float *Ji = p->J + (size_t)i * n;
        Ji[i] = 0.0f;
        for (int j = i + 1; j < n; ++j) {
          const uint64_t z = mix(seed * 0x9E3779B97F4A7C15ULL + ((uint64_t)i << 32) + (uint64_t)j + 1);
          float w8 = 0.0f;
          if (density >= 1.0 || mix(z ^ 0x5851F42D4C957F2DULL) < thr) {
            if (jmax == 1)
              w8 = (z & 1) ? 1.0f : -1.0f;
            else
              w8 = (float)((int64_t)(z % (uint64_t)(2 * jmax + 1)) - jmax);
          }
          Ji[j] = w8;
        }
      }
    });
  for (auto &t : th) t.join();
  // lower triangle from the upper one
  th.clear();
  for (unsigned w = 0; w < nt; ++w)
    th.emplace_back([=] {
      for (int i = (int)w; i < n; i += (int)nt) {
        float *Ji = p->J + (size_t)i * n;
        for (int j = 0; j < i; ++j) Ji[j] = p->J[(size_t)j * n + i];
      }
    });
  for (auto &t : th) t.join();
  if (p->h)
    for (int i = 0; i < n; ++i) {
      const uint64_t z = mix(seed * 0xD1B54A32D192ED03ULL + (uint64_t)i + 7);
      p->h[i] = (float)((int64_t)(z % (uint64_t)(2 * field_max + 1)) - field_max);
    }
  p->n = n;
  p->lib_owned = 1;
  sbh::problem_scan(p);
  return SB_OK;
}
