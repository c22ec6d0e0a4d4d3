// Internal host-side declarations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "sb.h"

namespace sbh {
// Runs fn(0) .. fn(nt - 1) on the calling thread and on a process-wide pool of host worker threads
// (created on first use, kept until exit, so a short parallel loop pays no thread start-up), and
// returns when all have finished. Safe to call from several threads at once; a caller waiting for
// its own tasks runs queued ones meanwhile.
void parallel_run(int nt, const std::function<void(int)> &fn);
// Host threads worth using for an n x n pass (1 below n = 1024), at most the pool's size.
int host_threads(int n);
void problem_scan(sb_problem *p);
sb_status load_graph(const char *path, const sb_graph_opts *opts, sb_problem *out,
                     std::string &err);
void set_thread_error(const std::string &e);
const char *thread_error();
// sb_energy_i64 / sb_coupling_std / sb_default_c0 on a given number of host threads (0: as many as
// pay for the size, up to 8); callers that already run one instance per thread pass 1.
sb_status energy_i64(const sb_problem *p, const int8_t *spins, int64_t *out, int threads);
double coupling_std(const sb_problem *p, int threads);
float default_c0(const sb_problem *p, int threads);
// The default c0 from the off-diagonal sums of J and J^2 (exact integers below 2^53): the value
// default_c0 computes for those couplings.
float c0_from_sums(int n, int64_t s, int64_t s2);

// Exact compact copy of integer couplings for the host int64 energy re-check, which otherwise
// reads the FP32 matrix: couplings in {-1, 0, +1} as two bit planes (row i, bit j: J_ij != 0,
// J_ij < 0; N^2 / 4 bytes, row sums by popcount), |J| <= 127 as int8 (N^2 bytes). The energy is
// the same integer sb_energy_i64 gives.
struct CouplingCopy {
  int n = 0;
  int mode = 0;  // kNone, kBits, kInt8
  int words = 0;  // 64-bit words per bit-plane row
  std::vector<uint64_t> nz, neg;
  std::vector<int32_t> upper;  // bit planes: nonzero couplings right of the diagonal, per row
  std::vector<int8_t> j8;
  std::vector<int64_t> h;  // empty: no field
  static constexpr int kNone = 0, kBits = 1, kInt8 = 2;
  // false (mode kNone) when a coupling or field is not integral or |J| > 127, or on `cancel`
  bool build(const sb_problem *p, const std::atomic<bool> *cancel = nullptr);
  int64_t energy(const int8_t *spins, int threads) const;
};

// Copies of several problems built on background threads (problem k on thread k % threads, in
// order), so that a solve's device time hides the build; a problem whose copy is not ready yet is
// evaluated from its FP32 couplings.
class CouplingCopies {
 public:
  explicit CouplingCopies(std::vector<const sb_problem *> probs, int threads = 1);
  ~CouplingCopies();  // stops the builder and joins it
  sb_status energy(size_t k, const int8_t *spins, int64_t *out, int threads) const;
  bool ready(size_t k) const;

 private:
  std::vector<const sb_problem *> probs_;
  std::vector<CouplingCopy> copies_;
  std::unique_ptr<std::atomic<int>[]> ready_;
  std::atomic<bool> cancel_{false};
  std::vector<std::thread> th_;
};
}  // namespace sbh

struct NmfaCache;
namespace sbh {
// "device status S (...)": the status word of a kernel run, its bits spelled out.
std::string device_status_text(uint32_t status);
// Frees an NMFA buffer cache (sb_nmfa.cpp); null is a no-op.
void nmfa_cache_free(NmfaCache *c);
}  // namespace sbh

namespace sbk {

// Tensor-core field engine for one dense instance with R replicas (sb_tc.cu).
struct TcEngine;

struct TcSetup {
  int variant;  // 1 bSB, 2 dSB, 3 NMFA
  int dtype;    // TcDtype
  int n, R;
  int xp;       // pitch of the x / y state rows (floats)
};

// Builds the tensor-core operand form of J from the padded FP32 J on the device ([n][jp]).
sb_status tc_create(TcEngine **out, const TcSetup &s, const float *dJ, int jp, std::string &err,
                    cudaStream_t st);
void tc_destroy(TcEngine *e);
// Re-converts new couplings (same n) into an existing engine's J operand.
cudaError_t tc_reload(TcEngine *e, const float *dJ, int jp, cudaStream_t st);
int64_t tc_footprint(const TcSetup &s);
// True when the packed-E2M1 kernel runs this shape (dSB, its units fit the SMs and a unit's J rows
// fit shared memory).
bool tc_fp4_fits(int n, int R);
// Builds the step-0 operand (sign(x) or x hi/lo) from the initial state.
cudaError_t tc_prepare(TcEngine *e, const float *x, cudaStream_t st);
// The whole step loop in one persistent cooperative launch: x / y live in TMEM between steps,
// the operand ping-pongs between buffers 0 and 1 (step t reads t & 1). energy_trace (may be
// null, dSB only): slot t (R doubles) += energy of s(t), t = 0 .. steps-1.
// pumps: device array, pumps[t] = a0 - a(t) for t = 0 .. steps-1.
cudaError_t tc_run(TcEngine *e, int steps, const float *pumps, float *x, float *y, const float *h,
                   float c0, float dt, float dta0, double *energy_trace, uint32_t *status,
                   cudaStream_t st);
// NMFA (TcSetup::variant 3, BF16 operands): `sweeps` sweeps in one persistent launch; s [R][xp] the
// states (in and out), z1 [R][xp] the stage's second noise sample, norm [n] the row norms, betas
// [sweeps] the inverse temperature of each sweep (both sweeps of a stage repeat it), rng [5][R][xp]
// the XORWOW words; the operand must hold s (tc_prepare) on entry.
cudaError_t tc_run_nmfa(TcEngine *e, int sweeps, const float *betas, float *s, float *z1, const float *norm,
                        uint32_t *rng, float noise, float keep, float mix, uint32_t *status, cudaStream_t st);
// Engines with BF16 or BF16 hi + lo couplings (NMFA, bSB, dSB with real J): energy[r] += the energy of
// sign(x_r), -1/2 s J s - h s, for every replica (the dSB energy contraction on the engine's
// couplings; exact for integer J and h); overwrites operand buffer 0.
cudaError_t tc_energy_signs(TcEngine *e, const float *x, const float *h, double *energy, uint32_t *status,
                            cudaStream_t st);
int tc_units(const TcEngine *e);
int tc_replica_tile(const TcEngine *e);
// Field-only pass on operand buffer (t & 1): energy of s(t) per replica (dSB, integer J).
cudaError_t tc_energy(TcEngine *e, int t, const float *x, const float *h, double *energy,
                      uint32_t *status, cudaStream_t st);
int tc_dtype(const TcEngine *e);
// Limit of every bounded wait in the engine's kernels (SM clock cycles; <= 0: the default, about
// one second), and the fault injection for the timeout path: skip_step >= 0 makes unit 0 leave
// out its step-skip_step flag, so its column's waits run out (skip_step < 0: off).
void tc_set_waits(TcEngine *e, long long wait_cycles, int skip_step);

// dSB on E2M1 or FP8 operands over buffers the caller provides; allocates nothing.
struct TcExternal {
  const float *J;   // device couplings, row pitch jp floats
  int jp;
  const float *h;   // device fields or null
  int n, R, xp;
  float *x, *y;     // device state [R][xp]: initial in, final out
  bool fp4;         // packed E2M1 operands (integers |J| <= 4, tc_fp4_fits) instead of FP8
  uint8_t *a;       // J operand, tc_external_sizes() a_bytes
  uint8_t *v0, *v1; // operand buffers, v_bytes each, zero on entry
  uint32_t *flags;  // flags_bytes (cleared by the solve itself)
  uint32_t *status; // one status word, outside the flag bytes
  const float *pumps;          // [steps]
  int steps;
  float c0, dt, dta0;
  double *energy;   // [R] final energies, zero on entry
};
// Buffer sizes of the external dSB solve; false when the shape has no single-pass kernel.
bool tc_external_sizes(int n, int R, bool fp4, size_t *a_bytes, size_t *v_bytes, size_t *flags_bytes);
cudaError_t tc_dsb_external(const TcExternal &ext, cudaStream_t st);

}  // namespace sbk
