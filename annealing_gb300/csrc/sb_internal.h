// Internal declarations shared by the host library (sb_api.cpp) and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sb.h"

namespace sbk {

// Error bits a kernel ORs into its status word instead of trapping.
enum : uint32_t {
  kErrWaitTimeout = 1u,     // a bounded mbarrier / flag wait gave up
  kErrBadShape = 2u,        // launch shape does not match the arguments
  kErrTmemAlloc = 4u,       // TMEM allocation failed
  kErrBounds = 8u,          // a checked build found an index outside its buffer (the access was skipped)
};

// Bounds checks of the checked build (-DSB_CHECKS, the debug stand-in for a memory sanitizer): a
// failing check records kErrBounds in the status word and the guarded access is skipped. In the
// normal build the condition is not evaluated and the access is unconditional.
#ifdef SB_CHECKS
#define SB_BOUNDS(cond, status) ((cond) ? true : (atomicOr((status), sbk::kErrBounds), false))
#else
#define SB_BOUNDS(cond, status) true
#endif

// Row pitch (elements) of the padded state and coupling layouts.
inline int pitch_for(int n, int align) { return (n + align - 1) / align * align; }

// ---------------------------------------------------------------------------------------------
// Plain FP32 path: one fused launch per SB step.
// Layouts: J [n][jp] float (row pitch jp, zero padded); x, y [R][xp] float (replica-major).
struct PlainStep {
  int variant;             // 0 aSB, 1 bSB, 2 dSB
  int n, R, jp, xp, rb;    // rb: replicas per CTA (grid.y = ceil(R / rb))
  const float *J, *h;      // h may be null
  const float *x_in;
  float *x_out, *y;        // y is updated in place (each element has one owner)
  float pump, c0, dt, dta0;            // bSB / dSB
  float coeff, amp_next, mts_dt, detune, kerr;  // aSB kick and the next step's local update
  int m, do_local;
  double *energy;          // [R] energy of s(x_in) (dSB only; may be null)
  uint32_t *status;
  // 1: launched with programmatic stream serialization, so the launch overlaps the previous
  // kernel's tail (J must not be written by that kernel: J copies start before the wait for it)
  int overlap;
  int stages;              // set by launch_plain_step
};

// Plain FP32 SB, the whole solve in one cooperative launch (sb_plain.cu): CTA (c, r) keeps rows
// [16 c, 16 c + 16) of J in registers (one row per warp; a lane holds the float4 groups g = lane +
// 32 k, which is the per-step kernel's summation order) and replica r's x, y of those rows. A step
// exchanges through one 128-byte line per CTA at words[parity][r][c]: dSB one word (step tag << 32 |
// 16 sign bits), bSB / aSB / NMFA sixteen (step tag << 32 | bits of x or of the state s). Eligible
// when jp <= kPersistMaxJp and G R CTAs (G = ceil(n / 16)) are co-resident.
struct PlainPersist {
  int variant;                // 0 aSB, 1 bSB (x exchanged), 2 dSB (signs exchanged), 3 NMFA (states exchanged)
  int n, R, jp, xp;
  const float *J, *h;         // J [n][jp], h [n] or null
  const float *x_in;          // x(0) [R][xp]
  float *x_out, *y;           // x(steps) (may alias x_in), y in place
  const float *pumps;         // [steps] a0 - a(t)
  float c0, dt, dta0;
  float coeff, mts_dt, detune, kerr;  // aSB kick and local sub-steps
  int m;
  int steps;
  unsigned long long *words;  // [2][R][G] words, one per 128-byte line (16 x 8 bytes), zero on entry
  uint32_t *status;
  // NMFA (variant 3): x holds the states s, pumps[t] the beta of sweep t (two sweeps per stage),
  // norm [n] the row norms, rng [5][R][xp] the XORWOW words (read at the start, written at the end),
  // samples [R][n] receives sign(s) after the last sweep (or null)
  const float *norm;
  uint32_t *rng;
  int32_t *samples;
  float noise, keep, mix;
};
constexpr int kPersistRows = 16;
constexpr int kPersistMaxJp = 2048;
// Number of CTAs (G R) of the persistent launch, or 0 when this shape does not qualify.
int plain_persist_ctas(int n, int R, int jp);
cudaError_t launch_plain_persist(const PlainPersist &a, cudaStream_t st);

struct PlainEnergy {
  int n, R, jp, xp, rb;
  const float *J, *h;
  const float *x;
  double *energy;          // [R] += energy of s(x)
  uint32_t *status;
  int stages;              // set by launch_plain_energy
};

// One NMFA sweep (noisy mean-field annealing, NMFA/CUDA_GPU/src/nmfa.cu:99-136) over every sample:
// the field J s through the plain kernel's rows machinery, then per (sample, spin)
// s' = keep s + mix tanh(beta (norm_i f_i + z)). sb_plain.cu.
struct NmfaSweep {
  int n, R, jp, xp, rb;    // R samples, rb samples per CTA
  const float *J;          // [n][jp]
  const float *norm;       // [n]: -1 / sqrt(sum_j |J_ij|), 0 for an empty row
  const float *s_in;       // [R][xp] states before the sweep (padding 0)
  float *s_out;            // [R][xp] states after it
  uint32_t *rng;           // [5][R][xp] XORWOW words of each (sample, spin)
  float *z1;               // [R][xp] the stage's second Gaussian sample
  int32_t *samples;        // [R][n] receives sign(s') as +-1 (the last sweep), or null
  float beta, noise, keep, mix;  // keep = 1 - recombination, mix = recombination
  int first;               // 1: first sweep of a stage, which draws the stage's two samples
  uint32_t *status;
  int overlap;             // as PlainStep::overlap
  int stages;              // set by launch_nmfa_sweep
};

// Sets kernel attributes (dynamic shared memory limits) once per process; call before any capture.
void init_kernel_attributes();
cudaError_t launch_nmfa_sweep(const NmfaSweep &a, cudaStream_t st);
// The NMFA row norms -1 / sqrt(sum_j |J_ij|) from the padded couplings [n][jp]; integral: every
// coupling an integer with n max|J| < 2^53 (the sum is then exact in any order).
cudaError_t launch_nmfa_norms(const float *J, int n, int jp, float *norm, bool integral, cudaStream_t st);
// samples[r][i] = +-1 from the signs of the states [R][xp].
cudaError_t launch_nmfa_signs(const float *s, int n, int R, int xp, int32_t *samples, cudaStream_t st);
// Initial XORWOW words of every (sample, spin); rng as in NmfaSweep.
cudaError_t launch_nmfa_seed(uint32_t *rng, int n, int R, int xp, uint32_t seed, cudaStream_t st);
cudaError_t launch_plain_step(const PlainStep &a, cudaStream_t st);
cudaError_t launch_plain_energy(const PlainEnergy &a, bool fp64, cudaStream_t st);

// Initial state, elementwise helpers.
cudaError_t launch_init_uniform(float *x, float *y, int n, int R, int xp, uint64_t seed,
                                cudaStream_t st);
cudaError_t launch_init_reference(float *x, float *y, int n, int R, int xp, cudaStream_t st);
cudaError_t launch_asb_local(float *x, float *y, int n, int R, int xp, float amp, int m,
                             float mts_dt, float detune, float kerr, cudaStream_t st);
// Copy a dense host-layout J [n][n] (already on the device) into the padded [n][jp] FP32 layout.
cudaError_t launch_pad_rows_f32(const float *src, float *dst, int n, int jp, cudaStream_t st);

// ---------------------------------------------------------------------------------------------
// Tensor-core (tcgen05) path. See sb_tc.cu.
enum TcDtype : int { kTcFp8 = 1, kTcBf16 = 2, kTcBf16Split = 3, kTcFp4 = 4, kTcFp16Split = 5 };
// Operands split in a high and a low part (real-valued couplings): BF16 hi + lo, or FP16 hi + lo
// with power-of-two scaling.
#if defined(__CUDACC__)
__host__ __device__
#endif
constexpr bool tc_split(int dt) { return dt == kTcBf16Split || dt == kTcFp16Split; }

struct TcPlanInfo;  // opaque, defined in sb_tc.cu
}  // namespace sbk
