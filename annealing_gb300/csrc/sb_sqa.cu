// Fully-connected simulated quantum annealing (SQA) on one GB300: sb_sqa_solve.
//
// The algorithm is the reference's GPU SQA, SQA_fully/fully_test/pre_calculate.cu: M Trotter
// slices of N spins, a diagonal wavefront of M + N - 1 iterations per annealing step in which slice
// m updates spin (a - m) mod N (:63, :221-224), the local field sum_i J[target][i] s[m][i] (its
// reduce kernel, :99-149), the energy change 2 M s (f - M J_perp (s[m-1] + s[m+1])) (:73-77) and the
// Metropolis test -log(u) / beta > delta (:79-81), the schedule of :206-225, and the slice-0 energy
// after each step (:230-236). The reference runs two launches per wavefront iteration (a
// block-reduce over all of J's rows for the M targets, then one block of M threads for the test).
//
// Here one CTA runs one replica (one of the reference's TIMES trials) for the whole anneal:
//   * the M x N spins live in shared memory as bits (bit 1 = spin -1), slice-major;
//   * J lives in global memory (L2-resident) as bit-planes per row: per 32-coupling word a sign
//     word (1 where J_ij < 0) and P magnitude words (bit k-1 of |J_ij|), then the row's sum of
//     |J_ij|. A field is sum_i J_i s_i = rowabs - 2 sum_k 2^(k-1) popc(mag_k & (sign ^ spin)):
//     32 couplings per XOR / AND / POPC, exact integers (P templated: one 8-byte load per word for
//     +-1 couplings);
//   * the wavefront needs rows a - M + 1 .. a at iteration a; they stream through a ring of
//     M + D row slots in shared memory by 1-D bulk copies (cp.async.bulk + mbarrier), D rows ahead,
//     so a row is read from L2 once per use window instead of M times;
//   * a group of 8 lanes sums one slice's field (4 slices per warp); the group's first lane makes
//     the slice's decision against a threshold -log(u) / beta made ahead of time (per step and
//     spin in reference mode, whose random word per spin is fixed; per chunk of iterations in hash
//     mode); one __syncthreads per iteration orders the flips before the next iteration's fields;
//   * slot and slice strides are padded (16 and 8 or 16 words mod 32) so the four groups of a warp
//     read different banks, and a ring shallow enough for two CTAs per SM is preferred.
// No two slices of one iteration touch the same spin, and a slice's Trotter neighbours read other
// spins than the ones it flips (M <= N), so the CTA reproduces the reference's iteration semantics
// exactly. The acceptance log is this library's own (sbm::log_unit, sb_math.cuh; the oracle carries the
// same function), so host and device results are bit-identical.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "sb.h"
#include "sb_ctx.h"
#include "sb_host.h"
#include "sb_internal.h"
#include "sb_math.cuh"
#include "sb_ptx.cuh"

namespace {

constexpr int kSqaMaxWarps = 32;
constexpr int kSqaAhead = 8;                 // rows the ring streams ahead of the wavefront
constexpr size_t kSqaSmemBudget = 220 * 1024;
constexpr size_t kSqaSmemHalf = 112 * 1024;  // two CTAs per SM (228 KB, less static and reserved)

struct SqaArgs {
  const uint32_t *rows;   // [n][RW]: sign plane [W], P magnitude planes [W] each, rowabs, 3 pad words
  uint32_t *spins;        // [R][M][W] bits, in: initial state, out: final state
  const uint32_t *rnd;    // [R][n] reference-mode random words, or null (hash mode)
  const float *beta;      // [steps]
  const float *jperp;     // [steps]
  int64_t *energy;        // [R][steps] (trace) or [R] (final): slice-0 energy
  uint32_t *status;
  uint64_t seed;
  int n, W, P, RW, M, steps, S, trace;
  int RS, SPS;            // shared-memory strides of a ring slot and of a slice (bank-spread padding)
};

__device__ __forceinline__ uint64_t sqa_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Field of `row` against slice bits `sm`, summed over the warp (every lane gets it). A row stores,
// per 32-coupling word w, the sign word then the P magnitude words (row[w (P + 1) + k]), and the
// row's sum of |J| after the W groups.
template <int P>
__device__ __forceinline__ int sqa_field(const uint32_t *row, const uint32_t *sm, int W, int lane) {
  int acc = 0;
#pragma unroll 4
  for (int w = lane; w < W; w += 32) {
    const uint32_t *g = row + (size_t)w * (P + 1);
    uint32_t v[P + 1];
    if constexpr (P == 1) {
      const uint2 t = *reinterpret_cast<const uint2 *>(g);
      v[0] = t.x;
      v[1] = t.y;
    } else if constexpr (P == 3) {
      const uint4 t = *reinterpret_cast<const uint4 *>(g);
      v[0] = t.x;
      v[1] = t.y;
      v[2] = t.z;
      v[3] = t.w;
    } else {
#pragma unroll
      for (int k = 0; k <= P; ++k) v[k] = g[k];
    }
    const uint32_t x = v[0] ^ sm[w];
#pragma unroll
    for (int k = 1; k <= P; ++k) acc += __popc(v[k] & x) << (k - 1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return (int)row[(size_t)W * (P + 1)] - 2 * acc;
}

// The same field computed by a group of G lanes (G a power of two dividing 32): lane gl of the
// group takes words gl, gl + G, ...; a group that has no slice (row == nullptr) contributes 0 and
// still joins the shuffles. Every lane of the group gets the group's field.
template <int P, int G>
__device__ __forceinline__ int sqa_field_group(const uint32_t *row, const uint32_t *sm, int W, int gl) {
  int acc = 0;
  if (row && P == 1) {
    // +-1 couplings: word pairs, one 16-byte load of (sign, magnitude) x 2 and one 8-byte load of
    // the two spin words (W is a multiple of 4)
#pragma unroll 4
    for (int w = 2 * gl; w < W; w += 2 * G) {
      const uint4 t = *reinterpret_cast<const uint4 *>(row + (size_t)w * 2);
      const uint2 sv = *reinterpret_cast<const uint2 *>(sm + w);
      acc += __popc(t.y & (t.x ^ sv.x)) + __popc(t.w & (t.z ^ sv.y));
    }
  } else if (row) {
#pragma unroll 4
    for (int w = gl; w < W; w += G) {
      const uint32_t *g = row + (size_t)w * (P + 1);
      uint32_t v[P + 1];
      if constexpr (P == 1) {
        const uint2 t = *reinterpret_cast<const uint2 *>(g);
        v[0] = t.x;
        v[1] = t.y;
      } else if constexpr (P == 3) {
        const uint4 t = *reinterpret_cast<const uint4 *>(g);
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
      } else {
#pragma unroll
        for (int k = 0; k <= P; ++k) v[k] = g[k];
      }
      const uint32_t x = v[0] ^ sm[w];
#pragma unroll
      for (int k = 1; k <= P; ++k) acc += __popc(v[k] & x) << (k - 1);
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return row ? (int)row[(size_t)W * (P + 1)] - 2 * acc : 0;
}

// Acceptance threshold -log(u) / beta of the reference's test (pre_calculate.cu:79), with this
// library's log.
__device__ __forceinline__ float sqa_threshold(float u, float beta) { return __fdiv_rn(-sbm::log_unit(u), beta); }

constexpr int kSqaChunk = 16;  // wavefront iterations whose hash-mode thresholds are made at once
constexpr int kSqaGroup = 8;   // lanes per slice in the field sums
constexpr int kSqaSlicesPerWarp = 32 / kSqaGroup;

template <int P>
__global__ void __launch_bounds__(kSqaMaxWarps * 32, 1) sqa_kernel(const __grid_constant__ SqaArgs p) {
  extern __shared__ __align__(128) uint8_t smem[];
  const int RW = p.RW, W = p.W, M = p.M, n = p.n, S = p.S, RS = p.RS, SPS = p.SPS;
  // slot stride RS = 16 (mod 32) words and slice stride SPS = 8 or 16 (mod 32): the four lane groups
  // of a warp read four slots / slices whose words fall in different banks
  uint32_t *ring = reinterpret_cast<uint32_t *>(smem);      // [S][RS] (RW words used)
  uint32_t *sp = ring + (size_t)S * RS;                      // [M][SPS] (W words used)
  float *thr = reinterpret_cast<float *>(sp + (size_t)M * SPS);  // [n] (reference) or [kSqaChunk][M] (hash)
  const size_t thr_words = p.rnd ? (size_t)n : (size_t)kSqaChunk * M;
  uint64_t *bar = reinterpret_cast<uint64_t *>(thr + ((thr_words + 3) & ~(size_t)3));  // [S]
  __shared__ long long ered[kSqaMaxWarps];
  __shared__ int abort_sh;

  const int r = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
  const int iters = M + n - 1;
  const long long per_step = (long long)n + 2 * M - 2;  // rows streamed per step: a - m for a in [0, iters), m in [0, M)
  const long long total = per_step * p.steps;
  const uint32_t row_bytes = (uint32_t)RW * 4u;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) sbk::ptx::mbar_init(&bar[s], 1);
    sbk::ptx::fence_mbar_init();
    abort_sh = 0;
  }
  for (int k = tid; k < M * W; k += blockDim.x) sp[(k / W) * SPS + k % W] = p.spins[(size_t)r * M * W + k];
  __syncthreads();

  // Stream index q -> row ((q mod per_step) - (M - 1)) mod n, slot q mod S, slot use (lap) q / S.
  // Every index below is kept by increments (no division in the loop): the issuer's position, and
  // per iteration the newest row's slot / lap (slice 0) and a mod n.
  long long issued = 0;
  int iss_slot = 0, iss_pos = 0;
  const int row_first = (n - (M - 1) % n) % n;  // row of stream position 0 within a step
  int iss_row = row_first;
  auto issue_upto = [&](long long last) {  // thread 0 only
    if (last >= total) last = total - 1;
    // a slot is rewritten only after the __syncthreads that ended the last iteration reading it
    // (a write after reads: the barrier orders them, no proxy fence)
    for (; issued <= last; ++issued) {
      sbk::ptx::mbar_arrive_expect_tx(&bar[iss_slot], row_bytes);
      if (SB_BOUNDS(iss_row >= 0 && iss_row < n && iss_slot < S, p.status))
        sbk::ptx::bulk_g2s(ring + (size_t)iss_slot * RS, p.rows + (size_t)iss_row * RW, row_bytes, &bar[iss_slot]);
      if (++iss_slot == S) iss_slot = 0;
      if (++iss_pos == per_step) {
        iss_pos = 0;
        iss_row = row_first;
      } else if (++iss_row == n) {
        iss_row = 0;
      }
    }
  };
  const int D = S - M;
  if (tid == 0) issue_upto((long long)M - 1 + D);

  bool ok = true;
  long long q0 = M - 1;         // stream index of slice 0's row in the current iteration
  int slot0 = M - 1, lap0 = 0;  // q0 mod S, q0 / S (M - 1 < S)
  for (int st = 0; st < p.steps && ok; ++st) {
    const float beta = p.beta[st], jp = p.jperp[st];
    const float mj = __fmul_rn((float)M, jp);
    const uint64_t e_step = ((uint64_t)r * p.steps + st) * (uint64_t)iters * (uint64_t)M;  // hash index of (a = 0, m = 0)
    if (p.rnd) {
      // reference mode: every spin keeps one random word, so a step's thresholds are one per spin
      for (int i = tid; i < n; i += blockDim.x)
        thr[i] = sqa_threshold(__fdiv_rn(__uint2float_rn(p.rnd[(size_t)r * n + i]), 4294967296.0f), beta);
      __syncthreads();
    }
    int t0 = 0, ci = 0;  // a mod n, a mod kSqaChunk
    for (int a = 0; a < iters; ++a) {
      if (!p.rnd && ci == 0) {
        // hash mode: thresholds of iterations a .. a + kSqaChunk - 1 (every slice) at once; the
        // previous chunk's last readers finished before the barrier that ended its iteration
        const int cnt = min(kSqaChunk, iters - a) * M;
        for (int k = tid; k < cnt; k += blockDim.x) {
          const uint64_t e = e_step + (uint64_t)a * M + (uint64_t)k;  // (a + k / M) M + k % M
          const uint64_t z = sqa_mix64((p.seed ^ 0xD1B54A32D192ED03ULL) + 0x9E3779B97F4A7C15ULL * (e + 1));
          thr[k] = sqa_threshold(__fmul_rn((float)(uint32_t)(z >> 40), 0x1p-24f), beta);
        }
        __syncthreads();
      }
      if (tid == 0 && a + st > 0) issue_upto(q0 + D);
      // fields: lane group lane / kSqaGroup of warp w takes slice w * kSqaSlicesPerWarp + group
      {
        const int m = warp * kSqaSlicesPerWarp + lane / kSqaGroup, gl = lane % kSqaGroup;
        const bool have = m < M;
        int slot = slot0 - m, lap = lap0;  // stream index q0 - m
        if (slot < 0) {
          slot += S;
          lap -= 1;
        }
        // one verdict per warp: the field's shuffles need every lane
        const bool got = have ? sbk::ptx::mbar_wait(&bar[slot], (uint32_t)(lap & 1)) : true;
        if (!__all_sync(0xffffffffu, got)) {
          atomicOr(p.status, sbk::kErrWaitTimeout);
          abort_sh = 1;
        } else {
          const int f = sqa_field_group<P, kSqaGroup>(have ? ring + (size_t)slot * RS : nullptr,
                                                      sp + (size_t)(have ? m : 0) * SPS, W, gl);
          if (have && gl == 0) {
            // the group's first lane decides slice m (pre_calculate.cu:73-81)
            const int target = t0 - m < 0 ? t0 - m + n : t0 - m;  // (a - m) mod n, m < n
            const uint32_t wi = (uint32_t)target >> 5, bi = 1u << (target & 31);
            const int up = m == 0 ? M - 1 : m - 1, lo = m == M - 1 ? 0 : m + 1;
            const int s = (sp[(size_t)m * SPS + wi] & bi) ? -1 : 1;
            const int nb = ((sp[(size_t)up * SPS + wi] & bi) ? -1 : 1) + ((sp[(size_t)lo * SPS + wi] & bi) ? -1 : 1);
            const float inner = __fsub_rn((float)f, __fmul_rn(mj, (float)nb));
            // the reference forms 2 M s * inner in double (pre_calculate.cu:76-77); that product is
            // exact (|2 M s| <= 256 times a 24-bit significand), so rounding it to float is one
            // correctly rounded float multiply: the same value without the (slow) FP64 pipe
            const float delta = __fmul_rn((float)(2 * M * s), inner);
            const float th = p.rnd ? thr[target] : thr[ci * M + m];
            if (th > delta) sp[(size_t)m * SPS + wi] ^= bi;
          }
        }
      }
      __syncthreads();
      if (abort_sh) {
        ok = false;
        break;
      }
      // next iteration: q0 + 1, a + 1
      ++q0;
      if (++slot0 == S) {
        slot0 = 0;
        ++lap0;
      }
      if (++t0 == n) t0 = 0;
      if (++ci == kSqaChunk) ci = 0;
    }
    // the next step starts at stream index base + per_step + M - 1: M - 1 past where the loop ended
    q0 += M - 1;
    slot0 += M - 1;
    if (slot0 >= S) {
      slot0 -= S;
      ++lap0;
    }
    if (!ok) break;
    // slice-0 energy: E = -1/2 sum_i s_i f_i, rows read from global memory
    if (p.trace || st == p.steps - 1) {
      long long acc = 0;
      for (int i = warp; i < n; i += nw) {
        const int f = sqa_field<P>(p.rows + (size_t)i * RW, sp, W, lane);
        acc += ((sp[i >> 5] >> (i & 31)) & 1u) ? -(long long)f : (long long)f;
      }
      if (lane == 0) ered[warp] = acc;
      __syncthreads();
      if (tid == 0) {
        long long t = 0;
        for (int w = 0; w < nw; ++w) t += ered[w];
        p.energy[p.trace ? (size_t)r * p.steps + st : (size_t)r] = -t / 2;
      }
    }
    // the next step's reference thresholds overwrite thr only after every decision of this one
    __syncthreads();
  }
  if (!ok && tid == 0) {
    // every issued copy completes before the CTA's shared memory goes away
    for (long long q = issued - 1; q >= 0 && q >= issued - S; --q)
      sbk::ptx::mbar_wait(&bar[q % S], (uint32_t)((q / S) & 1));
  }
  __syncthreads();
  if (ok)
    for (int k = tid; k < M * W; k += blockDim.x) p.spins[(size_t)r * M * W + k] = sp[(k / W) * SPS + k % W];
}

// Initial slices as bits [R][M][W]. Reference mode (pre_calculate.cu:38-51, :186-191, :213): spin i
// keeps one xorshift32 state seeded with i; replica r takes calls r M + 1 .. (r + 1) M for its
// slices and keeps the state after them as the spin's random word. Hash mode: one counter hash per
// (replica, slice, spin). One thread per spin, one ballot per 32 spins.
__global__ void sqa_init_kernel(uint32_t *spins, uint32_t *rnd, int n, int W, int M, int R, int mode,
                                uint64_t seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // grid covers W * 32 threads
  const bool in = i < n;
  uint32_t st = (uint32_t)i;
  for (int r = 0; r < R; ++r) {
    for (int m = 0; m < M; ++m) {
      bool neg;
      if (mode == 0) {
        uint32_t x = st;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        st = x;
        neg = (x & 1u) == 0u;  // ((x & 1) << 1) - 1 == -1
      } else {
        const uint64_t e = ((uint64_t)r * M + m) * n + i;
        neg = (sqa_mix64(seed + 0x9E3779B97F4A7C15ULL * (e + 1)) >> 63) != 0;
      }
      const uint32_t word = __ballot_sync(0xffffffffu, in && neg);
      if ((threadIdx.x & 31) == 0 && i < W * 32) spins[((size_t)r * M + m) * W + (i >> 5)] = word;
    }
    if (mode == 0 && in) rnd[(size_t)r * n + i] = st;
  }
}

// Bit-plane rows of J ([n][n] FP32 integers, |J| < 2^P) into [n][RW]: per 32-coupling word the sign
// word then the P magnitude words, the row's sum of |J| after them; one thread per word.
__global__ void sqa_rows_kernel(const float *J, int n, int W, int P, int RW, uint32_t *rows) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n * W) return;
  const int i = (int)(t / W), w = (int)(t % W);
  uint32_t sign = 0, mag[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int abs_sum = 0;
  for (int b = 0; b < 32; ++b) {
    const int j = w * 32 + b;
    if (j >= n || j == i) continue;
    const int v = (int)J[(size_t)i * n + j];
    const int a = v < 0 ? -v : v;
    if (v < 0) sign |= 1u << b;
    for (int k = 0; k < P; ++k)
      if ((a >> k) & 1) mag[k] |= 1u << b;
    abs_sum += a;
  }
  uint32_t *row = rows + (size_t)i * RW;
  row[(size_t)w * (P + 1)] = sign;
  for (int k = 0; k < P; ++k) row[(size_t)w * (P + 1) + k + 1] = mag[k];
  // the row's sum of |J| (warps of one row reduce through an atomic; the word starts at 0)
  atomicAdd(&row[(P + 1) * W], (uint32_t)abs_sum);
}

// The kernel for P magnitude planes (|J| < 2^P, P <= 7).
const void *sqa_kernel_for(int P) {
  switch (P) {
    case 1: return reinterpret_cast<const void *>(&sqa_kernel<1>);
    case 2: return reinterpret_cast<const void *>(&sqa_kernel<2>);
    case 3: return reinterpret_cast<const void *>(&sqa_kernel<3>);
    case 4: return reinterpret_cast<const void *>(&sqa_kernel<4>);
    case 5: return reinterpret_cast<const void *>(&sqa_kernel<5>);
    case 6: return reinterpret_cast<const void *>(&sqa_kernel<6>);
    default: return reinterpret_cast<const void *>(&sqa_kernel<7>);
  }
}

// cudaLaunchKernel argument array for a kernel taking one SqaArgs by value
void **args_of(SqaArgs &a) {
  static thread_local void *ptr[1];
  ptr[0] = &a;
  return ptr;
}

sb_status fail(sb_ctx *ctx, sb_status s, const std::string &msg) {
  ctx->last_error = msg;
  return s;
}

}  // namespace

extern "C" void sb_sqa_params_default(sb_sqa_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->trotter = 16;   // SQA_fully/fully_test/sqa.c:13 (pre_calculate.cu:16 uses 64)
  p->steps = 100;    // pre_calculate.cu:15
  p->replicas = 1;   // pre_calculate.cu:12 (TIMES)
  p->rng_mode = SB_SQA_RNG_HASH;
  p->seed = 1234;
}

// pre_calculate.cu:206-207, :210, :218-219, :225 (host arithmetic in the types the reference uses)
extern "C" void sb_sqa_schedule(int32_t steps, int32_t trotter, float *beta_out, float *jperp_out) {
  if (steps <= 0 || trotter <= 0 || !beta_out || !jperp_out) return;
  const float increase = (8 - 1 / (float)16) / (float)steps;
  const float G0 = 8.;
  float beta = 1 / (float)16;
  for (int p = 0; p < steps; ++p) {
    const float Gamma = (float)(G0 * (1. - (double)((float)p / (float)steps)));
    const float J_perp = (float)(-0.5 * (double)logf(tanhf((Gamma / (float)trotter) * beta)) / (double)beta);
    beta_out[p] = beta;
    jperp_out[p] = J_perp;
    beta += increase;
  }
}

extern "C" sb_status sb_sqa_solve(sb_ctx *ctx, const sb_problem *prob, const sb_sqa_params *prm,
                                  sb_sqa_result *res) {
  if (!ctx || !prob || !prm || !res || !prob->J) return SB_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  const auto t0 = std::chrono::steady_clock::now();
  const int n = prob->n, M = prm->trotter, R = prm->replicas, steps = prm->steps;
  if (n < 2 || M < 1 || M > 128 || M > n || R < 1 || steps < 1 ||
      (prm->rng_mode != SB_SQA_RNG_REFERENCE && prm->rng_mode != SB_SQA_RNG_HASH))
    return fail(ctx, SB_ERR_INVALID_ARG, "sb_sqa_solve: needs n >= 2, 1 <= trotter <= min(n, 128), replicas >= 1, "
                                         "steps >= 1 and a known rng_mode");
  if (!prob->integer_valued || prob->max_abs_j > 127)
    return fail(ctx, SB_ERR_UNSUPPORTED, "sb_sqa_solve: couplings must be integers with |J| <= 127 "
                                         "(the reference stores them as char)");
  if (prob->h)
    for (int i = 0; i < n; ++i)
      if (prob->h[i] != 0.0f)
        return fail(ctx, SB_ERR_UNSUPPORTED, "sb_sqa_solve: fields are not supported (the reference has none)");
  cudaSetDevice(ctx->device);
  int P = 1;
  while ((1 << P) <= prob->max_abs_j) ++P;
  const int W = (((n + 31) / 32) + 3) / 4 * 4;
  const int RW = (P + 1) * W + 4;
  const size_t spin_words = (size_t)M * W;
  // thresholds: one per spin (reference mode) or per (iteration, slice) of a chunk (hash mode)
  const size_t thr_words = ((prm->rng_mode == SB_SQA_RNG_REFERENCE ? (size_t)n : (size_t)kSqaChunk * M) + 3) & ~(size_t)3;
  // shared-memory strides: a slot of RS = 16 (mod 32) words; a slice of SPS = 16 (mod 32) words for
  // the word-pair loads of +-1 couplings, 8 (mod 32) otherwise
  const int RS = RW + ((16 - RW % 32) + 32) % 32;
  const int SPS = W + (((P == 1 ? 16 : 8) - W % 32) + 32) % 32;
  const size_t sp_words = (size_t)M * SPS;
  // ring slots: the M rows of one iteration plus up to kSqaAhead rows ahead; the deepest ring that
  // lets two CTAs (two replicas) share an SM, else the deepest that fits one
  int S = 0;
  for (size_t budget : {kSqaSmemHalf, kSqaSmemBudget})
    for (int d = kSqaAhead; d >= 2 && S == 0; --d) {
      const size_t bytes = (size_t)(M + d) * RS * 4 + sp_words * 4 + thr_words * 4 + (size_t)(M + d) * 8;
      if (bytes <= budget) S = M + d;
    }
  if (S == 0) return fail(ctx, SB_ERR_UNSUPPORTED, "sb_sqa_solve: trotter x n too large for one CTA's shared memory");
  const size_t smem = (size_t)S * RS * 4 + sp_words * 4 + thr_words * 4 + (size_t)S * 8;
  const int threads = 32 * ((M + kSqaSlicesPerWarp - 1) / kSqaSlicesPerWarp);
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  float *dJ = nullptr, *dbeta = nullptr, *djp = nullptr;
  uint32_t *drows = nullptr, *dspins = nullptr, *drnd = nullptr, *dstatus = nullptr;
  int64_t *den = nullptr;
  const size_t en_count = prm->trace ? (size_t)R * steps : (size_t)R;
  std::vector<float> hbeta((size_t)steps), hjp((size_t)steps);
  sb_sqa_schedule(steps, M, hbeta.data(), hjp.data());
  std::vector<int64_t> hen(en_count);
  std::vector<uint32_t> hbits;
  uint32_t hstatus = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float dev_ms = 0.0f;
  std::string where;
  sb_status out = SB_OK;
#define SQ_CUDA(call)                 \
  if ((e = (call)) != cudaSuccess) {  \
    where = #call;                    \
    goto cleanup;                     \
  }
  SQ_CUDA(cudaFuncSetAttribute(sqa_kernel_for(P), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SQ_CUDA(cudaEventCreate(&ev0));
  SQ_CUDA(cudaEventCreate(&ev1));
  SQ_CUDA(cudaMallocAsync((void **)&dJ, (size_t)n * n * sizeof(float), st));
  SQ_CUDA(cudaMallocAsync((void **)&drows, (size_t)n * RW * sizeof(uint32_t), st));
  SQ_CUDA(cudaMallocAsync((void **)&dspins, (size_t)R * spin_words * sizeof(uint32_t), st));
  if (prm->rng_mode == SB_SQA_RNG_REFERENCE) SQ_CUDA(cudaMallocAsync((void **)&drnd, (size_t)R * n * sizeof(uint32_t), st));
  SQ_CUDA(cudaMallocAsync((void **)&dbeta, (size_t)steps * sizeof(float), st));
  SQ_CUDA(cudaMallocAsync((void **)&djp, (size_t)steps * sizeof(float), st));
  SQ_CUDA(cudaMallocAsync((void **)&den, en_count * sizeof(int64_t), st));
  SQ_CUDA(cudaMallocAsync((void **)&dstatus, sizeof(uint32_t), st));
  SQ_CUDA(cudaMemcpyAsync(dJ, prob->J, (size_t)n * n * sizeof(float), cudaMemcpyHostToDevice, st));
  SQ_CUDA(cudaMemcpyAsync(dbeta, hbeta.data(), (size_t)steps * sizeof(float), cudaMemcpyHostToDevice, st));
  SQ_CUDA(cudaMemcpyAsync(djp, hjp.data(), (size_t)steps * sizeof(float), cudaMemcpyHostToDevice, st));
  SQ_CUDA(cudaMemsetAsync(drows, 0, (size_t)n * RW * sizeof(uint32_t), st));
  SQ_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(uint32_t), st));
  SQ_CUDA(cudaEventRecord(ev0, st));
  {
    const long long nt = (long long)n * W;
    sqa_rows_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(dJ, n, W, P, RW, drows);
    SQ_CUDA(cudaGetLastError());
    sqa_init_kernel<<<(W * 32 + 127) / 128, 128, 0, st>>>(dspins, drnd, n, W, M, R,
                                                          prm->rng_mode == SB_SQA_RNG_REFERENCE ? 0 : 1, prm->seed);
    SQ_CUDA(cudaGetLastError());
    SqaArgs a;
    a.rows = drows;
    a.spins = dspins;
    a.rnd = drnd;
    a.beta = dbeta;
    a.jperp = djp;
    a.energy = den;
    a.status = dstatus;
    a.seed = prm->seed;
    a.n = n;
    a.W = W;
    a.P = P;
    a.RW = RW;
    a.M = M;
    a.steps = steps;
    a.S = S;
    a.RS = RS;
    a.SPS = SPS;
    a.trace = prm->trace ? 1 : 0;
    SQ_CUDA(cudaLaunchKernel(sqa_kernel_for(P), dim3((unsigned)R), dim3((unsigned)threads), args_of(a), smem, st));
    SQ_CUDA(cudaGetLastError());
  }
  SQ_CUDA(cudaEventRecord(ev1, st));
  SQ_CUDA(cudaMemcpyAsync(hen.data(), den, en_count * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaMemcpyAsync(&hstatus, dstatus, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaStreamSynchronize(st));
  if (hstatus) {
    out = (hstatus & sbk::kErrWaitTimeout) ? SB_ERR_TIMEOUT : SB_ERR_CUDA;
    ctx->last_error = "sb_sqa_solve: " + sbh::device_status_text(hstatus);
    goto cleanup_noerr;
  }
  SQ_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
  {
    std::vector<double> fin((size_t)R);
    for (int r = 0; r < R; ++r) fin[r] = (double)hen[prm->trace ? (size_t)r * steps + steps - 1 : (size_t)r];
    int best = 0;
    for (int r = 1; r < R; ++r)
      if (fin[r] < fin[best]) best = r;
    const bool all = res->final_spins != nullptr;
    hbits.resize(all ? (size_t)R * spin_words : spin_words);
    SQ_CUDA(cudaMemcpyAsync(hbits.data(), dspins + (all ? 0 : (size_t)best * spin_words),
                            hbits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SQ_CUDA(cudaStreamSynchronize(st));
    const uint32_t *b0 = hbits.data() + (all ? (size_t)best * spin_words : 0);
    std::vector<int8_t> spins((size_t)n);
    for (int i = 0; i < n; ++i) spins[i] = ((b0[i >> 5] >> (i & 31)) & 1u) ? -1 : 1;
    if (all)
      for (int r = 0; r < R; ++r)
        for (int m = 0; m < M; ++m)
          for (int i = 0; i < n; ++i)
            res->final_spins[((size_t)r * M + m) * n + i] =
                ((hbits[((size_t)r * M + m) * W + (i >> 5)] >> (i & 31)) & 1u) ? -1 : 1;
    if (res->best_spins) memcpy(res->best_spins, spins.data(), (size_t)n);
    if (res->replica_energies) memcpy(res->replica_energies, fin.data(), (size_t)R * sizeof(double));
    if (res->energy_trace && prm->trace)
      for (size_t k = 0; k < en_count; ++k) res->energy_trace[k] = (double)hen[k];
    int64_t ei = 0;
    res->energy_check_ok = (sb_energy_i64(prob, spins.data(), &ei) == SB_OK && (double)ei == fin[best]) ? 1 : 0;
    res->best_energy_i64 = ei;
    res->best_energy = fin[best];
    res->best_replica = best;
    res->device_ms = dev_ms;
    res->kernel_launches = 3;
    const double updates = (double)R * M * (double)(n + M - 1) * steps;
    res->spin_updates_per_s = dev_ms > 0 ? updates / ((double)dev_ms * 1e-3) : 0.0;
  }
  goto cleanup_noerr;
cleanup:
  out = e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  ctx->last_error = std::string("sb_sqa_solve: ") + where + ": " + cudaGetErrorString(e);
cleanup_noerr:
  cudaFreeAsync(dJ, st);
  cudaFreeAsync(drows, st);
  cudaFreeAsync(dspins, st);
  if (drnd) cudaFreeAsync(drnd, st);
  cudaFreeAsync(dbeta, st);
  cudaFreeAsync(djp, st);
  cudaFreeAsync(den, st);
  cudaFreeAsync(dstatus, st);
  cudaStreamSynchronize(st);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
#undef SQ_CUDA
  if (out == SB_OK) res->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return out;
}
