// Tensor-core (tcgen05) SB kernel: the field J*V for R replicas as a GEMM on the 5th-generation
// tensor cores, with the SB update fused into the epilogue.
//
// Replaces the reference's per-step field call (cublasSgemv, SB/CUDA_GPU/m2_opt.cu:169; the
// tensor-op GEMM form cublasSgemm(N,1,N) of SB/CUDA_GPU/m2_opt2.cu:155-163; the FP16 form
// cublasHgemm of SB/CUDA_GPU/m2_opt3.cu:161-162) by a contraction over all replicas at once:
//     F[i][r] = sum_k J[i][k] * V[r][k],   V = sign(x) (dSB) or x (bSB).
//
// Kernel structure (one persistent cooperative launch for the whole solve):
//   * the work is tiled into units of 128 spins (TMEM lanes, MMA M) x NR replicas (MMA N); each
//     CTA owns one unit for every step, so its x and y live in TMEM for the whole solve
//     (columns [NR, 2NR) and [2NR, 3NR); the FP32 accumulator is columns [0, NR));
//   * warp 0 (one lane) streams J tiles and V tiles with 2-D TMA into 128-byte-swizzled shared
//     memory through a STAGES-deep mbarrier ring; warp 1 (one lane) issues tcgen05.mma
//     (kind::f8f6f4 for FP8 E4M3 operands, kind::f16 for BF16), committing each stage back to the
//     producer and the finished accumulator to the epilogue;
//   * warps 2..9 (two per TMEM lane quadrant, each half of the replica columns) read the
//     accumulator, x and y with tcgen05.ld, apply the SB update with the exact operation order of
//     the CPU oracle, write x and y back to TMEM and the next step's operand V (sign as FP8/BF16,
//     or x as BF16 hi + lo) to global memory; the accumulator is double-buffered in TMEM so the
//     next contraction can start while the epilogue drains (split operands instead accumulate K in
//     segments, each folded by the epilogue into an FP32 sum rounded to nearest);
//   * steps are ordered by per-unit release/acquire flags instead of a grid barrier: a unit
//     publishes its V(t+1) chunk and the units of its replica column wait only for the chunks they
//     load (bounded spins).
// VARIANT 3 is NMFA (noisy mean-field annealing, NMFA/CUDA_GPU/src/nmfa.cu:99-136) on the same
// pipeline: x holds the mean-field state s, y the stage's second Gaussian sample, h the row norms,
// pumps[t] the inverse temperature of sweep t; the operand is s as BF16 hi + lo against exact BF16
// couplings; the epilogue applies the NMFA update and draws each stage's noise pair (XORWOW words
// in rng) a stage ahead into TMEM, or on the stage's first sweep when the extra columns do not fit.
// Operand dtypes: FP8 E4M3 holds +-1 and integers |J| <= 16 exactly; BF16 holds integers up to 256;
// BF16 hi + lo (J = Jh + Jl, x = xh + xl) gives ~16 bits for real values, with the three products
// Jh*xh + Jh*xl + Jl*xh accumulated in FP32. Integer fields are exact whenever every partial sum
// stays below 2^24 in magnitude, which holds for n * max|J| < 2^24.
// Every wait is bounded; a timeout sets a status bit, the kernel still frees its TMEM and returns.
// tcgen05 SB kernel template (shared by the per-dtype instantiation files and the host engine).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sb_internal.h"
#include "sb_math.cuh"
#include "sb_ptx.cuh"

namespace sbk {
namespace tck {

constexpr int kEmodeStep = 0, kEmodeStepTrace = 1, kEmodeEnergy = 2;
constexpr int kEpiWarps = 8;     // two per TMEM lane quadrant
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kEpiFirstThread = 64;
constexpr int kTcThreads = 64 + kEpiThreads;  // producer warp, MMA warp, epilogue warps
constexpr int kBM = 128;         // spins per unit (MMA M, TMEM lanes)
constexpr int kChunkBytes = 128; // K bytes per stage (one 128-byte swizzle atom row)

struct alignas(64) TcArgs {
  CUtensorMap tmA[2];      // J operand parts: [Np rows][Kp] K-major
  CUtensorMap tmB[2][2];   // V operand [buffer][part]: [Rp rows][Kp] K-major
  CUtensorMap tmS[2];      // V operand [buffer], part 0, unswizzled 128-spin x NR boxes (TMA store)
  float *x, *y;            // [R][xp] state (read at start, written at the end)
  const float *h;          // [n] or null
  uint8_t *v[2][2];        // V operand [buffer][part] base pointers (bytes)
  double *energy;          // trace: [(steps + 1) * R] (step t -> slot t) or energy pass: [R]
  uint32_t *status;
  uint32_t *flags;         // [n_rtiles][n_mtiles] published step counters (zeroed before launch)
  int n, R, xp, Kp, Rp, n_mtiles, n_rtiles, k_chunks;
  int steps, t0;           // steps to run; schedule offset
  int buf0;                // V buffer holding V(t0)
  const float *pumps;      // pumps[t] = a0 - a(t), computed on the host (NMFA: beta of sweep t)
  float c0, dt, dta0;
  uint32_t *rng;           // NMFA: [5][R][xp] XORWOW words of each (sample, spin)
  float noise, keep, mix;  // NMFA: sigma, 1 - alpha, alpha
  long long wait_cycles;   // limit of every bounded wait (SM clock cycles)
  int seg_chunks;          // split operands: K chunks per accumulation segment
  int flag_stride;         // words between consecutive units' flags (32: one 128-byte line each)
  float jinv, xscale;      // FP16 hi + lo: J was scaled by 1 / jinv and x is scaled by xscale (powers of two)
  // host-side fault injection for the timeout path: unit skip_unit does not publish its flag(s)
  // of step skip_step (skip_step < 0: every unit publishes)
  int skip_unit, skip_step;
};

template <int DT>
struct DtTraits;
template <>
struct DtTraits<kTcFp8> {
  static constexpr int kElem = 1, kParts = 1;
};
template <>
struct DtTraits<kTcBf16> {
  static constexpr int kElem = 2, kParts = 1;
};
template <>
struct DtTraits<kTcBf16Split> {
  static constexpr int kElem = 2, kParts = 2;
};
template <>
struct DtTraits<kTcFp16Split> {
  static constexpr int kElem = 2, kParts = 2;
};

template <int DT, int VARIANT>
struct Cfg {
  static constexpr int kElem = DtTraits<DT>::kElem;
  static constexpr int kAParts = DtTraits<DT>::kParts;
  // V = sign(x) needs one part even when J is split; bSB's x is split with J; NMFA's state is split
  // against exact (integer) BF16 couplings.
  static constexpr int kBParts = ((tc_split(DT) && VARIANT == 1) || VARIANT == 3) ? 2 : 1;
  static constexpr int kKPerMma = 32 / kElem;  // 32 bytes of K per instruction
  static constexpr int kMmaPerChunk = kChunkBytes / 32;
};

__host__ __device__ constexpr uint32_t make_idesc(int dt, int m, int n) {
  // D = F32 (bits 4-5 = 1); A/B format: E4M3 = 0 (kind::f8f6f4), F16 = 0 or BF16 = 1 (kind::f16);
  // both K-major; N >> 3 at bits 17-22; M >> 4 at bits 24-28.
  return (1u << 4) | ((dt == kTcBf16 || dt == kTcBf16Split ? 1u : 0u) << 7) |
         ((dt == kTcBf16 || dt == kTcBf16Split ? 1u : 0u) << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

// +1 / -1 in a 16-bit operand type
template <int DT>
__host__ __device__ constexpr uint16_t one16(bool neg) {
  return DT == kTcFp16Split ? (neg ? (uint16_t)0xBC00 : (uint16_t)0x3C00) : (neg ? (uint16_t)0xBF80 : (uint16_t)0x3F80);
}

__device__ __forceinline__ float sgnf(float v) { return v > 0.0f ? 1.0f : -1.0f; }

__device__ __forceinline__ void sb_update(float f, float hv, float pump, float c0, float dt,
                                          float dta0, float &x, float &y) {
  const float fv = __fadd_rn(f, hv);
  const float g = __fmul_rn(c0, fv);
  const float force = __fmaf_rn(-pump, x, g);
  y = __fmaf_rn(dt, force, y);
  x = __fmaf_rn(dta0, y, x);
  if (fabsf(x) > 1.0f) {
    x = copysignf(1.0f, x);
    y = 0.0f;
  }
}

// Write element (r, i) of the next operand (FP16 hi + lo: x scaled by xscale, a power of two).
template <int DT, int VARIANT>
__device__ __forceinline__ void store_operand(uint8_t *const (&vb)[2], size_t idx, float x, float xscale) {
  if constexpr (DT == kTcFp8) {
    vb[0][idx] = x > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;  // E4M3 +1 / -1
  } else if constexpr (Cfg<DT, VARIANT>::kBParts == 1) {
    reinterpret_cast<uint16_t *>(vb[0])[idx] = one16<DT>(!(x > 0.0f));
  } else if constexpr (DT == kTcFp16Split) {
    const float xs = __fmul_rn(x, xscale);
    const __half hi = __float2half_rn(xs);
    const __half lo = __float2half_rn(__fsub_rn(xs, __half2float(hi)));
    reinterpret_cast<__half *>(vb[0])[idx] = hi;
    reinterpret_cast<__half *>(vb[1])[idx] = lo;
  } else {
    const __nv_bfloat16 hi = __float2bfloat16_rn(x);
    const __nv_bfloat16 lo = __float2bfloat16_rn(__fsub_rn(x, __bfloat162float(hi)));
    reinterpret_cast<__nv_bfloat16 *>(vb[0])[idx] = hi;
    reinterpret_cast<__nv_bfloat16 *>(vb[1])[idx] = lo;
  }
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Named barrier over the epilogue warps only (the producer and MMA lanes never join it).
__device__ __forceinline__ void epi_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
}

// AND of a predicate over the epilogue warps (a named-barrier reduction), so that they all leave a
// loop together and never strand one another at a later named barrier.
__device__ __forceinline__ bool epi_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)(v ? 1 : 0)), "n"(kEpiThreads)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Bounded wait until a unit's published step counter reaches `target`. Polls with relaxed loads
// (an acquire load per poll would order, and slow, everything else on this SM) and backs off;
// the acquire fence is taken once the flag is seen.
__device__ __forceinline__ bool wait_flag(const uint32_t *flag, uint32_t target, long long limit) {
  if (ld_relaxed(flag) < target) {
    const long long t0 = clock64();
    while (ld_relaxed(flag) < target) {
      if (clock64() - t0 > limit) return false;
      __nanosleep(64);
    }
  }
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  return true;
}

// One persistent launch runs `steps` SB steps. Unit (mt, rt) = spins [128 mt, 128 mt + 128) x
// replicas [NR rt, NR rt + NR). Step t's contraction needs V(t) for the unit's replica tile over
// all K, i.e. the chunks the units (*, rt) of the same replica column wrote at the end of step
// t - 1: each unit publishes flags[rt][mt] = t after writing its chunk, and the producer waits for
// flags[rt][chunk's unit] >= t before loading that chunk. Those same flags also order the reuse of
// the ping-pong operand buffer (a unit overwrites V(t+1)'s buffer only after consuming all of V(t),
// i.e. after every reader of V(t-1)'s chunk finished its step t-1 contraction).
template <int DT, int VARIANT, int NR, int STAGES, int EMODE>
__global__ void __launch_bounds__(kTcThreads, 1) tc_sb_kernel(const __grid_constant__ TcArgs p) {
  using C = Cfg<DT, VARIANT>;
  constexpr int kATile = kBM * kChunkBytes;  // bytes per A part per stage
  constexpr int kBTile = NR * kChunkBytes;   // bytes per B part per stage
  constexpr int kStage = C::kAParts * kATile + C::kBParts * kBTile;
  // Single-part operands (FP8 / BF16 signs) leave the epilogue through a shared-memory tile and one
  // TMA store per unit per step; split operands are stored element by element.
  constexpr bool kStageV = C::kBParts == 1;
  constexpr int kVRow = kBM * C::kElem;      // bytes of one replica row of the unit's V tile
  constexpr uint32_t kTx = (uint32_t)kStage;
  // NMFA draws stage k+1's noise pair ahead, in the idle time after stage k's sweeps publish (the
  // first chunk of a thread's columns after the first sweep, the rest after the second), when three
  // more column blocks fit TMEM (z0, and z1 alternating between y and y1 by stage parity);
  // otherwise on the stage's first sweep
  constexpr bool kNoiseAhead = VARIANT == 3 && 6 * NR <= 512;
  constexpr int kUsedCols = kNoiseAhead ? 6 * NR : 4 * NR;
  constexpr uint32_t kCols = kUsedCols <= 32 ? 32 : (kUsedCols <= 64 ? 64 : (kUsedCols <= 128 ? 128 : (kUsedCols <= 256 ? 256 : 512)));
  constexpr uint32_t kIdesc = make_idesc(DT, kBM, NR);
  constexpr int kHalf = NR / 2;               // columns per epilogue warp
  // Split couplings (BF16 hi + lo, real-valued J): the tensor core rounds the sum of each MMA into
  // its FP32 accumulator toward zero, a bias that grows with the number of MMAs one accumulator
  // takes and with its magnitude. So the contraction over K runs in segments of p.seg_chunks chunks,
  // each into a fresh accumulator (column block 0), and the epilogue warps, idle during the
  // contraction, load each finished segment (the MMA lane waits only for that load) and add it into
  // a running FP32 sum (round to nearest; column block 1). x and y keep blocks 2 and 3.
  constexpr bool kSeg = tc_split(DT);
  // FP16 hi + lo: the accumulated field is scaled back by an exact power of two
  const float fscale = DT == kTcFp16Split ? (C::kBParts == 2 ? p.jinv / p.xscale : p.jinv) : 1.0f;
  static_assert(NR % 32 == 0 && NR >= 32 && NR <= 128, "replica tile");
  static_assert(4 * NR <= 512, "two accumulators + x + y must fit TMEM");

  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accf_bar[2], acce_bar[2], drain_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float ered[4][NR];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % p.n_mtiles, rt = blockIdx.x / p.n_mtiles;
  const int m0 = mt * kBM, r0 = rt * NR;
  constexpr bool kEOnly = EMODE == kEmodeEnergy;   // one contraction, energies only
  constexpr bool want_e = EMODE != kEmodeStep;      // per-replica energies of s(t)
  const int nsteps = kEOnly ? 1 : p.steps;
  uint32_t *col_flags = p.flags + (size_t)rt * p.n_mtiles * p.flag_stride;
  bool ok = true;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&accf_bar[b], 1);
      ptx::mbar_init(&acce_bar[b], kEpiWarps);
    }
    ptx::mbar_init(&drain_bar, 1);
    ptx::fence_mbar_init();
    for (int a = 0; a < C::kAParts; ++a) ptx::prefetch_tmap(&p.tmA[a]);
    for (int b = 0; b < C::kBParts; ++b) {
      ptx::prefetch_tmap(&p.tmB[0][b]);
      ptx::prefetch_tmap(&p.tmB[1][b]);
    }
  }
  if (warp == 1) {
    ptx::tmem_alloc(&tmem_base_sh, kCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  // columns: accumulators [0, NR) and [NR, 2NR), x [2NR, 3NR), y [3NR, 4NR); NMFA with the noise
  // drawn ahead: z0 [4NR, 5NR), y1 [5NR, 6NR) (stage k's z1 in y for even k, in y1 for odd k)
  const uint32_t t_x = tmem + 2 * NR, t_y = tmem + 3 * NR, t_z0 = tmem + 4 * NR, t_y1 = tmem + 5 * NR;
  const uint32_t t_sum = tmem + NR;  // split operands: the running sum of the segments
  const int nseg = kSeg ? (p.k_chunks + p.seg_chunks - 1) / p.seg_chunks : 1;

  if (warp == 0) {
    // ---------------- TMA producer (lane 0 issues; the warp polls the column's flags) ----------------
    // Every lane runs the same loop and meets the others only at warp-collective points, so a
    // lane that gives up on a wait never strands the rest.
    uint32_t g = 0;  // chunks issued so far (the MMA lane counts identically)
    int pre = 0;     // chunks of the coming step whose J part is already in flight
    uint32_t armed = 0;  // stage uses whose barrier lane 0 has armed (loads in flight or landed)
    for (int ls = 0; ls < nsteps && ok; ++ls) {
      const int buf = (p.buf0 + ls) & 1;
      int ready = ls == 0 ? p.n_mtiles : 0;  // units of this column known to have published V(ls)
      for (int kc = 0; kc < p.k_chunks && ok; ++kc, ++g) {
        const int kx = kc * (kChunkBytes / C::kElem);
        if (kx / kBM >= ready) {
          // poll the next 32 units of the column at once (one L2 round trip for all of them)
          const int u = ready + lane;
          const bool fl = u < p.n_mtiles ? wait_flag(col_flags + (size_t)u * p.flag_stride, (uint32_t)ls, p.wait_cycles) : true;
          if (!__all_sync(0xffffffffu, fl)) ok = false;
          ready = ready + 32 < p.n_mtiles ? ready + 32 : p.n_mtiles;
          ptx::fence_proxy_async_global();
        }
        if (lane == 0 && ok) {
          const int s = g % STAGES;
          const uint32_t use = g / STAGES;
          uint8_t *st = smem + s * kStage;
          bool issue = true;
          if (kc >= pre) {
            if (use > 0 && !ptx::mbar_wait(&empty_bar[s], (use - 1) & 1, p.wait_cycles)) {
              ok = false;
              issue = false;
            } else {
              ptx::mbar_arrive_expect_tx(&full_bar[s], kTx);
              for (int a = 0; a < C::kAParts; ++a)
                ptx::tma_load_2d(st + a * kATile, &p.tmA[a], kx, m0, &full_bar[s]);
              armed = g + 1;
            }
          }
          if (issue)
            for (int b = 0; b < C::kBParts; ++b)
              ptx::tma_load_2d(st + C::kAParts * kATile + b * kBTile, &p.tmB[buf][b], kx, r0, &full_bar[s]);
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
      // J does not change between steps: start the next step's first J tiles now.
      pre = 0;
      if (lane == 0 && ok && ls + 1 < nsteps) {
        const int npre = p.k_chunks < STAGES ? p.k_chunks : STAGES;
        for (int kc = 0; kc < npre; ++kc) {
          const uint32_t gg = g + kc;
          const int s = gg % STAGES;
          const uint32_t use = gg / STAGES;
          if (use > 0 && !ptx::mbar_wait(&empty_bar[s], (use - 1) & 1, p.wait_cycles)) {
            ok = false;
            break;
          }
          ptx::mbar_arrive_expect_tx(&full_bar[s], kTx);
          for (int a = 0; a < C::kAParts; ++a)
            ptx::tma_load_2d(smem + s * kStage + a * kATile, &p.tmA[a], kc * (kChunkBytes / C::kElem), m0,
                             &full_bar[s]);
          armed = gg + 1;
          ++pre;
        }
      }
      pre = __shfl_sync(0xffffffffu, pre, 0);
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    }
    if (!ok && lane == 0) {
      // a wait gave up: let the copies this CTA started land before it exits (each stage's last
      // armed use; a use whose J part alone was started never completes its phase, and the
      // bounded wait then outlasts those loads)
      for (int s = 0; s < STAGES; ++s)
        if (armed > (uint32_t)s) ptx::mbar_wait(&full_bar[s], ((armed - 1 - s) / STAGES) & 1, p.wait_cycles);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      uint32_t g = 0;
      uint32_t gs = 0;  // split operands: segments issued
      for (int ls = 0; ls < nsteps && ok; ++ls) {
        const int ab = ls & 1;
        if constexpr (!kSeg) {
          if (ls >= 2 && !ptx::mbar_wait(&acce_bar[ab], (uint32_t)((ls >> 1) - 1) & 1, p.wait_cycles)) { ok = false; break; }
          ptx::tc_fence_after();
        }
        int kin = 0;  // chunk index inside the current segment
        for (int kc = 0; kc < p.k_chunks; ++kc, ++g) {
          const uint32_t t_acc = tmem + (kSeg ? 0 : ab) * NR;
          if (kSeg && kin == 0) {
            // the segment block is free once the epilogue has loaded the previous segment
            if (gs >= 1 && !ptx::mbar_wait_spin(&acce_bar[0], (uint32_t)(gs - 1) & 1, p.wait_cycles)) { ok = false; break; }
            ptx::tc_fence_after();
          }
          const int s = g % STAGES;
          const uint32_t use = g / STAGES;
          if (!ptx::mbar_wait(&full_bar[s], use & 1, p.wait_cycles)) { ok = false; break; }
          ptx::tc_fence_after();
          const uint32_t sa = ptx::smem_u32(smem + s * kStage);
          const uint32_t sb = sa + C::kAParts * kATile;
          int prod = 0;
#pragma unroll
          for (int a = 0; a < C::kAParts; ++a) {
#pragma unroll
            for (int b = 0; b < C::kBParts; ++b) {
              if (a + b > 1) continue;  // lo * lo is below the FP32 accumulator's resolution
#pragma unroll
              for (int k = 0; k < C::kMmaPerChunk; ++k) {
                const uint64_t ad = ptx::smem_desc_sw128(sa + a * kATile + k * 32);
                const uint64_t bd = ptx::smem_desc_sw128(sb + b * kBTile + k * 32);
                const uint32_t acc = ((kSeg ? kin : kc) > 0 || prod > 0 || k > 0) ? 1u : 0u;
                if constexpr (DT == kTcFp8)
                  ptx::mma_f8(t_acc, ad, bd, kIdesc, acc);
                else
                  ptx::mma_f16(t_acc, ad, bd, kIdesc, acc);
              }
              ++prod;
            }
          }
          ptx::mma_commit(&empty_bar[s]);
          if constexpr (kSeg) {
            if (++kin == p.seg_chunks || kc + 1 == p.k_chunks) {
              ptx::mma_commit(&accf_bar[0]);
              ++gs;
              kin = 0;
            }
          }
        }
        if (!ok) break;
        if constexpr (!kSeg) ptx::mma_commit(&accf_bar[ab]);
      }
      if (!ok) {
        // a wait gave up: the MMAs already issued finish before TMEM is freed
        ptx::mma_commit(&drain_bar);
        ptx::mbar_wait(&drain_bar, 0, p.wait_cycles);
      }
    }
  } else {
    // ---------------- epilogue: 8 warps, two per TMEM lane quadrant ----------------
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int c_lo = half * kHalf;
    const int row = m0 + 32 * q + lane;
    const uint32_t lane_off = (uint32_t)(32 * q) << 16;
    const float hv = (p.h && row < p.n) ? p.h[row] : 0.0f;
    if constexpr (!kEOnly) {
      for (int c = c_lo; c < c_lo + kHalf; c += 16) {
        uint32_t vx[16], vy[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int r = r0 + c + j;
          const bool in = row < p.n && r < p.R;
          vx[j] = __float_as_uint(in ? p.x[(size_t)r * p.xp + row] : 0.0f);
          vy[j] = __float_as_uint(in ? p.y[(size_t)r * p.xp + row] : 0.0f);
        }
        ptx::tmem_st16(t_x + lane_off + c, vx);
        ptx::tmem_st16(t_y + lane_off + c, vy);
      }
      ptx::tmem_st_wait();
    }
    // NMFA: one stage's Gaussian pair (nmfa.cu:103-109) for this thread's columns [c0, c1) (whole
    // 16-column chunks), z0 into the z0 columns and z1 into t_zdst; the XORWOW words are loaded
    // kDrawBatch elements at a time
    constexpr int kDrawBatch = 4;
    auto draw_stage = [&](int c0, int c1, uint32_t t_zdst) {
      const size_t plane = (size_t)p.R * p.xp;
#pragma unroll 1
      for (int c = c0; c < c1; c += 16) {
        uint32_t z0[16], z1[16];
#pragma unroll
        for (int g = 0; g < 16; g += kDrawBatch) {
          uint32_t wd[kDrawBatch][5];
#pragma unroll
          for (int jj = 0; jj < kDrawBatch; ++jj) {
            const int r = r0 + c + g + jj;
            const bool in = row < p.n && r < p.R && SB_BOUNDS(row < p.xp, p.status);
#pragma unroll
            for (int q = 0; q < 5; ++q) wd[jj][q] = in ? p.rng[q * plane + (size_t)r * p.xp + row] : 0u;
          }
#pragma unroll
          for (int jj = 0; jj < kDrawBatch; ++jj) {
            const int r = r0 + c + g + jj;
            float a = 0.0f, b = 0.0f;
            if (row < p.n && r < p.R && row < p.xp) {
              sbm::nmfa_gauss(wd[jj], p.noise, a, b);
#pragma unroll
              for (int q = 0; q < 5; ++q) p.rng[q * plane + (size_t)r * p.xp + row] = wd[jj][q];
            }
            z0[g + jj] = __float_as_uint(a);
            z1[g + jj] = __float_as_uint(b);
          }
        }
        ptx::tmem_st16(t_z0 + lane_off + c, z0);
        ptx::tmem_st16(t_zdst + lane_off + c, z1);
      }
      ptx::tmem_st_wait();
    };
    // the persistent NMFA run starts on a stage's first sweep (t0 even): draw that stage
    if constexpr (kNoiseAhead) {
      if (nsteps > 0 && (p.t0 & 1) == 0) draw_stage(c_lo, c_lo + kHalf, ((p.t0 >> 1) & 1) ? t_y1 : t_y);
    }
    float pump_next = (!kEOnly && nsteps > 0) ? p.pumps[p.t0] : 0.0f;
    uint32_t gs = 0;  // split operands: segments consumed
    for (int ls = 0; ls < nsteps; ++ls) {
      const int t = p.t0 + ls;
      const int buf = (p.buf0 + ls) & 1;
      if constexpr (kSeg) {
        // every segment, the step's last too: load it (then the MMA lane may start the next one into
        // the same block, the next step's first included) and add it into the sum, which is the field
        bool seg_ok = true;
        for (int sg = 0; sg < nseg; ++sg, ++gs) {
          const bool got_s = ptx::mbar_wait_spin(&accf_bar[0], gs & 1, p.wait_cycles);
          if (!epi_all(got_s)) { seg_ok = false; break; }
          ptx::tc_fence_after();
          uint32_t va[kHalf];
          if constexpr (kHalf == 64) {
            ptx::tmem_ld64(tmem + lane_off + c_lo, *reinterpret_cast<uint32_t(*)[64]>(va));
          } else {
#pragma unroll
            for (int i = 0; i < kHalf / 16; ++i)
              ptx::tmem_ld16(tmem + lane_off + c_lo + 16 * i, *reinterpret_cast<uint32_t(*)[16]>(va + 16 * i));
          }
          ptx::tmem_ld_wait();
          ptx::tc_fence_before();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(&acce_bar[0]);
#pragma unroll
          for (int i = 0; i < kHalf / 16; ++i) {
            uint32_t vs[16];
            const uint32_t ts = t_sum + lane_off + c_lo + 16 * i;
            if (sg > 0) {
              ptx::tmem_ld16(ts, vs);
              ptx::tmem_ld_wait();
#pragma unroll
              for (int j = 0; j < 16; ++j)
                vs[j] = __float_as_uint(__fadd_rn(__uint_as_float(vs[j]), __uint_as_float(va[16 * i + j])));
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j) vs[j] = va[16 * i + j];
            }
            ptx::tmem_st16(ts, vs);
          }
          ptx::tmem_st_wait();
        }
        if (!seg_ok) { ok = false; break; }
      }
      const int ab = ls & 1;
      const uint32_t t_acc = kSeg ? t_sum : tmem + ab * NR;
      if constexpr (!kSeg) {
        const bool got = ptx::mbar_wait(&accf_bar[ab], (uint32_t)(ls >> 1) & 1, p.wait_cycles);
        if (!epi_all(got)) { ok = false; break; }
      }
      ptx::tc_fence_after();
      // the schedule value was fetched one step ahead (a global load on the critical path otherwise)
      const float pump = pump_next;
      if (!kEOnly && ls + 1 < nsteps) pump_next = p.pumps[t + 1];
      uint8_t *const vnext[2] = {p.v[buf ^ 1][0], p.v[buf ^ 1][1]};
      uint8_t *const vtile = smem + STAGES * kStage;  // [NR][kVRow] staging tile
      constexpr int kChunks = kHalf / 16;
#pragma unroll 1
      for (int i = 0; i < kChunks; ++i) {
        const int c = c_lo + 16 * i;
        uint32_t va[16], vx[16], vy[16];
        ptx::tmem_ld16(t_acc + lane_off + c, va);
        if constexpr (!kEOnly) {
          ptx::tmem_ld16(t_x + lane_off + c, vx);
          // NMFA with the noise drawn ahead: vy holds this sweep's sample (z0 on a stage's first
          // sweep, z1 = y on its second), and y is never written here
          ptx::tmem_ld16((kNoiseAhead ? ((t & 1) == 0 ? t_z0 : (((t >> 1) & 1) ? t_y1 : t_y)) : t_y) + lane_off + c,
                         vy);
        }
        ptx::tmem_ld_wait();
        float e2[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int r = r0 + c + j;
          const bool in = row < p.n && r < p.R;
          const float f = DT == kTcFp16Split ? __fmul_rn(__uint_as_float(va[j]), fscale) : __uint_as_float(va[j]);
          float x, y;
          if constexpr (kEOnly) {
            x = in ? p.x[(size_t)r * p.xp + row] : 0.0f;
            y = 0.0f;
          } else {
            x = __uint_as_float(vx[j]);
            y = __uint_as_float(vy[j]);
          }
          // 2 x (energy contribution) of s(t): -s f - 2 h s, an integer for integer J and h
          if constexpr (want_e) {
            const float sg = sgnf(x);
            e2[j] = in ? __fsub_rn(-__fmul_rn(sg, f), __fmul_rn(2.0f * hv, sg)) : 0.0f;
          }
          if (!kEOnly && in) {
            if constexpr (VARIANT == 3) {
              // even sweeps open a stage: its first sample (drawn ahead, or drawn here with the
              // second kept in y); odd sweeps use the second
              float z = y;
              if constexpr (kNoiseAhead) {
              } else if (((t & 1) == 0) && SB_BOUNDS(row < p.xp, p.status)) {
                const size_t plane = (size_t)p.R * p.xp, k = (size_t)r * p.xp + row;
                uint32_t wd[5];
#pragma unroll
                for (int q = 0; q < 5; ++q) wd[q] = p.rng[q * plane + k];
                sbm::nmfa_gauss(wd, p.noise, z, y);
#pragma unroll
                for (int q = 0; q < 5; ++q) p.rng[q * plane + k] = wd[q];
              }
              x = sbm::nmfa_update(f, hv, z, pump, p.keep, p.mix, x);
            } else {
              sb_update(f, hv, pump, p.c0, p.dt, p.dta0, x, y);
            }
            if constexpr (!kStageV)
              if (SB_BOUNDS((size_t)r * p.Kp + row < (size_t)p.Rp * p.Kp, p.status))
                store_operand<DT, VARIANT>(vnext, (size_t)r * p.Kp + row, x, p.xscale);
          }
          if constexpr (kStageV && !kEOnly) {
            // every element of the tile is written (zero outside the problem) so the padding stays 0
            uint8_t *dst = vtile + (c + j) * kVRow + (row - m0) * C::kElem;
            if constexpr (DT == kTcFp8)
              *dst = in ? (x > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8) : (uint8_t)0;
            else
              *reinterpret_cast<uint16_t *>(dst) = in ? one16<DT>(!(x > 0.0f)) : (uint16_t)0;
          }
          vx[j] = __float_as_uint(x);
          vy[j] = __float_as_uint(y);
        }
        if constexpr (!kEOnly) {
          ptx::tmem_st16(t_x + lane_off + c, vx);
          if constexpr (!kNoiseAhead) ptx::tmem_st16(t_y + lane_off + c, vy);
        }
        if constexpr (want_e) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float v = e2[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) ered[q][c + j] = v;
          }
        }
      }
      if constexpr (!kEOnly) ptx::tmem_st_wait();
      // the accumulator may be overwritten from here on (split operands: released by the folds)
      ptx::tc_fence_before();
      __syncwarp();
      if (!kSeg && lane == 0) ptx::mbar_arrive(&acce_bar[ab]);
      // publish this unit's V(t+1) chunk to the replica column
      if constexpr (kStageV && !kEOnly) ptx::fence_proxy_async_shared();  // tile writes -> TMA store
      epi_sync();
      if (!kEOnly && threadIdx.x == kEpiFirstThread) {
        if constexpr (kStageV) {
          ptx::tma_store_2d(&p.tmS[buf ^ 1], vtile, m0, r0);
          ptx::bulk_commit();
          ptx::bulk_wait_all();  // the tile is in global memory (and may be rewritten next step)
        }
        ptx::fence_proxy_async_global();
        __threadfence();
        if (SB_BOUNDS(rt < p.n_rtiles && mt < p.n_mtiles, p.status) &&
            !((int)blockIdx.x == p.skip_unit && ls == p.skip_step))
          st_release(p.flags + ((size_t)rt * p.n_mtiles + mt) * p.flag_stride, (uint32_t)(ls + 1));
      }
      // NMFA: the next stage's noise, while the column's units finish this sweep and the next
      // contraction streams in: its first chunk after this stage's first sweep (whose z0 is
      // consumed; its z1 goes to the other z1 block), the rest after the second
      if constexpr (kNoiseAhead) {
        const uint32_t t_znext = (((t >> 1) + 1) & 1) ? t_y1 : t_y;
        constexpr int kFirst = kHalf > 16 ? 16 : 0;  // columns drawn after the first sweep
        if ((t & 1) == 0 && ls + 2 < nsteps && kFirst > 0) draw_stage(c_lo, c_lo + kFirst, t_znext);
        if ((t & 1) == 1 && ls + 1 < nsteps) draw_stage(c_lo + kFirst, c_lo + kHalf, t_znext);
      }
      if constexpr (want_e) {
        for (int c = threadIdx.x - kEpiFirstThread; c < NR; c += kEpiThreads) {
          const int r = r0 + c;
          if (r < p.R) {
            double *slot = kEOnly ? p.energy : p.energy + (size_t)t * p.R;
            const double sum = ((double)ered[0][c] + (double)ered[1][c]) + ((double)ered[2][c] + (double)ered[3][c]);
            atomicAdd(slot + r, 0.5 * sum);
          }
        }
        epi_sync();  // ered is rewritten by the next step
      }
    }
    // write the state back
    if (!kEOnly && ok) {
      for (int c = c_lo; c < c_lo + kHalf; c += 16) {
        uint32_t vx[16], vy[16];
        ptx::tmem_ld16(t_x + lane_off + c, vx);
        ptx::tmem_ld16(t_y + lane_off + c, vy);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int r = r0 + c + j;
          if (row < p.n && r < p.R && SB_BOUNDS(row < p.xp, p.status)) {
            p.x[(size_t)r * p.xp + row] = __uint_as_float(vx[j]);
            p.y[(size_t)r * p.xp + row] = __uint_as_float(vy[j]);
          }
        }
      }
    }
  }
  if (!ok) atomicOr(p.status, kErrWaitTimeout);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kCols);
  }
}

// Pipeline depth: as many stages as fit 200 KB of shared memory (at most 8).
template <int DT, int VARIANT, int NR>
constexpr int tc_vtile_bytes() {
  return Cfg<DT, VARIANT>::kBParts == 1 ? NR * kBM * Cfg<DT, VARIANT>::kElem : 0;
}

template <int DT, int VARIANT, int NR>
constexpr int tc_stages() {
  constexpr int kStage = Cfg<DT, VARIANT>::kAParts * kBM * kChunkBytes + Cfg<DT, VARIANT>::kBParts * NR * kChunkBytes;
  constexpr int kBudget = 216 * 1024 - tc_vtile_bytes<DT, VARIANT, NR>();
  return kBudget / kStage > 8 ? 8 : kBudget / kStage;
}

template <int DT, int VARIANT, int NR>
constexpr size_t tc_smem() {
  constexpr int kStage = Cfg<DT, VARIANT>::kAParts * kBM * kChunkBytes + Cfg<DT, VARIANT>::kBParts * NR * kChunkBytes;
  return (size_t)tc_stages<DT, VARIANT, NR>() * kStage + tc_vtile_bytes<DT, VARIANT, NR>() + 1024;
}

// Kernel for one epilogue mode; MODES is the bit set of modes compiled in.
template <int DT, int VARIANT, int NR, int MODES>
inline bool tc_lookup(int emode, const void **k, size_t *smem) {
  constexpr int S = tc_stages<DT, VARIANT, NR>();
  *smem = tc_smem<DT, VARIANT, NR>();
  *k = nullptr;
  if constexpr ((MODES & 1) != 0)
    if (emode == kEmodeStep) *k = reinterpret_cast<const void *>(&tc_sb_kernel<DT, VARIANT, NR, S, kEmodeStep>);
  if constexpr ((MODES & 2) != 0)
    if (emode == kEmodeStepTrace) *k = reinterpret_cast<const void *>(&tc_sb_kernel<DT, VARIANT, NR, S, kEmodeStepTrace>);
  if constexpr ((MODES & 4) != 0)
    if (emode == kEmodeEnergy) *k = reinterpret_cast<const void *>(&tc_sb_kernel<DT, VARIANT, NR, S, kEmodeEnergy>);
  return *k != nullptr;
}

}  // namespace tck
}  // namespace sbk
