// Tensor-core (tcgen05) SB engine: the field J*V for R replicas as a GEMM on the 5th-generation
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
//   * warps 2..5 (one per TMEM lane quadrant) read the accumulator, x and y with tcgen05.ld, apply
//     the SB update with the exact operation order of the CPU oracle, write x and y back to TMEM
//     and the next step's operand V (sign as FP8/BF16, or x as BF16 hi + lo) to global memory;
//   * a grid-wide barrier (release/acquire counter, bounded spin) separates the steps, because
//     every unit needs all of V(t) before step t's contraction.
// Operand dtypes: FP8 E4M3 holds +-1 and integers |J| <= 16 exactly; BF16 holds integers up to 256;
// BF16 hi + lo (J = Jh + Jl, x = xh + xl) gives ~16 bits for real values, with the three products
// Jh*xh + Jh*xl + Jl*xh accumulated in FP32. Integer fields are exact whenever every partial sum
// stays below 2^24 in magnitude, which holds for n * max|J| < 2^24.
// Every wait is bounded; a timeout sets a status bit, the kernel still frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "sb_host.h"
#include "sb_internal.h"
#include "sb_ptx.cuh"

namespace sbk {
namespace {

constexpr int kTcThreads = 192;  // 6 warps: producer, MMA, 4 epilogue
constexpr int kBM = 128;         // spins per unit (MMA M, TMEM lanes)
constexpr int kChunkBytes = 128; // K bytes per stage (one 128-byte swizzle atom row)

struct alignas(64) TcArgs {
  CUtensorMap tmA[2];      // J operand parts: [Np rows][Kp] K-major
  CUtensorMap tmB[2][2];   // V operand [buffer][part]: [Rp rows][Kp] K-major
  float *x, *y;            // [R][xp] state (read at start, written at the end)
  const float *h;          // [n] or null
  uint8_t *v[2][2];        // V operand [buffer][part] base pointers (bytes)
  double *energy;          // trace: [(steps + 1) * R] (step t -> slot t) or energy pass: [R]
  uint32_t *status;
  uint32_t *barrier;       // grid barrier counter (zeroed before the launch)
  int n, R, xp, Kp, Rp, n_mtiles, n_rtiles, k_chunks;
  int steps, t0;           // steps to run; schedule offset
  int energy_only;         // 1: one contraction on V[buf0], energy of sign(x) into energy[R]
  int buf0;                // V buffer holding V(t0)
  const float *pumps;      // pumps[t] = a0 - a(t), computed on the host
  float c0, dt, dta0;
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

template <int DT, int VARIANT>
struct Cfg {
  static constexpr int kElem = DtTraits<DT>::kElem;
  static constexpr int kAParts = DtTraits<DT>::kParts;
  // V = sign(x) needs one part even when J is split; bSB's x is split with J.
  static constexpr int kBParts = (DT == kTcBf16Split && VARIANT == 1) ? 2 : 1;
  static constexpr int kKPerMma = 32 / kElem;  // 32 bytes of K per instruction
  static constexpr int kMmaPerChunk = kChunkBytes / 32;
};

__host__ __device__ constexpr uint32_t make_idesc(int dt, int m, int n) {
  // D = F32 (bits 4-5 = 1); A/B format: E4M3 = 0 (kind::f8f6f4) or BF16 = 1 (kind::f16);
  // both K-major; N >> 3 at bits 17-22; M >> 4 at bits 24-28.
  return (1u << 4) | ((dt == kTcFp8 ? 0u : 1u) << 7) | ((dt == kTcFp8 ? 0u : 1u) << 10) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
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

// Write element (r, i) of the next operand.
template <int DT, int VARIANT>
__device__ __forceinline__ void store_operand(uint8_t *const (&vb)[2], size_t idx, float x) {
  if constexpr (DT == kTcFp8) {
    vb[0][idx] = x > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;  // E4M3 +1 / -1
  } else if constexpr (Cfg<DT, VARIANT>::kBParts == 1) {
    reinterpret_cast<uint16_t *>(vb[0])[idx] = x > 0.0f ? (uint16_t)0x3F80 : (uint16_t)0xBF80;
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
__device__ __forceinline__ void red_release_add(uint32_t *p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier for a cooperative launch: every CTA adds 1, then waits (bounded) until the
// counter reaches `target`. Returns false everywhere in the CTA if the wait gave up.
__device__ __forceinline__ bool grid_barrier(uint32_t *counter, uint32_t target) {
  __shared__ int ok_sh;
  ptx::fence_proxy_async_global();
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    red_release_add(counter, 1u);
    if (ld_acquire(counter) < target) {
      const long long t0 = clock64();
      while (ld_acquire(counter) < target) {
        if (clock64() - t0 > ptx::kWaitCycles) {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    ptx::fence_proxy_async_global();
    ok_sh = ok;
  }
  __syncthreads();
  return ok_sh != 0;
}

template <int DT, int VARIANT, int NR, int STAGES>
__global__ void __launch_bounds__(kTcThreads, 1) tc_sb_kernel(const __grid_constant__ TcArgs p) {
  using C = Cfg<DT, VARIANT>;
  constexpr int kATile = kBM * kChunkBytes;  // bytes per A part per stage
  constexpr int kBTile = NR * kChunkBytes;   // bytes per B part per stage
  constexpr int kStage = C::kAParts * kATile + C::kBParts * kBTile;
  constexpr uint32_t kTx = (uint32_t)kStage;
  constexpr uint32_t kCols = 4 * NR <= 32 ? 32 : (4 * NR <= 64 ? 64 : (4 * NR <= 128 ? 128 : (4 * NR <= 256 ? 256 : 512)));
  constexpr uint32_t kIdesc = make_idesc(DT, kBM, NR);
  static_assert(NR % 16 == 0 && NR >= 16 && NR <= 128, "replica tile");
  static_assert(3 * NR <= 512, "accumulator + x + y must fit TMEM");

  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accum_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float ered[4][NR];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % p.n_mtiles, rt = blockIdx.x / p.n_mtiles;
  const int m0 = mt * kBM, r0 = rt * NR;
  bool ok = true;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    ptx::mbar_init(&accum_bar, 1);
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
  const uint32_t t_acc = tmem, t_x = tmem + NR, t_y = tmem + 2 * NR;

  // epilogue geometry
  const int q = warp & 3;                // TMEM lane quadrant of this warp
  const int row = m0 + 32 * q + lane;    // spin index of this thread
  const uint32_t lane_off = (uint32_t)(32 * q) << 16;
  const bool is_epi = warp >= 2;
  const float hv = (is_epi && p.h && row < p.n) ? p.h[row] : 0.0f;

  // load x, y into TMEM
  if (is_epi && !p.energy_only) {
    for (int c = 0; c < NR; c += 16) {
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

  const int nsteps = p.energy_only ? 1 : p.steps;
  const bool want_e = p.energy != nullptr && (p.energy_only || VARIANT == 2);
  uint32_t gchunk = 0;  // chunks issued so far (producer and MMA count identically)
  int pre = 0;          // producer: chunks of the coming step whose J part is already in flight
  for (int ls = 0; ls < nsteps; ++ls) {
    const int t = p.t0 + ls;
    const int buf = (p.buf0 + ls) & 1;
    if (warp == 0 && lane == 0) {
      // ---- TMA producer ----
      for (int kc = 0; kc < p.k_chunks && ok; ++kc, ++gchunk) {
        const int s = gchunk % STAGES;
        const uint32_t use = gchunk / STAGES;
        uint8_t *st = smem + s * kStage;
        const int kx = kc * (kChunkBytes / C::kElem);
        if (kc >= pre) {
          if (use > 0 && !ptx::mbar_wait(&empty_bar[s], (use - 1) & 1)) {
            ok = false;
            break;
          }
          ptx::mbar_arrive_expect_tx(&full_bar[s], kTx);
          for (int a = 0; a < C::kAParts; ++a)
            ptx::tma_load_2d(st + a * kATile, &p.tmA[a], kx, m0, &full_bar[s]);
        }
        for (int b = 0; b < C::kBParts; ++b)
          ptx::tma_load_2d(st + C::kAParts * kATile + b * kBTile, &p.tmB[buf][b], kx, r0,
                           &full_bar[s]);
      }
      // J does not change between steps: start the next step's first J tiles now, so they land
      // while the epilogue and the grid barrier run.
      pre = 0;
      if (ok && ls + 1 < nsteps) {
        const int npre = p.k_chunks < STAGES ? p.k_chunks : STAGES;
        for (int kc = 0; kc < npre; ++kc) {
          const uint32_t g = gchunk + kc;
          const int s = g % STAGES;
          const uint32_t use = g / STAGES;
          if (use > 0 && !ptx::mbar_wait(&empty_bar[s], (use - 1) & 1)) {
            ok = false;
            break;
          }
          ptx::mbar_arrive_expect_tx(&full_bar[s], kTx);
          for (int a = 0; a < C::kAParts; ++a)
            ptx::tma_load_2d(smem + s * kStage + a * kATile, &p.tmA[a], kc * (kChunkBytes / C::kElem), m0,
                             &full_bar[s]);
          ++pre;
        }
      }
    } else if (warp == 1 && lane == 0) {
      // ---- MMA issuer ----
      for (int kc = 0; kc < p.k_chunks && ok; ++kc, ++gchunk) {
        const int s = gchunk % STAGES;
        const uint32_t use = gchunk / STAGES;
        if (!ptx::mbar_wait(&full_bar[s], use & 1)) {
          ok = false;
          break;
        }
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
              const uint32_t acc = (kc > 0 || prod > 0 || k > 0) ? 1u : 0u;
              if constexpr (DT == kTcFp8)
                ptx::mma_f8(t_acc, ad, bd, kIdesc, acc);
              else
                ptx::mma_f16(t_acc, ad, bd, kIdesc, acc);
            }
            ++prod;
          }
        }
        ptx::mma_commit(&empty_bar[s]);
      }
      ptx::mma_commit(&accum_bar);
    } else if (is_epi) {
      // ---- epilogue ----
      if (!ptx::mbar_wait(&accum_bar, (uint32_t)(ls & 1))) ok = false;
      ptx::tc_fence_after();
      const float pump = p.energy_only ? 0.0f : p.pumps[t];
      uint8_t *const vnext[2] = {p.v[buf ^ 1][0], p.v[buf ^ 1][1]};
      for (int c = 0; c < NR; c += 16) {
        uint32_t va[16], vx[16], vy[16];
        ptx::tmem_ld16(t_acc + lane_off + c, va);
        if (!p.energy_only) {
          ptx::tmem_ld16(t_x + lane_off + c, vx);
          ptx::tmem_ld16(t_y + lane_off + c, vy);
        }
        ptx::tmem_ld_wait();
        float e2[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int r = r0 + c + j;
          const bool in = ok && row < p.n && r < p.R;
          const float f = __uint_as_float(va[j]);
          float x, y;
          if (p.energy_only) {
            x = in ? p.x[(size_t)r * p.xp + row] : 0.0f;
            y = 0.0f;
          } else {
            x = __uint_as_float(vx[j]);
            y = __uint_as_float(vy[j]);
          }
          // 2 x (energy contribution) of s(t): -s f - 2 h s, an integer for integer J and h
          if (want_e) {
            const float s = sgnf(x);
            e2[j] = in ? __fsub_rn(-__fmul_rn(s, f), __fmul_rn(2.0f * hv, s)) : 0.0f;
          }
          if (!p.energy_only && in) {
            sb_update(f, hv, pump, p.c0, p.dt, p.dta0, x, y);
            store_operand<DT, VARIANT>(vnext, (size_t)r * p.Kp + row, x);
          }
          vx[j] = __float_as_uint(x);
          vy[j] = __float_as_uint(y);
        }
        if (!p.energy_only) {
          ptx::tmem_st16(t_x + lane_off + c, vx);
          ptx::tmem_st16(t_y + lane_off + c, vy);
        }
        if (want_e) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float v = e2[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) ered[q][c + j] = v;
          }
        }
      }
      if (!p.energy_only) ptx::tmem_st_wait();
    }
    ptx::tc_fence_before();
    // energy of s(t): one atomic per replica per CTA
    if (want_e) {
      __syncthreads();
      for (int c = threadIdx.x; c < NR; c += kTcThreads) {
        const int r = r0 + c;
        if (r < p.R) {
          double *slot = p.energy_only ? p.energy : p.energy + (size_t)t * p.R;
          const double sum = ((double)ered[0][c] + (double)ered[1][c]) + ((double)ered[2][c] + (double)ered[3][c]);
          atomicAdd(slot + r, 0.5 * sum);
        }
      }
    }
    if (p.energy_only) break;
    // every unit needs all of V(t+1) before the next contraction
    if (!grid_barrier(p.barrier, (uint32_t)(ls + 1) * gridDim.x)) ok = false;
    ptx::tc_fence_after();
    if (!ok) break;
  }

  // write the state back
  if (is_epi && !p.energy_only && ok) {
    for (int c = 0; c < NR; c += 16) {
      uint32_t vx[16], vy[16];
      ptx::tmem_ld16(t_x + lane_off + c, vx);
      ptx::tmem_ld16(t_y + lane_off + c, vy);
      ptx::tmem_ld_wait();
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int r = r0 + c + j;
        if (row < p.n && r < p.R) {
          p.x[(size_t)r * p.xp + row] = __uint_as_float(vx[j]);
          p.y[(size_t)r * p.xp + row] = __uint_as_float(vy[j]);
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

// ---- operand preparation ----

__global__ void convert_j_kernel(const float *J, int n, int jp, uint8_t *a0, uint8_t *a1, int Np,
                                 int Kp, int dt) {
  const size_t total = (size_t)Np * Kp;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / Kp, j = k % Kp;
    const float v = (i < (size_t)n && j < (size_t)n) ? J[i * jp + j] : 0.0f;
    if (dt == kTcFp8) {
      a0[k] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
    } else {
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      reinterpret_cast<__nv_bfloat16 *>(a0)[k] = hi;
      if (dt == kTcBf16Split)
        reinterpret_cast<__nv_bfloat16 *>(a1)[k] = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi)));
    }
  }
}

__global__ void prepare_v_kernel(const float *x, int n, int R, int xp, uint8_t *v0, uint8_t *v1,
                                 int Kp, int dt, int variant) {
  const size_t total = (size_t)n * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / n, i = k % n;
    const float xv = x[r * xp + i];
    const size_t idx = r * Kp + i;
    if (dt == kTcFp8) {
      v0[idx] = xv > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;
    } else if (dt == kTcBf16 || variant == 2) {
      reinterpret_cast<uint16_t *>(v0)[idx] = xv > 0.0f ? (uint16_t)0x3F80 : (uint16_t)0xBF80;
    } else {
      const __nv_bfloat16 hi = __float2bfloat16_rn(xv);
      reinterpret_cast<__nv_bfloat16 *>(v0)[idx] = hi;
      reinterpret_cast<__nv_bfloat16 *>(v1)[idx] = __float2bfloat16_rn(__fsub_rn(xv, __bfloat162float(hi)));
    }
  }
}

int grid_1d(size_t total) {
  size_t g = (total + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g ? g : 1);
}

// ---- tensor maps ----

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool encode_2d(CUtensorMap *m, void *base, int elem, uint64_t inner, uint64_t outer, uint32_t box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {inner * (uint64_t)elem};
  const cuuint32_t box[2] = {(cuuint32_t)(kChunkBytes / elem), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, elem == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                         base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int DT, int VARIANT, int NR, int STAGES>
constexpr size_t smem_bytes() {
  using C = Cfg<DT, VARIANT>;
  return (size_t)STAGES * (C::kAParts * kBM * kChunkBytes + C::kBParts * NR * kChunkBytes) + 1024;
}

}  // namespace

// ---------------------------------------------------------------------------------------------

struct TcEngine {
  TcSetup s{};
  int nr = 128, Np = 0, Kp = 0, Rp = 0, n_mtiles = 0, n_rtiles = 0, units = 0;
  uint8_t *a[2] = {nullptr, nullptr};
  uint8_t *v[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  uint32_t *barrier = nullptr;
  TcArgs args{};
  const void *kernel = nullptr;
  size_t smem = 0;
};

namespace {

template <int DT, int VARIANT, int NR>
void pick_kernel(TcEngine *e) {
  constexpr int kStageBytes = Cfg<DT, VARIANT>::kAParts * kBM * kChunkBytes + Cfg<DT, VARIANT>::kBParts * NR * kChunkBytes;
  constexpr int STAGES = (200 * 1024) / kStageBytes > 8 ? 8 : (200 * 1024) / kStageBytes;
  e->kernel = reinterpret_cast<const void *>(&tc_sb_kernel<DT, VARIANT, NR, STAGES>);
  e->smem = smem_bytes<DT, VARIANT, NR, STAGES>();
}

template <int DT, int VARIANT>
bool pick_nr(TcEngine *e, int nr) {
  switch (nr) {
    case 32: pick_kernel<DT, VARIANT, 32>(e); return true;
    case 64: pick_kernel<DT, VARIANT, 64>(e); return true;
    case 128: pick_kernel<DT, VARIANT, 128>(e); return true;
    default: return false;
  }
}

bool pick(TcEngine *e, int dt, int variant, int nr) {
  if (variant == 2) {
    if (dt == kTcFp8) return pick_nr<kTcFp8, 2>(e, nr);
    if (dt == kTcBf16) return pick_nr<kTcBf16, 2>(e, nr);
    return pick_nr<kTcBf16Split, 2>(e, nr);
  }
  if (dt == kTcBf16Split) return pick_nr<kTcBf16Split, 1>(e, nr);
  return false;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Replica tile: the largest of {128, 64, 32} that keeps every unit co-resident (one CTA per SM).
int choose_nr(int n, int R, int sms) {
  const int mt = (n + kBM - 1) / kBM;
  for (int nr : {128, 64, 32}) {
    const int rt = (R + nr - 1) / nr;
    if (mt * rt <= sms) {
      // prefer the smaller tile when it does not need more units than SMs and wastes less padding
      return nr;
    }
  }
  return 0;
}

}  // namespace

int64_t tc_footprint(const TcSetup &s) {
  const int elem = s.dtype == kTcFp8 ? 1 : 2;
  const int64_t Np = (s.n + kBM - 1) / kBM * kBM, Kp = (s.n + 127) / 128 * 128;
  const int64_t Rp = (s.R + 127) / 128 * 128;
  const int ap = s.dtype == kTcBf16Split ? 2 : 1;
  const int bp = (s.dtype == kTcBf16Split && s.variant == 1) ? 2 : 1;
  return Np * Kp * elem * ap + 2 * Rp * Kp * elem * bp + 64;
}

sb_status tc_create(TcEngine **out, const TcSetup &s, const float *dJ, int jp, std::string &err,
                    cudaStream_t st) {
  *out = nullptr;
  if (s.variant != 1 && s.variant != 2) {
    err = "tensor-core path runs bSB and dSB";
    return SB_ERR_UNSUPPORTED;
  }
  if (s.variant == 1 && s.dtype != kTcBf16Split) {
    err = "bSB on tensor cores needs the BF16 hi+lo operands";
    return SB_ERR_UNSUPPORTED;
  }
  const int sms = sm_count();
  const int nr = choose_nr(s.n, s.R, sms);
  if (nr == 0) {
    err = "problem too large for the single-pass tensor-core kernel (units > SMs)";
    return SB_ERR_UNSUPPORTED;
  }
  TcEngine *e = new TcEngine();
  e->s = s;
  e->nr = nr;
  if (!pick(e, s.dtype, s.variant, nr)) {
    delete e;
    err = "no kernel for this dtype / variant";
    return SB_ERR_UNSUPPORTED;
  }
  const int elem = s.dtype == kTcFp8 ? 1 : 2;
  e->Np = (s.n + kBM - 1) / kBM * kBM;
  e->Kp = (s.n + 127) / 128 * 128;
  e->Rp = (s.R + nr - 1) / nr * nr;
  e->n_mtiles = e->Np / kBM;
  e->n_rtiles = e->Rp / nr;
  e->units = e->n_mtiles * e->n_rtiles;
  const int ap = s.dtype == kTcBf16Split ? 2 : 1;
  const int bp = (s.dtype == kTcBf16Split && s.variant == 1) ? 2 : 1;
  auto fail = [&](const char *what, cudaError_t ce) {
    err = std::string(what) + (ce != cudaSuccess ? std::string(": ") + cudaGetErrorString(ce) : "");
    tc_destroy(e);
    return ce == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  };
  cudaError_t ce;
  const size_t abytes = (size_t)e->Np * e->Kp * elem, vbytes = (size_t)e->Rp * e->Kp * elem;
  for (int a = 0; a < ap; ++a)
    if ((ce = cudaMalloc(&e->a[a], abytes)) != cudaSuccess) return fail("cudaMalloc(J operand)", ce);
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < bp; ++pp) {
      if ((ce = cudaMalloc(&e->v[b][pp], vbytes)) != cudaSuccess) return fail("cudaMalloc(V operand)", ce);
      if ((ce = cudaMemsetAsync(e->v[b][pp], 0, vbytes, st)) != cudaSuccess) return fail("memset", ce);
    }
  if ((ce = cudaMalloc(&e->barrier, 64)) != cudaSuccess) return fail("cudaMalloc(barrier)", ce);
  convert_j_kernel<<<grid_1d((size_t)e->Np * e->Kp), 256, 0, st>>>(dJ, s.n, jp, e->a[0], e->a[1], e->Np, e->Kp, s.dtype);
  if ((ce = cudaGetLastError()) != cudaSuccess) return fail("convert_j_kernel", ce);
  TcArgs &g = e->args;
  memset(&g, 0, sizeof(g));
  for (int a = 0; a < ap; ++a)
    if (!encode_2d(&g.tmA[a], e->a[a], elem, (uint64_t)e->Kp, (uint64_t)e->Np, kBM)) return fail("cuTensorMapEncodeTiled(J)", cudaSuccess);
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < bp; ++pp) {
      if (!encode_2d(&g.tmB[b][pp], e->v[b][pp], elem, (uint64_t)e->Kp, (uint64_t)e->Rp, (uint32_t)nr))
        return fail("cuTensorMapEncodeTiled(V)", cudaSuccess);
      g.v[b][pp] = e->v[b][pp];
    }
  g.barrier = e->barrier;
  g.n = s.n;
  g.R = s.R;
  g.xp = s.xp;
  g.Kp = e->Kp;
  g.Rp = e->Rp;
  g.n_mtiles = e->n_mtiles;
  g.n_rtiles = e->n_rtiles;
  g.k_chunks = e->Kp * elem / kChunkBytes;
  if ((ce = cudaFuncSetAttribute(e->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smem)) != cudaSuccess)
    return fail("cudaFuncSetAttribute", ce);
  *out = e;
  return SB_OK;
}

void tc_destroy(TcEngine *e) {
  if (!e) return;
  cudaFree(e->a[0]);
  cudaFree(e->a[1]);
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < 2; ++pp) cudaFree(e->v[b][pp]);
  cudaFree(e->barrier);
  delete e;
}

cudaError_t tc_reload(TcEngine *e, const float *dJ, int jp, cudaStream_t st) {
  convert_j_kernel<<<grid_1d((size_t)e->Np * e->Kp), 256, 0, st>>>(dJ, e->s.n, jp, e->a[0], e->a[1], e->Np, e->Kp,
                                                                   e->s.dtype);
  return cudaGetLastError();
}

int tc_dtype(const TcEngine *e) { return e ? e->s.dtype : 0; }
int tc_units(const TcEngine *e) { return e ? e->units : 0; }
int tc_replica_tile(const TcEngine *e) { return e ? e->nr : 0; }

cudaError_t tc_prepare(TcEngine *e, const float *x, cudaStream_t st) {
  prepare_v_kernel<<<grid_1d((size_t)e->s.n * e->s.R), 256, 0, st>>>(x, e->s.n, e->s.R, e->s.xp, e->v[0][0], e->v[0][1], e->Kp,
                                                                      e->s.dtype, e->s.variant);
  return cudaGetLastError();
}

static cudaError_t launch(TcEngine *e, const TcArgs &a, cudaStream_t st) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)e->units);
  cfg.blockDim = dim3(kTcThreads);
  cfg.dynamicSmemBytes = e->smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void *params[1] = {const_cast<TcArgs *>(&a)};
  return cudaLaunchKernelExC(&cfg, e->kernel, params);
}

cudaError_t tc_run(TcEngine *e, int steps, const float *pumps, float *x, float *y, const float *h, float c0,
                   float dt, float dta0, double *energy_trace, uint32_t *status, cudaStream_t st) {
  if (steps <= 0) return cudaSuccess;
  TcArgs a = e->args;
  a.x = x;
  a.y = y;
  a.h = h;
  a.energy = energy_trace;
  a.status = status;
  a.steps = steps;
  a.t0 = 0;
  a.energy_only = 0;
  a.buf0 = 0;
  a.pumps = pumps;
  a.c0 = c0;
  a.dt = dt;
  a.dta0 = dta0;
  cudaError_t ce = cudaMemsetAsync(e->barrier, 0, 64, st);
  if (ce != cudaSuccess) return ce;
  return launch(e, a, st);
}

cudaError_t tc_step(TcEngine *, int, float *, float *, const float *, float, float, float, float, double *,
                    uint32_t *, cudaStream_t) {
  return cudaErrorNotSupported;  // the persistent kernel runs every step in one launch (tc_run)
}

void tc_external_sizes(int n, int R, int *nr, size_t *a_bytes, size_t *v_bytes) {
  const int r = choose_nr(n, R, sm_count());
  const size_t Np = (size_t)(n + kBM - 1) / kBM * kBM, Kp = (size_t)(n + 127) / 128 * 128;
  const size_t Rp = r > 0 ? (size_t)(R + r - 1) / r * r : 0;
  *nr = r;
  *a_bytes = Np * Kp;
  *v_bytes = Rp * Kp;
}

cudaError_t tc_dsb_fp8_external(const TcExternal &ext, cudaStream_t st) {
  TcEngine e;  // on the stack: every buffer below belongs to the caller
  e.s = TcSetup{2, kTcFp8, ext.n, ext.R, ext.xp};
  e.nr = choose_nr(ext.n, ext.R, sm_count());
  if (e.nr == 0 || !pick(&e, kTcFp8, 2, e.nr)) return cudaErrorInvalidValue;
  e.Np = (ext.n + kBM - 1) / kBM * kBM;
  e.Kp = (ext.n + 127) / 128 * 128;
  e.Rp = (ext.R + e.nr - 1) / e.nr * e.nr;
  e.n_mtiles = e.Np / kBM;
  e.n_rtiles = e.Rp / e.nr;
  e.units = e.n_mtiles * e.n_rtiles;
  e.a[0] = ext.a;
  e.v[0][0] = ext.v0;
  e.v[1][0] = ext.v1;
  e.barrier = ext.barrier;
  TcArgs &g = e.args;
  memset(&g, 0, sizeof(g));
  if (!encode_2d(&g.tmA[0], e.a[0], 1, (uint64_t)e.Kp, (uint64_t)e.Np, kBM) ||
      !encode_2d(&g.tmB[0][0], e.v[0][0], 1, (uint64_t)e.Kp, (uint64_t)e.Rp, (uint32_t)e.nr) ||
      !encode_2d(&g.tmB[1][0], e.v[1][0], 1, (uint64_t)e.Kp, (uint64_t)e.Rp, (uint32_t)e.nr))
    return cudaErrorInvalidValue;
  g.v[0][0] = e.v[0][0];
  g.v[1][0] = e.v[1][0];
  g.barrier = e.barrier;
  g.n = ext.n;
  g.R = ext.R;
  g.xp = ext.xp;
  g.Kp = e.Kp;
  g.Rp = e.Rp;
  g.n_mtiles = e.n_mtiles;
  g.n_rtiles = e.n_rtiles;
  g.k_chunks = e.Kp / kChunkBytes;
  cudaError_t ce = cudaFuncSetAttribute(e.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem);
  if (ce != cudaSuccess) return ce;
  convert_j_kernel<<<grid_1d((size_t)e.Np * e.Kp), 256, 0, st>>>(ext.J, ext.n, ext.jp, e.a[0], nullptr, e.Np, e.Kp,
                                                                 kTcFp8);
  if ((ce = cudaGetLastError()) != cudaSuccess) return ce;
  if ((ce = tc_prepare(&e, ext.x, st)) != cudaSuccess) return ce;
  if ((ce = tc_run(&e, ext.steps, ext.pumps, ext.x, ext.y, ext.h, ext.c0, ext.dt, ext.dta0, nullptr, ext.status,
                   st)) != cudaSuccess)
    return ce;
  return tc_energy(&e, ext.steps, ext.x, ext.h, ext.energy, ext.status, st);
}

cudaError_t tc_energy(TcEngine *e, int t, const float *x, const float *h, double *energy, uint32_t *status,
                      cudaStream_t st) {
  TcArgs a = e->args;
  a.x = const_cast<float *>(x);
  a.y = nullptr;
  a.h = h;
  a.energy = energy;
  a.status = status;
  a.steps = 1;
  a.t0 = 0;
  a.energy_only = 1;
  a.buf0 = t & 1;
  return launch(e, a, st);
}

}  // namespace sbk
