// Tensor-core dSB step kernel with packed E2M1 operands and the couplings resident in shared memory.
//
// Same contraction as tc_sb_kernel (F[i][r] = sum_k J[i][k] sign(x[r][k]), the reference's per-step
// field call SB/CUDA_GPU/m2_opt.cu:169 for all replicas at once) and the same persistent,
// flag-ordered structure, with three changes:
//   * operands are E2M1 (4-bit floats, two per byte): sign(x) is +-1 and every integer coupling
//     with |J| <= 4 is exact, so the products and their FP32 sums are the integers the FP8 and
//     INT8 forms give (bit-identical fields); the MMA is tcgen05 kind::mxf4 with every block scale
//     1.0 (UE8M0 0x7F written once into TMEM);
//   * a unit's J rows (128 spins x Kp/2 bytes, at most ~160 KB) are loaded into shared memory once
//     per launch, so each SB step streams only the unit's V tile (NR replicas x Kp/2 bytes) from L2;
//   * the replica tile is split in two halves that move through the step one after the other:
//     half 0's epilogue publishes its part of V(t+1) (a dedicated publisher warp does the TMA store
//     and the release) while half 1 is still being updated, so the units of the column start the
//     next contraction on half 0 while this one finishes half 1. Flags are per (unit, half).
// TMEM columns: accumulators [0, NR) (half h at [h NR/2, (h+1) NR/2)), x [NR, 2NR), y [2NR, 3NR),
// A scales [3NR, 3NR + 16), B scales [3NR + 16, 3NR + 32). The nibble order inside a byte (spin 2j
// in the low half) is the same for J and V, so the dot products do not depend on how the tensor
// core orders the pair.
#pragma once
#include "sb_tc_kernel.cuh"

namespace sbk {
namespace tck {

// E2M1 code of a small integer (sign in bit 3; 1 -> 0x2, 2 -> 0x4, 3 -> 0x5, 4 -> 0x6), or 0xFF
// when the value is not one of 0, +-1, +-2, +-3, +-4.
__host__ __device__ inline uint8_t e2m1_code(float v) {
  const float a = v < 0.0f ? -v : v;
  uint8_t m;
  if (a == 0.0f) return 0;
  else if (a == 1.0f) m = 0x2;
  else if (a == 2.0f) m = 0x4;
  else if (a == 3.0f) m = 0x5;
  else if (a == 4.0f) m = 0x6;
  else return 0xFF;
  return v < 0.0f ? (uint8_t)(m | 0x8) : m;
}
constexpr uint8_t kE2m1Plus = 0x2, kE2m1Minus = 0xA;

// Block-scaled instruction descriptor: A and B E2M1 (code 1 for kind::mxf4) at bits 7-9 / 10-12,
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, UE8M0 scales (bit 23), M >> 4 at bits
// 24-28; scale-factor ids 0 (bits 4-5, 29-30); dense K = 64 (bit 31 = 0).
__host__ __device__ constexpr uint32_t make_idesc_mxf4(int m, int n) {
  return (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | (1u << 23) | ((uint32_t)(m >> 4) << 24);
}

// Replica halves and pipeline depth per replica tile: each epilogue warp takes a multiple of 16
// columns of a half.
// PAIR: two CTAs (a cluster of two, spin tiles 2k and 2k + 1 of the same replica tile) run one
// M = 256 MMA per K chunk (tcgen05 cta_group::2): each stages its own 128 J rows and half of the V
// chunk's replicas, so a CTA streams half the V bytes per step.
template <int NR, bool PAIR = false>
struct Fp4Cfg {
  static constexpr int kHalves = NR >= 64 ? 2 : 1;
  static constexpr int kNH = NR / kHalves;           // replicas per half: MMA N
  static constexpr int kBRows = PAIR ? kNH / 2 : kNH;  // V box rows this CTA loads
  static constexpr int kBTile = kBRows * kChunkBytes;  // this CTA's part of one V chunk of one half
  static constexpr int kStages = PAIR ? 16 : 8;        // the same 64 KB ring
  static constexpr int kWarpCols = kNH / 2;          // columns of a half per epilogue warp
};
constexpr int kFp4Threads = kTcThreads + 32;  // + the publisher warp

constexpr int kFp4ATile = kBM * kChunkBytes;  // one J chunk: 128 spins x 256 spins of K
// Shared memory of one CTA for k_chunks 128-byte chunks of K (256 spins each).
// At least enough that no more CTAs share an SM than its 512 TMEM columns hold (a CTA waiting
// in tcgen05.alloc would stall the flag-ordered grid).
template <int NR, bool PAIR = false>
constexpr size_t fp4_smem(int k_chunks) {
  constexpr int kCols = 3 * NR + 32 <= 128 ? 128 : (3 * NR + 32 <= 256 ? 256 : 512);
  constexpr size_t kFloor = 233472 / (512 / kCols + 1) + 1024;  // 228 KB of shared memory per SM
  const size_t need = 1024 + (size_t)Fp4Cfg<NR, PAIR>::kStages * Fp4Cfg<NR, PAIR>::kBTile +
                      (size_t)k_chunks * kFp4ATile + (size_t)NR * (kBM / 2);
  return need > kFloor ? need : kFloor;
}

// Buffers as in tc_sb_kernel; p.k_chunks = Kp / 256 (Kp a multiple of 256, J and V rows of Kp / 2
// bytes); p.tmA loads 128-byte x 128-row J boxes, p.tmB 128-byte x NR/2-row V boxes (NR/2 = the
// half's replicas; the whole NR when NR = 32), p.tmS stores one half tile (64 bytes x NR/2 rows).
// p.flags[((rt * halves + h) * n_mtiles + mt) * p.flag_stride] = steps whose half h this unit has published.
// PAIR (a cluster of two CTAs): p.tmB boxes hold kBRows = NH / 2 rows; the first CTA of the pair
// (rank 0) issues the MMAs and owns the copy barriers (full_bar, a_bar) that both CTAs' loads
// complete, and the accumulator-free barrier (acce_bar) that both CTAs' epilogues arrive on; its
// commits arrive on the same barrier of both CTAs. Every wait stays bounded; both CTAs meet at a
// cluster barrier before freeing tensor memory and exiting.
template <int NR, int EMODE, bool PAIR = false>
__global__ void __launch_bounds__(kFp4Threads, 1) tc_fp4_kernel(const __grid_constant__ TcArgs p) {
  using F = Fp4Cfg<NR, PAIR>;
  constexpr int H = F::kHalves, NH = F::kNH, STAGES = F::kStages, kBTile = F::kBTile;
  constexpr int kVRow = kBM / 2;  // bytes of one replica row of the unit's V tile
  constexpr uint32_t kSf = 3 * NR;
  constexpr uint32_t kCols = kSf + 32 <= 128 ? 128 : (kSf + 32 <= 256 ? 256 : 512);
  constexpr uint32_t kIdesc = make_idesc_mxf4(PAIR ? 2 * kBM : kBM, NH);
  static_assert(NR % 32 == 0 && NR >= 32 && NR <= 128 && F::kWarpCols % 16 == 0, "replica tile");
  static_assert(!PAIR || NR == 128, "CTA pairs run the 128-replica tile");

  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *ring = smem;                                   // [STAGES][NH][128] V chunks
  uint8_t *jres = smem + STAGES * kBTile;                  // [k_chunks][128][128] resident J
  uint8_t *vtile = jres + (size_t)p.k_chunks * kFp4ATile;  // [NR][64] next V tile (half h: rows h NH ..)
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], a_bar, accf_bar[H], acce_bar[H], pub_bar[H],
      drain_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float ered[4][NR];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x % p.n_mtiles, rt = blockIdx.x / p.n_mtiles;
  const int m0 = mt * kBM, r0 = rt * NR;
  constexpr bool kEOnly = EMODE == kEmodeEnergy;
  constexpr bool want_e = EMODE != kEmodeStep;
  const int nsteps = kEOnly ? 1 : p.steps;
  bool ok = true;
  const uint32_t crank = PAIR ? ptx::cluster_rank() : 0u;  // 0: the pair's MMA issuer
  const bool issuer = crank == 0;
  // shared::cluster address of the issuer's J-load barrier, which both CTAs' loads complete
  const uint32_t a_bar_c = PAIR ? ptx::mapa(ptx::smem_u32(&a_bar), 0) : 0u;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    ptx::mbar_init(&a_bar, 1);
    ptx::mbar_init(&drain_bar, 1);
    for (int h = 0; h < H; ++h) {
      ptx::mbar_init(&accf_bar[h], 1);
      ptx::mbar_init(&acce_bar[h], PAIR ? 2 * kEpiWarps : kEpiWarps);
      ptx::mbar_init(&pub_bar[h], kEpiWarps);
    }
    ptx::fence_mbar_init();
    ptx::prefetch_tmap(&p.tmA[0]);
    ptx::prefetch_tmap(&p.tmB[0][0]);
    ptx::prefetch_tmap(&p.tmB[1][0]);
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      ptx::tmem_alloc_pair(&tmem_base_sh, kCols);
      ptx::tmem_relinquish_pair();
    } else {
      ptx::tmem_alloc(&tmem_base_sh, kCols);
      ptx::tmem_relinquish();
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  const uint32_t t_x = tmem + NR, t_y = tmem + 2 * NR;
  if (warp >= 2 && warp < 2 + kEpiWarps) {
    // every block scale = 2^0: UE8M0 0x7F in all bytes of the scale columns, all 128 lanes
    uint32_t ones[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) ones[j] = 0x7F7F7F7Fu;
    const uint32_t lane_off = (uint32_t)(32 * (warp & 3)) << 16;
    ptx::tmem_st16(tmem + kSf + 16 * ((warp - 2) >> 2) + lane_off, ones);
    ptx::tmem_st_wait();
  }
  ptx::tc_fence_before();
  if constexpr (PAIR)
    ptx::cluster_sync();  // both CTAs' barriers initialised and scale columns written
  else
    __syncthreads();
  ptx::tc_fence_after();

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      if constexpr (PAIR) {
        if (issuer) ptx::mbar_arrive_expect_tx(&a_bar, (uint32_t)(2 * p.k_chunks * kFp4ATile));
        for (int kc = 0; kc < p.k_chunks; ++kc)
          ptx::tma_load_2d_pair(jres + (size_t)kc * kFp4ATile, &p.tmA[0], kc * kChunkBytes, m0, a_bar_c);
      } else {
        ptx::mbar_arrive_expect_tx(&a_bar, (uint32_t)(p.k_chunks * kFp4ATile));
        for (int kc = 0; kc < p.k_chunks; ++kc)
          ptx::tma_load_2d(jres + (size_t)kc * kFp4ATile, &p.tmA[0], kc * kChunkBytes, m0, &a_bar);
      }
    }
    uint32_t g = 0, issued = 0;  // chunks walked / V loads issued (lane 0)
    for (int ls = 0; ls < nsteps && ok; ++ls) {
      const int buf = (p.buf0 + ls) & 1;
      for (int h = 0; h < H && ok; ++h) {
        if (ls > 0) {
          // half h of V(ls) complete: every unit of the replica column has published it (the warp
          // polls 32 units per L2 round trip)
          const uint32_t *hf = p.flags + (size_t)(rt * H + h) * p.n_mtiles * p.flag_stride;
          for (int u0 = 0; u0 < p.n_mtiles && ok; u0 += 32) {
            const int u = u0 + lane;
            const bool fl = u < p.n_mtiles ? wait_flag(hf + (size_t)u * p.flag_stride, (uint32_t)ls, p.wait_cycles) : true;
            if (!__all_sync(0xffffffffu, fl)) ok = false;
          }
          ptx::fence_proxy_async_global();
        }
        for (int kc = 0; kc < p.k_chunks && ok; ++kc, ++g) {
          if (lane == 0) {
            const int s = g % STAGES;
            const uint32_t use = g / STAGES;
            const bool freed = use == 0 || (PAIR ? ptx::mbar_wait_cluster(&empty_bar[s], (use - 1) & 1, p.wait_cycles)
                                                  : ptx::mbar_wait(&empty_bar[s], (use - 1) & 1, p.wait_cycles));
            if (!freed) {
              ok = false;
            } else if constexpr (PAIR) {
              // the issuer's full_bar[s] counts both CTAs' halves of the chunk
              if (issuer) ptx::mbar_arrive_expect_tx(&full_bar[s], (uint32_t)(2 * kBTile));
              ptx::tma_load_2d_pair(ring + s * kBTile, &p.tmB[buf][0], kc * kChunkBytes,
                                    r0 + h * NH + (int)crank * F::kBRows, ptx::mapa(ptx::smem_u32(&full_bar[s]), 0));
              ++issued;
            } else {
              ptx::mbar_arrive_expect_tx(&full_bar[s], (uint32_t)kBTile);
              ptx::tma_load_2d(ring + s * kBTile, &p.tmB[buf][0], kc * kChunkBytes, r0 + h * NH, &full_bar[s]);
              ++issued;
            }
          }
          ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        }
      }
    }
    if (!ok && lane == 0) {
      // a wait gave up: let the copies this CTA started land before it exits (each stage's last
      // issued load, and the resident J)
      if constexpr (PAIR) {
        // this CTA's loads complete barriers of the issuer, which it cannot wait on: a bounded pause
        // far longer than any copy, then the issuer's own bounded waits
        const long long t0 = clock64();
        while (clock64() - t0 < (p.wait_cycles < 2000000LL ? p.wait_cycles : 2000000LL)) __nanosleep(1000);
        if (issuer) {
          for (int s = 0; s < STAGES; ++s)
            if (issued > (uint32_t)s) ptx::mbar_wait_cluster(&full_bar[s], ((issued - 1 - s) / STAGES) & 1, p.wait_cycles);
          ptx::mbar_wait_cluster(&a_bar, 0, p.wait_cycles);
        }
      } else {
        for (int s = 0; s < STAGES; ++s)
          if (issued > (uint32_t)s) ptx::mbar_wait(&full_bar[s], ((issued - 1 - s) / STAGES) & 1, p.wait_cycles);
        ptx::mbar_wait(&a_bar, 0, p.wait_cycles);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && issuer) {
      // ---------------- MMA issuer ----------------
      ok = PAIR ? ptx::mbar_wait_cluster(&a_bar, 0, p.wait_cycles) : ptx::mbar_wait(&a_bar, 0, p.wait_cycles);
      uint32_t g = 0;
      for (int ls = 0; ls < nsteps && ok; ++ls) {
        for (int h = 0; h < H && ok; ++h) {
          if (ls >= 1 && !(PAIR ? ptx::mbar_wait_cluster(&acce_bar[h], (uint32_t)(ls - 1) & 1, p.wait_cycles)
                                : ptx::mbar_wait(&acce_bar[h], (uint32_t)(ls - 1) & 1, p.wait_cycles))) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t t_acc = tmem + h * NH;
          for (int kc = 0; kc < p.k_chunks; ++kc, ++g) {
            const int s = g % STAGES;
            const uint32_t use = g / STAGES;
            if (!(PAIR ? ptx::mbar_wait_cluster(&full_bar[s], use & 1, p.wait_cycles)
                       : ptx::mbar_wait(&full_bar[s], use & 1, p.wait_cycles))) {
              ok = false;
              break;
            }
            ptx::tc_fence_after();
            const uint32_t sa = ptx::smem_u32(jres + (size_t)kc * kFp4ATile);
            const uint32_t sb = ptx::smem_u32(ring + s * kBTile);
#pragma unroll
            for (int k = 0; k < kChunkBytes / 32; ++k) {
              if constexpr (PAIR)
                ptx::mma_mxf4_pair(t_acc, ptx::smem_desc_sw128(sa + k * 32), ptx::smem_desc_sw128(sb + k * 32), kIdesc,
                                   tmem + kSf, tmem + kSf + 16, (kc > 0 || k > 0) ? 1u : 0u);
              else
                ptx::mma_mxf4(t_acc, ptx::smem_desc_sw128(sa + k * 32), ptx::smem_desc_sw128(sb + k * 32), kIdesc,
                              tmem + kSf, tmem + kSf + 16, (kc > 0 || k > 0) ? 1u : 0u);
            }
            if constexpr (PAIR)
              ptx::mma_commit_pair(&empty_bar[s]);
            else
              ptx::mma_commit(&empty_bar[s]);
          }
          if (!ok) break;
          if constexpr (PAIR)
            ptx::mma_commit_pair(&accf_bar[h]);
          else
            ptx::mma_commit(&accf_bar[h]);
        }
      }
      if constexpr (PAIR) {
        // both CTAs wait on drain_bar before freeing tensor memory: the MMAs issued are done
        ptx::mma_commit_pair(&drain_bar);
        ptx::mbar_wait_cluster(&drain_bar, 0, p.wait_cycles);
      } else if (!ok) {
        // a wait gave up: the MMAs already issued finish before TMEM is freed
        ptx::mma_commit(&drain_bar);
        ptx::mbar_wait(&drain_bar, 0, p.wait_cycles);
      }
    }
  } else if (warp == 2 + kEpiWarps) {
    // ---------------- publisher: half tile -> global (TMA store), then the flag ----------------
    if (!kEOnly && lane == 0) {
      for (int ls = 0; ls < nsteps && ok; ++ls) {
        const int buf = (p.buf0 + ls) & 1;
        for (int h = 0; h < H; ++h) {
          if (!ptx::mbar_wait(&pub_bar[h], (uint32_t)ls & 1, p.wait_cycles)) { ok = false; break; }
          ptx::tma_store_2d(&p.tmS[buf ^ 1], vtile + (size_t)h * NH * kVRow, m0 / 2, r0 + h * NH);
          ptx::bulk_commit();
          ptx::bulk_wait_all();             // the half tile is in global memory
          ptx::fence_proxy_async_global();  // the bulk store's writes, then the flag (release)
          if (SB_BOUNDS(rt < p.n_rtiles && mt < p.n_mtiles, p.status) &&
              !((int)blockIdx.x == p.skip_unit && ls == p.skip_step))
            st_release(p.flags + ((size_t)(rt * H + h) * p.n_mtiles + mt) * p.flag_stride, (uint32_t)(ls + 1));
        }
      }
    }
  } else {
    // ---------------- epilogue: 8 warps, two per TMEM lane quadrant ----------------
    const int q = warp & 3;
    const int sub = (warp - 2) >> 2;  // which kWarpCols columns of each half
    const int row = m0 + 32 * q + lane;
    const uint32_t lane_off = (uint32_t)(32 * q) << 16;
    const float hv = (p.h && row < p.n) ? p.h[row] : 0.0f;
    const bool odd = (lane & 1) != 0;
    if constexpr (!kEOnly) {
      for (int h = 0; h < H; ++h)
        for (int c = h * NH + sub * F::kWarpCols; c < h * NH + (sub + 1) * F::kWarpCols; c += 16) {
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
    float pump_next = (!kEOnly && nsteps > 0) ? p.pumps[p.t0] : 0.0f;
    for (int ls = 0; ls < nsteps && ok; ++ls) {
      const int t = p.t0 + ls;
      const float pump = pump_next;
      if (!kEOnly && ls + 1 < nsteps) pump_next = p.pumps[t + 1];
      for (int h = 0; h < H; ++h) {
        const bool got = PAIR ? ptx::mbar_wait_cluster(&accf_bar[h], (uint32_t)ls & 1, p.wait_cycles)
                              : ptx::mbar_wait(&accf_bar[h], (uint32_t)ls & 1, p.wait_cycles);
        if (!epi_all(got)) { ok = false; break; }
        ptx::tc_fence_after();
        const int c_lo = h * NH + sub * F::kWarpCols;
#pragma unroll 1
        for (int c = c_lo; c < c_lo + F::kWarpCols; c += 16) {
          uint32_t va[16], vx[16], vy[16];
          ptx::tmem_ld16(tmem + lane_off + c, va);
          if constexpr (!kEOnly) {
            ptx::tmem_ld16(t_x + lane_off + c, vx);
            ptx::tmem_ld16(t_y + lane_off + c, vy);
          }
          ptx::tmem_ld_wait();
          float e2[16];
          uint32_t nib_lo = 0, nib_hi = 0;  // this spin's next-operand nibbles for replicas c..c+7, c+8..c+15
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int r = r0 + c + j;
            const bool in = row < p.n && r < p.R;
            const float f = __uint_as_float(va[j]);
            float x, y;
            if constexpr (kEOnly) {
              x = in ? p.x[(size_t)r * p.xp + row] : 0.0f;
              y = 0.0f;
            } else {
              x = __uint_as_float(vx[j]);
              y = __uint_as_float(vy[j]);
            }
            if constexpr (want_e) {
              const float sg = sgnf(x);
              e2[j] = in ? __fsub_rn(-__fmul_rn(sg, f), __fmul_rn(2.0f * hv, sg)) : 0.0f;
            }
            if constexpr (!kEOnly) {
              // padded spins and replicas hold x = y = 0 and see f = h = 0, so they stay +0: the
              // update runs unpredicated and only the operand is masked
              sb_update(f, hv, pump, p.c0, p.dt, p.dta0, x, y);
              const uint32_t nib = in ? (x > 0.0f ? kE2m1Plus : kE2m1Minus) : 0u;
              if (j < 8) nib_lo |= nib << (4 * j);
              else nib_hi |= nib << (4 * (j - 8));
            }
            vx[j] = __float_as_uint(x);
            vy[j] = __float_as_uint(y);
          }
          if constexpr (!kEOnly) {
            ptx::tmem_st16(t_x + lane_off + c, vx);
            ptx::tmem_st16(t_y + lane_off + c, vy);
            // spins 2s (even lane, low nibble) and 2s + 1 (odd lane, high nibble) share a byte:
            // the even lane writes replicas c..c+7, the odd lane c+8..c+15
            const uint32_t o_lo = __shfl_xor_sync(0xffffffffu, nib_lo, 1);
            const uint32_t o_hi = __shfl_xor_sync(0xffffffffu, nib_hi, 1);
            const uint32_t lo_n = odd ? o_hi : nib_lo;  // even spin's nibbles for this lane's 8 replicas
            const uint32_t hi_n = odd ? nib_hi : o_lo;  // odd spin's nibbles
            uint8_t *dst = vtile + (size_t)(c + (odd ? 8 : 0)) * kVRow + ((32 * q + lane) >> 1);
#pragma unroll
            for (int j = 0; j < 8; ++j)
              dst[j * kVRow] = (uint8_t)(((lo_n >> (4 * j)) & 0xFu) | (((hi_n >> (4 * j)) & 0xFu) << 4));
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
        // the accumulator half may be overwritten from here on
        ptx::tc_fence_before();
        if constexpr (!kEOnly) ptx::fence_proxy_async_shared();  // tile writes -> the publisher's TMA store
        __syncwarp();
        if (lane == 0) {
          if constexpr (PAIR)
            ptx::mbar_arrive_cluster(ptx::mapa(ptx::smem_u32(&acce_bar[h]), 0));
          else
            ptx::mbar_arrive(&acce_bar[h]);
          if constexpr (!kEOnly) ptx::mbar_arrive(&pub_bar[h]);
        }
        // the next step rewrites this half tile only after its accumulator, which needs this
        // unit's own published half, i.e. after the publisher's store has completed
        if constexpr (want_e) {
          epi_sync();
          for (int c = h * NH + threadIdx.x - kEpiFirstThread; c < (h + 1) * NH; c += kEpiThreads) {
            const int r = r0 + c;
            if (r < p.R) {
              double *slot = kEOnly ? p.energy : p.energy + (size_t)t * p.R;
              const double sum = ((double)ered[0][c] + (double)ered[1][c]) + ((double)ered[2][c] + (double)ered[3][c]);
              atomicAdd(slot + r, 0.5 * sum);
            }
          }
          epi_sync();  // ered is rewritten by the next half
        }
      }
    }
    // write the state back
    if (!kEOnly && ok) {
      for (int h = 0; h < H; ++h)
        for (int c = h * NH + sub * F::kWarpCols; c < h * NH + (sub + 1) * F::kWarpCols; c += 16) {
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
  if constexpr (PAIR) {
    // the pair's second CTA: the issuer's MMAs write this CTA's tensor memory and read its shared
    // memory; once this CTA's own work is done, wait for their completion (the issuer's last commit)
    if (!issuer && warp == 1 && lane == 0 && !ptx::mbar_wait_cluster(&drain_bar, 0, p.wait_cycles))
      atomicOr(p.status, kErrWaitTimeout);
    ptx::cluster_sync();  // neither CTA leaves while the other may still touch its memory
  }
  if (warp == 1) {
    ptx::tc_fence_after();
    if constexpr (PAIR)
      ptx::tmem_dealloc_pair(tmem, kCols);
    else
      ptx::tmem_dealloc(tmem, kCols);
  }
}

}  // namespace tck
}  // namespace sbk
