// Grouped tcgen05 SB step over many instances of uneven size (dSB; packed E2M1, packed E2M3 or
// FP8 E4M3 operands).
//
// Uneven batches (hundreds of instances with N from 64 to 16384, each with its own replicas) and
// the serving stream do not fit the one-unit-per-SM residency of
// the single-instance kernel (sb_tc_kernel.cuh): their state is far larger than TMEM. Here one
// launch advances every instance by one SB step:
//   * work item = (instance, 128-spin tile, NR-replica tile); the CTAs of a persistent grid (one
//     per SM) walk a cost-sorted item list round-robin;
//   * warp 0 (lane 0) streams each item's J tile and V tile with 2-D TMA through the shared-memory
//     ring, using the instance's tensor maps, which live in device memory next to its descriptor;
//   * warp 1 (lane 0) issues tcgen05.mma (kind::f8f6f4, or kind::mxf4 for E2M1) into one of two
//     TMEM accumulators, so the
//     epilogue of item k overlaps the contraction of item k + 1;
//   * 8 epilogue warps read the accumulator, load x and y from global memory (coalesced), apply
//     the dSB update in the oracle's operation order, store x and y and the next operand.
// The kernel boundary orders the steps; the step loop is captured in a CUDA graph. Each instance
// carries its own schedule (pump table) and its own step counter offset, so instances admitted at
// different times advance side by side (continuous batching). Every wait is bounded.
#pragma once
#include "sb_grouped.h"
#include "sb_tc_fp4.cuh"
#include "sb_tc_kernel.cuh"

namespace sbk {

namespace tck {

// OP (GOperand): FP8 E4M3; packed E2M3 (kind::f8f6f4 with both formats E2M3: J / 4 against signs of
// +-4, sixteen 6-bit values per 12 bytes in global memory, spread by the tensor map to one 16-byte
// slot per sixteen values in shared memory, the layout the MMA reads); or
// FP4: packed E2M1 operands (kind::mxf4, every block scale 1.0 in TMEM columns [2NR, 2NR + 32)),
// a 128-byte chunk holding 256 spins of K; V written as nibble pairs (spin 2s low, 2s + 1 high).
template <int NR, int STAGES, int EMODE, int OP>
__global__ void __launch_bounds__(kTcThreads, 1)
    grouped_kernel(const GInst *__restrict__ insts, const GItem *__restrict__ items, int n_items, int tick,
                   uint32_t *status) {
  using C = Cfg<kTcFp8, 2>;
  constexpr int kATile = kBM * kChunkBytes;
  constexpr int kBTile = NR * kChunkBytes;
  constexpr int kStage = kATile + kBTile;
  constexpr uint32_t kSf = 2 * NR;
  constexpr bool FP4 = OP == kGopE2m1, FP6 = OP == kGopE2m3;
  // bytes a stage's copies count on its barrier: the packed E2M3 boxes count their global bytes,
  // 12 per 16-byte shared-memory slot
  constexpr uint32_t kTx = FP6 ? (uint32_t)kStage / 4 * 3 : (uint32_t)kStage;
  constexpr uint32_t kNeed = FP4 ? 2 * NR + 32 : 2 * NR;
  constexpr uint32_t kCols = kNeed <= 32 ? 32 : (kNeed <= 64 ? 64 : (kNeed <= 128 ? 128 : (kNeed <= 256 ? 256 : 512)));
  // kind::f8f6f4 formats (A bits 7-9, B bits 10-12): E4M3 = 0, E2M3 = 3
  constexpr uint32_t kIdesc = FP4 ? make_idesc_mxf4(kBM, NR)
                                  : (make_idesc(kTcFp8, kBM, NR) | (FP6 ? ((3u << 7) | (3u << 10)) : 0u));
  constexpr int kHalf = NR / 2;
  constexpr bool kEOnly = EMODE == kEmodeEnergy;
  static_assert(NR == 32 || NR == 64 || NR == 128, "replica tile");

  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accf_bar[2], acce_bar[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ float ered[4][NR];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(&tmem_base_sh, kCols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  if constexpr (FP4) {
    if (warp >= 2) {
      // every block scale = 2^0: UE8M0 0x7F in all bytes of the 32 scale columns, all 128 lanes
      uint32_t ones[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) ones[j] = 0x7F7F7F7Fu;
      ptx::tmem_st16(tmem + kSf + 16 * ((warp - 2) >> 2) + ((uint32_t)(32 * (warp & 3)) << 16), ones);
      ptx::tmem_st_wait();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
  }

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      uint32_t g = 0;
      for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        const GItem w = items[it];
        const GInst *in = insts + w.inst;
        const int buf = (tick - in->t0) & 1;
        for (int kc = 0; kc < w.kchunks; ++kc, ++g) {
          const int s = g % STAGES;
          const uint32_t use = g / STAGES;
          if (use > 0 && !ptx::mbar_wait(&empty_bar[s], (use - 1) & 1)) {
            ok = false;
            break;
          }
          uint8_t *st = smem + s * kStage;
          ptx::mbar_arrive_expect_tx(&full_bar[s], kTx);
          ptx::tma_load_2d(st, &in->tmA, kc * kChunkBytes, w.m0, &full_bar[s]);
          ptx::tma_load_2d(st + kATile, &in->tmB[buf], kc * kChunkBytes, w.r0, &full_bar[s]);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      uint32_t g = 0;
      int li = 0;
      for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
        const int kchunks = items[it].kchunks;
        const int ab = li & 1;
        const uint32_t t_acc = tmem + ab * NR;
        if (li >= 2 && !ptx::mbar_wait(&acce_bar[ab], (uint32_t)((li >> 1) - 1) & 1)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        for (int kc = 0; kc < kchunks; ++kc, ++g) {
          const int s = g % STAGES;
          const uint32_t use = g / STAGES;
          if (!ptx::mbar_wait(&full_bar[s], use & 1)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t sa = ptx::smem_u32(smem + s * kStage);
#pragma unroll
          for (int k = 0; k < C::kMmaPerChunk; ++k) {
            const uint64_t ad = ptx::smem_desc_sw128(sa + k * 32), bd = ptx::smem_desc_sw128(sa + kATile + k * 32);
            if constexpr (FP4)
              ptx::mma_mxf4(t_acc, ad, bd, kIdesc, tmem + kSf, tmem + kSf + 16, (kc > 0 || k > 0) ? 1u : 0u);
            else
              ptx::mma_f8(t_acc, ad, bd, kIdesc, (kc > 0 || k > 0) ? 1u : 0u);
          }
          ptx::mma_commit(&empty_bar[s]);
        }
        ptx::mma_commit(&accf_bar[ab]);
      }
    }
  } else {
    // ---------------- epilogue ----------------
    // A thread updates its row's state 16 replica columns at a time. The state does not depend on
    // the contraction, so the first group's x and y are loaded before the accumulator wait (their
    // latency overlaps the MMA), and each next group's loads are issued before the current group's
    // stores (two groups in flight).
    constexpr int kGroup = 16;
    constexpr int kSub = kGroup / 16;
    constexpr int kGroups = kHalf / kGroup;
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int c_lo = half * kHalf;
    const uint32_t lane_off = (uint32_t)(32 * q) << 16;
    int li = 0;
#pragma unroll 1
    for (int it = blockIdx.x; it < n_items; it += gridDim.x, ++li) {
      const GItem w = items[it];
      const GInst *in = insts + w.inst;
      const int ab = li & 1;
      const uint32_t t_acc = tmem + ab * NR;
      const int n = in->n, R = in->R, xp = in->xp, kb = in->kbytes;
      const int row = w.m0 + 32 * q + lane;
      // element (replica r, spin row) of x and y sits at r * xp + row: 32-bit offsets from the row's
      // base (an instance's state is far below 2^32 elements) keep the group's addresses cheap
      float *xs = in->x + row, *ys = in->y + row;
      const uint32_t uxp = (uint32_t)xp;
      float xv[kGroup], yv[kGroup];
      auto load_group = [&](int g0, float (&ox)[kGroup], float (&oy)[kGroup]) {
        const int rlim = row < n ? R - (w.r0 + g0) : 0;  // columns j < rlim are inside the instance
        const uint32_t o0 = (uint32_t)(w.r0 + g0) * uxp;
#pragma unroll
        for (int j = 0; j < kGroup; ++j) {
          const uint32_t o = o0 + (uint32_t)j * uxp;
          ox[j] = j < rlim ? xs[o] : 0.0f;
          if constexpr (!kEOnly) oy[j] = j < rlim ? ys[o] : 0.0f;
        }
      };
      load_group(c_lo, xv, yv);
      const bool got = ptx::mbar_wait(&accf_bar[ab], (uint32_t)(li >> 1) & 1);
      if (!epi_all(got)) {
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      const int t = tick - in->t0;
      const float hv = (in->h && row < n) ? in->h[row] : 0.0f;
      const float pump = kEOnly ? 0.0f : in->pumps[t];
      const float c0 = in->c0, dt = in->dt, dta0 = in->dta0;
      uint8_t *vn = in->v[(t + 1) & 1];
#pragma unroll 1
      for (int gi = 0; gi < kGroups; ++gi) {
        const int g0 = c_lo + gi * kGroup;
        float xn[kGroup], yn[kGroup];
        if (gi + 1 < kGroups) load_group(g0 + kGroup, xn, yn);
        uint32_t va[kSub][16];
#pragma unroll
        for (int s = 0; s < kSub; ++s) ptx::tmem_ld16(t_acc + lane_off + g0 + 16 * s, va[s]);
        ptx::tmem_ld_wait();
        float e2[kGroup];
#pragma unroll
        for (int j = 0; j < kGroup; ++j) {
          const int r = w.r0 + g0 + j;
          const bool ins = row < n && r < R;
          const float f = __uint_as_float(va[j / 16][j % 16]);
          float x = xv[j];
          if constexpr (kEOnly) {
            const float sg = sgnf(x);
            e2[j] = ins ? __fsub_rn(-__fmul_rn(sg, f), __fmul_rn(2.0f * hv, sg)) : 0.0f;
          } else {
            float y = yv[j];
            sb_update(f, hv, pump, c0, dt, dta0, x, y);
            xv[j] = x;
            yv[j] = y;
          }
        }
        if constexpr (!kEOnly) {
          const int rlim = row < n ? R - (w.r0 + g0) : 0;
          const uint32_t o0 = (uint32_t)(w.r0 + g0) * uxp, v0 = (uint32_t)(w.r0 + g0) * (uint32_t)kb;
#pragma unroll
          for (int j = 0; j < kGroup; ++j) {
            if (j < rlim && SB_BOUNDS(row < xp && (FP4 || FP6 || row < kb) && w.r0 + g0 + j < in->Rp, status)) {
              const uint32_t o = o0 + (uint32_t)j * uxp;
              xs[o] = xv[j];
              ys[o] = yv[j];
              if constexpr (OP == kGopFp8) vn[row + v0 + (uint32_t)j * (uint32_t)kb] = xv[j] > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;
            }
          }
          if constexpr (FP6) {
            // E2M3 signs (+4: 0x18, -4: 0x38, outside the instance 0), sixteen spins per 12 bytes (value i
            // of a group at bits 6 i .. 6 i + 5, little-endian). The warp ballots each column's valid and
            // negative spins, then lane l packs column l / 2, group l % 2: four spins at a time, bit b of a
            // mask goes to bit 6 b (spread4), times 0x18 for the valid bits 3 and 4, shifted by 5 for the
            // sign bit; the three 32-bit words of the group are cut from those 24-bit pieces.
            uint32_t myv = 0, mys = 0;
#pragma unroll
            for (int j = 0; j < kGroup; ++j) {
              const bool ins = row < n && w.r0 + g0 + j < R;
              const uint32_t vm = __ballot_sync(0xffffffffu, ins);
              const uint32_t sm = __ballot_sync(0xffffffffu, ins && !(xv[j] > 0.0f));
              if ((lane >> 1) == j) {
                myv = vm;
                mys = sm;
              }
            }
            const int grp = lane & 1;
            const int r = w.r0 + g0 + (lane >> 1);
            const uint32_t v16 = (myv >> (16 * grp)) & 0xFFFFu, s16 = (mys >> (16 * grp)) & 0xFFFFu;
            auto spread4 = [](uint32_t b) { return (b & 1u) | ((b & 2u) << 5) | ((b & 4u) << 10) | ((b & 8u) << 15); };
            uint32_t piece[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
              piece[k] = spread4((v16 >> (4 * k)) & 0xFu) * 0x18u | (spread4((s16 >> (4 * k)) & 0xFu) << 5);
            const uint32_t gbyte = (uint32_t)((w.m0 + 32 * q) / 16 + grp) * 12u;
            if (r < R && SB_BOUNDS(r < in->Rp && gbyte + 12u <= (uint32_t)kb, status)) {
              uint32_t *dst = reinterpret_cast<uint32_t *>(vn + (size_t)r * (uint32_t)kb + gbyte);
              dst[0] = piece[0] | (piece[1] << 24);
              dst[1] = (piece[1] >> 8) | (piece[2] << 16);
              dst[2] = (piece[2] >> 16) | (piece[3] << 8);
            }
          }
          if constexpr (FP4) {
#pragma unroll
            for (int s = 0; s < kSub; ++s) {
              // spins 2s (even lane, low nibble) and 2s + 1 (odd lane, high nibble) share a byte: per
              // 16 columns, the even lane writes replicas c..c+7, the odd lane c+8..c+15
              const int c = g0 + 16 * s;
              uint32_t nib_lo = 0, nib_hi = 0;
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const bool ins = row < n && w.r0 + c + j < R;
                const uint32_t nib = ins ? (xv[16 * s + j] > 0.0f ? kE2m1Plus : kE2m1Minus) : 0u;
                if (j < 8) nib_lo |= nib << (4 * j);
                else nib_hi |= nib << (4 * (j - 8));
              }
              const bool odd = (lane & 1) != 0;
              const uint32_t o_lo = __shfl_xor_sync(0xffffffffu, nib_lo, 1);
              const uint32_t o_hi = __shfl_xor_sync(0xffffffffu, nib_hi, 1);
              const uint32_t lo_n = odd ? o_hi : nib_lo, hi_n = odd ? nib_hi : o_lo;
              const int row_e = row & ~1;
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int r = w.r0 + c + (odd ? 8 : 0) + j;
                if (row_e < n && r < R && SB_BOUNDS((row_e >> 1) < kb && r < in->Rp, status))
                  vn[(size_t)r * kb + (row_e >> 1)] =
                      (uint8_t)(((lo_n >> (4 * j)) & 0xFu) | (((hi_n >> (4 * j)) & 0xFu) << 4));
              }
            }
          }
        }
        if constexpr (kEOnly) {
#pragma unroll
          for (int j = 0; j < kGroup; ++j) {
            float v = e2[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) ered[q][g0 + j] = v;
          }
        }
        if (gi + 1 < kGroups) {
#pragma unroll
          for (int j = 0; j < kGroup; ++j) {
            xv[j] = xn[j];
            if constexpr (!kEOnly) yv[j] = yn[j];
          }
        }
      }
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&acce_bar[ab]);
      if constexpr (kEOnly) {
        epi_sync();
        for (int c = threadIdx.x - kEpiFirstThread; c < NR; c += kEpiThreads) {
          const int r = w.r0 + c;
          if (r < R) {
            const double sum = ((double)ered[0][c] + (double)ered[1][c]) + ((double)ered[2][c] + (double)ered[3][c]);
            atomicAdd(in->energy + r, 0.5 * sum);
          }
        }
        epi_sync();
      }
    }
  }
  if (!ok) atomicOr(status, kErrWaitTimeout);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kCols);
  }
}

template <int NR>
constexpr int grouped_stages() {
  return (208 * 1024) / (kBM * kChunkBytes + NR * kChunkBytes) > 8 ? 8 : (208 * 1024) / (kBM * kChunkBytes + NR * kChunkBytes);
}

template <int NR>
constexpr size_t grouped_smem() {
  return (size_t)grouped_stages<NR>() * (kBM * kChunkBytes + NR * kChunkBytes) + 1024;
}

}  // namespace tck
}  // namespace sbk
