// Plain FP32 SB path: one fused kernel per step, plus initial-state and energy kernels.
//
// Replaces, per step, the reference's two launches UpdateTwice<<<N/64,64>>> + cublasSgemv
// (SB/CUDA_GPU/m2_opt.cu:168-169) with one kernel that computes the field and the update:
//   * each CTA owns 8 rows of J (one warp per row) and up to 8 replicas;
//   * up to two replicas per CTA (the latency-bound case: one replica per trial), the CTA's J rows
//     and its replicas' x are staged into shared memory by bulk copies (cp.async.bulk) in
//     512-float chunks through an mbarrier ring of up to four stages (all of K in flight at once
//     for N <= 2048 and one replica); dSB takes sign(x) as it reads x. With more replicas per CTA
//     (bound by shared-memory loads of the replica vectors) J goes through a two-stage ring and the
//     replicas' chunk (signs for dSB) is staged once by the CTA's threads;
//   * consecutive steps overlap through programmatic dependent launch: a step's kernel starts
//     during the previous one's tail, requests its J rows, and waits for the previous step only
//     before it touches x;
//   * each warp forms its row's dot products with float4 shared-memory reads and a shuffle
//     reduction; the fields then go through shared memory to consecutive threads, which apply the
//     SB update (the aSB sub-steps in FP64 on one or two warps per CTA) and write x (ping-pong)
//     and y (in place: every element has exactly one owner);
//   * dSB also reduces -1/2 s_i f_i - h_i s_i per replica (block reduction + one atomic per
//     replica), which is the energy of s(t) and costs nothing extra because f = J s(t).
// Every wait is bounded: a timeout sets a status bit and the kernel returns.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "sb_internal.h"
#include "sb_math.cuh"
#include "sb_ptx.cuh"

namespace sbk {
namespace {

constexpr int kRows = 8;
constexpr int kThreads = 256;
constexpr int kChunk = 512;  // floats per row per stage
constexpr int kMaxRB = 8;
constexpr int kMaxStages = 4;
// Shared memory: up to two replicas per CTA a ring of up to kStageBudget bytes (all of K for
// N <= 2048 at one replica, 3 CTAs per SM); with more, the two-stage J ring and one replica
// chunk buffer (48 KB, 4 CTAs per SM).
constexpr int kStageBudget = 72 * 1024;
constexpr size_t kWideSmem = (size_t)(2 * kRows * kChunk + kMaxRB * kChunk) * sizeof(float);
constexpr size_t kSmemBytes = kStageBudget;

__device__ __forceinline__ float sgn(float v) { return v > 0.0f ? 1.0f : -1.0f; }

// The dSB / bSB update, the exact operation order the CPU oracle restates.
__device__ __forceinline__ void sb_update(float f, float hv, float pump, float c0, float dt,
                                          float dta0, float &x, float &y) {
  float fv = __fadd_rn(f, hv);
  float g = __fmul_rn(c0, fv);
  float force = __fmaf_rn(-pump, x, g);
  y = __fmaf_rn(dt, force, y);
  x = __fmaf_rn(dta0, y, x);
  if (fabsf(x) > 1.0f) {
    x = copysignf(1.0f, x);
    y = 0.0f;
  }
}

// aSB local sub-steps (UpdateTwice, SB/CUDA_GPU/m2_opt.cu:66-71): the reference evaluates them in
// double because its constants are double literals; explicit _rn ops keep the order fixed.
__device__ __forceinline__ void asb_local(float &x, float &y, float amp, int m, float mts_dt,
                                          float detune, float kerr) {
  double dd = detune, dk = kerr, dh = mts_dt, da = amp;
  for (int s = 0; s < m; ++s) {
    x = (float)__dadd_rn((double)x, __dmul_rn(__dmul_rn(dd, (double)y), dh));
    double lx = (double)x;
    double x3 = __dmul_rn(__dmul_rn(__dmul_rn(dk, lx), lx), lx);
    double lin = __dmul_rn(__dadd_rn(dd, -da), lx);
    y = (float)__dadd_rn((double)y, -__dmul_rn(dh, __dadd_rn(x3, lin)));
  }
}

template <typename Acc>
struct RowAcc {
  Acc v[kMaxRB];
};

// One chunk of a row's dot products with rb replica vectors in shared memory (row stride `stride`
// floats); SIGN: use sign(v).
template <bool SIGN, typename Acc>
__device__ __forceinline__ void dot_chunk(const float4 *jr, const float *sx, int stride, int len, int rb,
                                          int lane, Acc (&acc)[kMaxRB]) {
  for (int q = lane; q < (len >> 2); q += 32) {
    const float4 jv = jr[q];
#pragma unroll
    for (int rr = 0; rr < kMaxRB; ++rr) {
      if (rr < rb) {
        float4 vv = reinterpret_cast<const float4 *>(sx + rr * stride)[q];
        if (SIGN) {
          vv.x = sgn(vv.x);
          vv.y = sgn(vv.y);
          vv.z = sgn(vv.z);
          vv.w = sgn(vv.w);
        }
        if constexpr (sizeof(Acc) == 8) {
          acc[rr] += (double)jv.x * (double)vv.x + (double)jv.y * (double)vv.y +
                     (double)jv.z * (double)vv.z + (double)jv.w * (double)vv.w;
        } else {
          acc[rr] = __fmaf_rn(jv.x, vv.x, acc[rr]);
          acc[rr] = __fmaf_rn(jv.y, vv.y, acc[rr]);
          acc[rr] = __fmaf_rn(jv.z, vv.z, acc[rr]);
          acc[rr] = __fmaf_rn(jv.w, vv.w, acc[rr]);
        }
      }
    }
  }
}

// Butterfly sums: every lane of the row's warp ends with the row's fields.
template <typename Acc>
__device__ __forceinline__ void warp_sums(Acc (&acc)[kMaxRB]) {
#pragma unroll
  for (int rr = 0; rr < kMaxRB; ++rr) {
    Acc v = acc[rr];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    acc[rr] = v;
  }
}

// Field of the CTA's rows for at most two replicas per CTA, where a step is latency-bound. Stage s
// of the ring holds J[rows][kChunk] and x[rb][kChunk] of one chunk of K, both copied by
// cp.async.bulk and counted on full[s]; `stages` chunks are in flight (all of K for N <= 2048 at
// one replica). dSB takes sign(x) as it reads x. J does not change during a solve, so the first
// stages' J rows are requested before grid_dep_wait: when this launch overlaps the previous step's
// kernel, those copies run during its tail and only the x copies wait for it.
template <int MODE, typename Acc>
__device__ __forceinline__ bool field_rows_ring(const float *__restrict__ J, int jp, int row0, int rows,
                                                const float *__restrict__ xv, int xp, int r0, int rb,
                                                int stages, float *smem, uint64_t *full,
                                                Acc (&acc)[kMaxRB], size_t jlim, size_t xlim,
                                                uint32_t *status) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nchunks = (jp + kChunk - 1) / kChunk;
  const int stage_floats = (kRows + rb) * kChunk;
  auto len_of = [&](int c) { return min(kChunk, jp - c * kChunk); };
  auto issue_j = [&](int c) {
    const int s = c % stages;
    const uint32_t bytes = (uint32_t)len_of(c) * 4u;
    ptx::mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)(rows + rb));
    for (int w = 0; w < rows; ++w)
      if (SB_BOUNDS((size_t)(row0 + w) * jp + c * kChunk + bytes / 4 <= jlim, status))
        ptx::bulk_g2s(smem + s * stage_floats + w * kChunk, J + (size_t)(row0 + w) * jp + c * kChunk,
                      bytes, &full[s]);
  };
  auto issue_x = [&](int c) {
    const int s = c % stages;
    const uint32_t bytes = (uint32_t)len_of(c) * 4u;
    for (int rr = 0; rr < rb; ++rr)
      if (SB_BOUNDS((size_t)(r0 + rr) * xp + c * kChunk + bytes / 4 <= xlim, status))
        ptx::bulk_g2s(smem + s * stage_floats + (kRows + rr) * kChunk,
                      xv + (size_t)(r0 + rr) * xp + c * kChunk, bytes, &full[s]);
  };
  const int pre = min(nchunks, stages);
  if (tid == 0)
    for (int c = 0; c < pre; ++c) issue_j(c);
  // every thread: x (and, in the caller, y) are the previous step's output
  ptx::grid_dep_wait();
  ptx::grid_dep_launch();
  if (tid == 0)
    for (int c = 0; c < pre; ++c) issue_x(c);
  bool ok = true;
  for (int c = 0; c < nchunks; ++c) {
    const int s = c % stages;
    if (!ptx::mbar_wait(&full[s], (uint32_t)((c / stages) & 1))) ok = false;
    if (warp < rows && ok)
      dot_chunk<MODE == 1>(reinterpret_cast<const float4 *>(smem + s * stage_floats + warp * kChunk),
                           smem + s * stage_floats + kRows * kChunk, kChunk, len_of(c), rb, lane, acc);
    if (c + stages < nchunks) {
      __syncthreads();  // every warp is done with stage s before it is refilled
      if (tid == 0 && ok) {
        issue_j(c + stages);
        issue_x(c + stages);
      }
    }
  }
  return ok;
}

// Field of the CTA's rows for three to eight replicas per CTA, where a step is bound by
// shared-memory loads of the replica vectors: J rows through a two-stage ring of bulk copies, the
// replicas' chunk (signs for dSB) staged once by the CTA's threads with 128-bit loads and shared by
// the eight row warps. Ring: sJ[2][kRows][kChunk], then sV[kMaxRB][kChunk]. These launches do not
// overlap the previous step's (a wave of many CTAs gains nothing from it), so nothing here waits.
template <int MODE, typename Acc>
__device__ __forceinline__ bool field_rows_wide(const float *__restrict__ J, int jp, int row0, int rows,
                                                const float *__restrict__ xv, int xp, int r0, int rb,
                                                float *smem, uint64_t *full, Acc (&acc)[kMaxRB], size_t jlim,
                                                size_t xlim, uint32_t *status) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nchunks = (jp + kChunk - 1) / kChunk;
  float *sJ = smem, *sV = smem + 2 * kRows * kChunk;
  auto issue = [&](int c) {
    const int k0 = c * kChunk;
    const uint32_t bytes = (uint32_t)min(kChunk, jp - k0) * 4u;
    ptx::mbar_arrive_expect_tx(&full[c & 1], bytes * (uint32_t)rows);
    for (int w = 0; w < rows; ++w)
      if (SB_BOUNDS((size_t)(row0 + w) * jp + k0 + bytes / 4 <= jlim, status))
        ptx::bulk_g2s(sJ + ((c & 1) * kRows + w) * kChunk, J + (size_t)(row0 + w) * jp + k0, bytes,
                      &full[c & 1]);
  };
  if (tid == 0) {
    issue(0);
    if (nchunks > 1) issue(1);
  }
  bool ok = true;
  for (int c = 0; c < nchunks; ++c) {
    const int k0 = c * kChunk;
    const int len = min(kChunk, jp - k0);
    for (int rr = 0; rr < rb; ++rr) {
      const float *src = xv + (size_t)(r0 + rr) * xp + k0;
      float *dst = sV + rr * kChunk;
      for (int q = tid * 4; q < len; q += kThreads * 4) {
        if (!SB_BOUNDS((size_t)(r0 + rr) * xp + k0 + q + 4 <= xlim, status)) continue;
        float4 t = *reinterpret_cast<const float4 *>(src + q);
        if (MODE == 1) {
          t.x = sgn(t.x);
          t.y = sgn(t.y);
          t.z = sgn(t.z);
          t.w = sgn(t.w);
        }
        *reinterpret_cast<float4 *>(dst + q) = t;
      }
    }
    if (!ptx::mbar_wait(&full[c & 1], (uint32_t)((c >> 1) & 1))) ok = false;
    __syncthreads();
    if (warp < rows && ok)
      dot_chunk<false>(reinterpret_cast<const float4 *>(sJ + ((c & 1) * kRows + warp) * kChunk), sV,
                       kChunk, len, rb, lane, acc);
    __syncthreads();
    if (tid == 0 && c + 2 < nchunks && ok) issue(c + 2);
  }
  return ok;
}

// The CTA's fields; WIDE (the launch's replicas per CTA > 2) selects the layout at compile time
// (one layout per kernel instantiation). Returns the CTA-wide verdict of the bounded waits; every
// lane of row w's warp holds its fields.
template <int MODE, bool WIDE, typename Acc>
__device__ __forceinline__ bool field_rows(const float *__restrict__ J, int jp, int row0, int rows,
                                           const float *__restrict__ xv, int xp, int r0, int rb, int stages,
                                           float *smem, uint64_t *full, Acc (&acc)[kMaxRB], size_t jlim,
                                           size_t xlim, uint32_t *status) {
#pragma unroll
  for (int q = 0; q < kMaxRB; ++q) acc[q] = Acc(0);
  bool ok;
  if constexpr (WIDE)
    ok = field_rows_wide<MODE, Acc>(J, jp, row0, rows, xv, xp, r0, rb, smem, full, acc, jlim, xlim, status);
  else
    ok = field_rows_ring<MODE, Acc>(J, jp, row0, rows, xv, xp, r0, rb, stages, smem, full, acc, jlim, xlim,
                                    status);
  // every thread leaves with the same verdict, so no thread skips a later barrier
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  warp_sums(acc);
  return ok;
}

template <int VARIANT, bool WIDE>
__global__ void __launch_bounds__(kThreads) plain_step_kernel(PlainStep a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ double red[kRows][kMaxRB];
  __shared__ float fsh[kRows][kMaxRB];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kRows;
  const int r0 = blockIdx.y * a.rb;
  const int rb = min(a.rb, a.R - r0);
  const int rows = min(kRows, a.n - row0);
  if (rows <= 0 || rb <= 0 || rb > kMaxRB || a.stages < 1 || a.stages > kMaxStages) {
    ptx::grid_dep_wait();
    if (tid == 0) atomicOr(a.status, kErrBadShape);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < a.stages; ++s) ptx::mbar_init(&full[s], 1);
    ptx::fence_mbar_init();
  }
  if (tid < kRows * kMaxRB) red[tid / kMaxRB][tid % kMaxRB] = 0.0;
  __syncthreads();
  float acc[kMaxRB];
  const bool ok = field_rows<VARIANT == 2 ? 1 : 0, WIDE, float>(
      a.J, a.jp, row0, rows, a.x_in, a.xp, r0, rb, a.stages, reinterpret_cast<float *>(smem), full, acc,
      (size_t)a.n * a.jp, (size_t)a.R * a.xp, a.status);
  if (!ok) {
    if (tid == 0) atomicOr(a.status, kErrWaitTimeout);
    return;
  }
  // The fields go through shared memory so that the update runs on consecutive threads (thread
  // t: row t % kRows, replica t / kRows) instead of one lane in each row's warp: the aSB local
  // sub-steps are FP64, and packing the CTA's elements into one or two warps issues that FP64
  // work once per CTA instead of once per row.
  if (lane == 0 && warp < rows) {
#pragma unroll
    for (int rr = 0; rr < kMaxRB; ++rr)
      if (rr < rb) fsh[warp][rr] = acc[rr];
  }
  __syncthreads();
  const int w = tid % kRows, rr = tid / kRows;
  if (rr < rb && w < rows) {
    const float f = fsh[w][rr];
    const int i = row0 + w, r = r0 + rr;
    const size_t k = (size_t)r * a.xp + i;
    float x = a.x_in[k], y = a.y[k];
    const float hv = a.h ? a.h[i] : 0.0f;
    if (VARIANT == 0) {
      y = __fmaf_rn(a.coeff, f, y);
      if (a.do_local) asb_local(x, y, a.amp_next, a.m, a.mts_dt, a.detune, a.kerr);
    } else {
      const float s = sgn(x);
      if (VARIANT == 2 && a.energy)
        red[w][rr] = -0.5 * (double)s * (double)f - (double)hv * (double)s;
      sb_update(f, hv, a.pump, a.c0, a.dt, a.dta0, x, y);
    }
    if (SB_BOUNDS(k < (size_t)a.R * a.xp && i < a.n, a.status)) {
      a.x_out[k] = x;
      a.y[k] = y;
    }
  }
  if (VARIANT == 2 && a.energy) {
    __syncthreads();
    if (tid < rb) {
      double e = 0.0;
      for (int q = 0; q < rows; ++q) e += red[q][tid];
      atomicAdd(a.energy + r0 + tid, e);
    }
  }
}

template <typename Acc, bool WIDE>
__global__ void __launch_bounds__(kThreads) plain_energy_kernel(PlainEnergy a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ double red[kRows][kMaxRB];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kRows;
  const int r0 = blockIdx.y * a.rb;
  const int rb = min(a.rb, a.R - r0);
  const int rows = min(kRows, a.n - row0);
  if (rows <= 0 || rb <= 0 || rb > kMaxRB || a.stages < 1 || a.stages > kMaxStages) {
    ptx::grid_dep_wait();
    if (tid == 0) atomicOr(a.status, kErrBadShape);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < a.stages; ++s) ptx::mbar_init(&full[s], 1);
    ptx::fence_mbar_init();
  }
  if (tid < kRows * kMaxRB) red[tid / kMaxRB][tid % kMaxRB] = 0.0;
  __syncthreads();
  Acc acc[kMaxRB];
  const bool ok =
      field_rows<1, WIDE, Acc>(a.J, a.jp, row0, rows, a.x, a.xp, r0, rb, a.stages,
                               reinterpret_cast<float *>(smem), full, acc, (size_t)a.n * a.jp, (size_t)a.R * a.xp,
                               a.status);
  if (!ok) {
    if (tid == 0) atomicOr(a.status, kErrWaitTimeout);
    return;
  }
  if (warp < rows && lane < rb) {
    Acc f = Acc(0);
#pragma unroll
    for (int rr = 0; rr < kMaxRB; ++rr)
      if (rr == lane) f = acc[rr];
    const int i = row0 + warp, r = r0 + lane;
    const double s = sgn(a.x[(size_t)r * a.xp + i]);
    const double hv = a.h ? (double)a.h[i] : 0.0;
    red[warp][lane] = -0.5 * s * (double)f - hv * s;
  }
  __syncthreads();
  if (tid < rb) {
    double e = 0.0;
    for (int w = 0; w < rows; ++w) e += red[w][tid];
    atomicAdd(a.energy + r0 + tid, e);
  }
}

// ---- NMFA: noisy mean-field annealing (NMFA/CUDA_GPU/src/nmfa.cu:54-140) ----
// The reference runs one CTA per sample and one thread per spin with its row of J in registers; here
// the samples are the replicas of the plain kernel's layout (8 rows of J per CTA, up to 8 samples),
// and each of a stage's two sweeps is one fused launch. A sweep reads the states of the previous
// sweep (the reference's sweeps inside a stage have no barrier between one warp's writes and
// another's reads; for up to 32 spins, one warp, it computes exactly this).

template <bool WIDE>
__global__ void __launch_bounds__(kThreads) nmfa_sweep_kernel(NmfaSweep a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ float fsh[kRows][kMaxRB];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kRows;
  const int r0 = blockIdx.y * a.rb;
  const int rb = min(a.rb, a.R - r0);
  const int rows = min(kRows, a.n - row0);
  if (rows <= 0 || rb <= 0 || rb > kMaxRB || a.stages < 1 || a.stages > kMaxStages) {
    ptx::grid_dep_wait();
    if (tid == 0) atomicOr(a.status, kErrBadShape);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < a.stages; ++s) ptx::mbar_init(&full[s], 1);
    ptx::fence_mbar_init();
  }
  __syncthreads();
  float acc[kMaxRB];
  const bool ok = field_rows<0, WIDE, float>(a.J, a.jp, row0, rows, a.s_in, a.xp, r0, rb, a.stages,
                                             reinterpret_cast<float *>(smem), full, acc, (size_t)a.n * a.jp,
                                             (size_t)a.R * a.xp, a.status);
  if (!ok) {
    if (tid == 0) atomicOr(a.status, kErrWaitTimeout);
    return;
  }
  if (lane == 0 && warp < rows) {
#pragma unroll
    for (int q = 0; q < kMaxRB; ++q)
      if (q < rb) fsh[warp][q] = acc[q];
  }
  __syncthreads();
  const int w = tid % kRows, rr = tid / kRows;
  if (rr < rb && w < rows) {
    const int i = row0 + w, r = r0 + rr;
    const size_t k = (size_t)r * a.xp + i;
    const size_t plane = (size_t)a.R * a.xp;
    if (!SB_BOUNDS(k < plane && i < a.n, a.status)) return;
    float z;
    if (a.first) {
      uint32_t wd[5];
#pragma unroll
      for (int q = 0; q < 5; ++q) wd[q] = a.rng[q * plane + k];
      float z1;
      sbm::nmfa_gauss(wd, a.noise, z, z1);
#pragma unroll
      for (int q = 0; q < 5; ++q) a.rng[q * plane + k] = wd[q];
      a.z1[k] = z1;
    } else {
      z = a.z1[k];
    }
    const float st = sbm::nmfa_update(fsh[w][rr], a.norm[i], z, a.beta, a.keep, a.mix, a.s_in[k]);
    a.s_out[k] = st;
    if (a.samples) a.samples[(size_t)r * a.n + i] = st > 0.0f ? 1 : -1;
  }
}

// norm[i] = -1 / sqrt(sum_j |J_ij|) (nmfa.cu:88-93) with the sum in double over j in index order and
// the result rounded once to float (the host oracle's operations, IEEE double); 0 for an empty row.
__global__ void nmfa_norms_kernel(const float *J, int n, int jp, float *norm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *row = J + (size_t)i * jp;
  double a = 0.0;
  for (int j = 0; j < n; ++j) a = __dadd_rn(a, fabs((double)row[j]));
  norm[i] = a > 0.0 ? __double2float_rn(__ddiv_rn(-1.0, __dsqrt_rn(a))) : 0.0f;
}

// The same norms for integer couplings (n max|J| < 2^53): every partial sum is an exact integer in
// double, so one warp per row sums coalesced strips and a butterfly, with the sequential sum's value.
__global__ void nmfa_norms_int_kernel(const float *J, int n, int jp, float *norm) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= n) return;
  const float *row = J + (size_t)i * jp;
  double a = 0.0;
  for (int j = lane; j < n; j += 32) a += fabs((double)row[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) norm[i] = a > 0.0 ? __double2float_rn(__ddiv_rn(-1.0, __dsqrt_rn(a))) : 0.0f;
}

// samples[r][i] = s > 0 ? +1 : -1 (nmfa.cu:139) from the final states [R][xp]
__global__ void nmfa_signs_kernel(const float *s, int n, int R, int xp, int32_t *samples) {
  const size_t total = (size_t)n * R;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / n, i = e % n;
    samples[e] = s[r * xp + i] > 0.0f ? 1 : -1;
  }
}

// Initial words of (sample r, spin i), as nmfa.cu:62-76 seeds thread i of block r: t = seed + n r + i
// (32-bit), four xorshift32 steps (nmfa.cu:43-47) giving words 0..3, the counter word 0.
__global__ void nmfa_seed_kernel(uint32_t *rng, int n, int R, int xp, uint32_t seed) {
  const size_t total = (size_t)n * R, plane = (size_t)R * xp;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / n, i = e % n, k = r * xp + i;
    uint32_t t = seed + (uint32_t)n * (uint32_t)r + (uint32_t)i;
    for (int q = 0; q < 4; ++q) {
      t ^= t << 13;
      t ^= t >> 17;
      t ^= t << 5;
      rng[q * plane + k] = t;
    }
    rng[4 * plane + k] = 0u;
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return z;
}

__device__ __forceinline__ float uniform_value(uint64_t seed, uint64_t e) {
  const uint64_t z = mix64(seed + 0x9E3779B97F4A7C15ULL * (e + 1));
  const uint32_t u = (uint32_t)(z >> 40);
  const float f = __fmul_rn((float)u, 5.9604644775390625e-08f);
  const float t = __fadd_rn(__fmul_rn(f, 2.0f), -1.0f);
  return __fmul_rn(t, 0.1f);
}

__global__ void init_uniform_kernel(float *x, float *y, int n, int R, int xp, uint64_t seed) {
  const size_t total = (size_t)n * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / n, i = k % n;
    const uint64_t e = 2 * (uint64_t)k;
    x[r * xp + i] = uniform_value(seed, e);
    y[r * xp + i] = uniform_value(seed, e + 1);
  }
}

// prepare_points (SB/CUDA_GPU/m2_opt.cu:48-56) with per-spin state i (m2_opt.cu:136-137);
// replica r gets trial r's draws. The float division by (float)MAX = 2^32 is an exact scaling.
__global__ void init_reference_kernel(float *x, float *y, int n, int R, int xp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t st = (uint32_t)i;
  for (int r = 0; r < R; ++r) {
    uint32_t u[2];
    for (int d = 0; d < 2; ++d) {
      st ^= st << 13;
      st ^= st >> 17;
      st ^= st << 5;
      u[d] = st;
    }
    const float qx = __fmul_rn(__uint2float_rn(u[0]), 2.3283064365386963e-10f);
    const float qy = __fmul_rn(__uint2float_rn(u[1]), 2.3283064365386963e-10f);
    x[(size_t)r * xp + i] = __double2float_rn(__ddiv_rn((double)qx, 10.0));
    y[(size_t)r * xp + i] = __double2float_rn(__ddiv_rn((double)qy, 10.0));
  }
}

__global__ void asb_local_kernel(float *x, float *y, int n, int R, int xp, float amp, int m,
                                 float mts_dt, float detune, float kerr) {
  const size_t total = (size_t)n * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / n, i = k % n, idx = r * xp + i;
    float lx = x[idx], ly = y[idx];
    asb_local(lx, ly, amp, m, mts_dt, detune, kerr);
    x[idx] = lx;
    y[idx] = ly;
  }
}

__global__ void pad_rows_f32_kernel(const float *src, float *dst, int n, int jp) {
  const size_t total = (size_t)n * jp;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / jp, j = k % jp;
    dst[k] = j < (size_t)n ? src[i * n + j] : 0.0f;
  }
}

int grid_for(size_t total) {
  size_t g = (total + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g > 0 ? g : 1);
}


// ---------------------------------------------------------------------------------------------
// Plain FP32 solves (aSB, bSB, dSB, and NMFA sweeps), the whole solve in one cooperative launch
// (PlainPersist). Warp w of CTA (c, r) owns row i = 16 c + w of replica r: its J row sits in the
// lanes' registers (lane L: float4 groups g = L + 32 k, k < kPersistGroups, the order dot_chunk
// sums in), its x, y in registers too. A dSB step needs sign(x(t)) of every spin; CTA c's 16 signs
// travel in one 64-bit word
// (tag t + 1 << 32 | bit w = x_i <= 0) at words[t & 1][r][c]: the tag is the flag, so one L2 round
// trip per step moves all the data; the thread that polls a word writes its 16 signs into shared
// memory as +-1.0, so the field sums the same products as the bSB / aSB form, which exchanges x
// itself as sixteen tagged words per CTA. A CTA rewrites parity t & 1 with step t + 2 only after
// every CTA has published step t + 1, which each did after reading all of step t's words.
constexpr int kPersistThreads = 32 * kPersistRows;
constexpr int kPersistGroups = kPersistMaxJp / 128;  // float4 groups per lane

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <int VARIANT>
__global__ void __launch_bounds__(kPersistThreads, 1) plain_persist_kernel(PlainPersist a) {
  // dSB exchanges signs: one word per CTA (tag << 32 | 16 sign bits). bSB / aSB exchange x: the 16
  // words of a CTA's line are its rows' (tag << 32 | bits of x), one written by each warp.
  constexpr bool kSigns = VARIANT == 2;
  __shared__ __align__(16) float xs[kPersistMaxJp];  // x(t) of every spin (dSB: its sign, +-1)
  __shared__ uint32_t sout[kPersistRows];
  __shared__ float sx[kPersistRows], sy[kPersistRows];  // aSB: the rows' x, y for the FP64 sub-steps
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c = blockIdx.x, r = blockIdx.y, G = gridDim.x;
  const int row = c * kPersistRows + warp;
  const bool have = row < a.n;
  const int ng = a.jp >> 2;  // float4 groups of a row
  if (G * kPersistRows < a.n || G > kPersistMaxJp / kPersistRows || ng > kPersistGroups * 32 || ng > 4 * G ||
      r >= a.R) {
    if (tid == 0) atomicOr(a.status, kErrBadShape);
    return;
  }
  float4 jr[kPersistGroups];
#pragma unroll
  for (int k = 0; k < kPersistGroups; ++k) {
    const int g = lane + 32 * k;
    jr[k] = (have && g < ng && SB_BOUNDS((size_t)row * a.jp + 4 * g + 4 <= (size_t)a.n * a.jp, a.status))
                ? reinterpret_cast<const float4 *>(a.J + (size_t)row * a.jp)[g]
                : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const size_t k_xy = (size_t)r * a.xp + row;
  float x = 0.0f, y = 0.0f;
  if (have && SB_BOUNDS(k_xy < (size_t)a.R * a.xp, a.status)) {
    x = a.x_in[k_xy];
    if constexpr (VARIANT != 3) y = a.y[k_xy];
  }
  const float hv = (have && a.h) ? a.h[row] : 0.0f;
  // NMFA: the row norm, the spin's XORWOW words and the stage's second Gaussian sample (drawn with
  // the first on the stage's first sweep, used on its second)
  const size_t plane = (size_t)a.R * a.xp;
  float nv = 0.0f, z1 = 0.0f;
  uint32_t wd[5] = {0u, 0u, 0u, 0u, 0u};
  if constexpr (VARIANT == 3) {
    if (have && SB_BOUNDS(k_xy < plane, a.status)) {
      nv = a.norm[row];
#pragma unroll
      for (int q = 0; q < 5; ++q) wd[q] = a.rng[q * plane + k_xy];
    }
  }
  // one 128-byte line per CTA: its store(s) and the other CTAs' polls share no line with any other
  // CTA's words
  constexpr int kLine = 16;                                       // words per line
  unsigned long long *wr = a.words + (size_t)r * G * kLine;      // parity 0 of replica r
  const size_t par = (size_t)a.R * G * kLine;                     // parity stride
  // rows past n publish x = 0 (sign -1), as the per-step kernel reads padding spins
  auto publish = [&](int t) {  // x(t) or its signs, with tag t + 1
    const unsigned long long tag = (unsigned long long)(uint32_t)(t + 1) << 32;
    unsigned long long *line = wr + (size_t)(t & 1) * par + (size_t)c * kLine;
    if constexpr (kSigns) {
      if (lane == 0) sout[warp] = (!have || !(x > 0.0f)) ? 1u : 0u;  // sgn: x > 0 -> +1, else -1
      __syncthreads();
      if (warp == 0) {
        const uint32_t b = __ballot_sync(0xffffffffu, lane < kPersistRows && sout[lane] != 0u);
        if (lane == 0) st_relaxed_u64(line, tag | b);
      }
    } else {
      if (lane == 0) st_relaxed_u64(line + warp, tag | __float_as_uint(have ? x : 0.0f));
      __syncthreads();
    }
  };
  // one word with tag t + 1 into v: a first load, then bounded polling; false when it gave up
  auto poll = [&](const unsigned long long *src, int t, unsigned long long &v) -> bool {
    v = ld_relaxed_u64(src);
    if ((uint32_t)(v >> 32) == (uint32_t)(t + 1)) return true;
    const long long t0 = clock64();
    int spins = 0;
    do {
      if (++spins > 8) __nanosleep(32);
      v = ld_relaxed_u64(src);
      if (clock64() - t0 > ptx::kWaitCycles) return false;
    } while ((uint32_t)(v >> 32) != (uint32_t)(t + 1));
    return true;
  };
  // x(t) of every spin into xs (dSB: the signs as +-1.0); false when a wait gave up
  auto gather = [&](int t) -> bool {
    if constexpr (kSigns) {
      // thread q < G polls CTA q's word and writes its 16 signs (bit w set: spin 16 q + w is -1)
      if (tid >= G) return true;
      const unsigned long long *src = wr + (size_t)(t & 1) * par + (size_t)tid * kLine;
      unsigned long long v;
      if (!poll(src, t, v)) return false;
      const uint32_t b = (uint32_t)v;
      float4 *dst = reinterpret_cast<float4 *>(xs) + 4 * tid;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        dst[k] = make_float4((b >> (4 * k)) & 1u ? -1.0f : 1.0f, (b >> (4 * k + 1)) & 1u ? -1.0f : 1.0f,
                             (b >> (4 * k + 2)) & 1u ? -1.0f : 1.0f, (b >> (4 * k + 3)) & 1u ? -1.0f : 1.0f);
      return true;
    } else {
      // sixteen threads read a CTA's line together (one 128-byte request per line and poll, where
      // one thread per line took sixteen): thread tid takes word tid % 16 of lines tid / 16 + 32 k,
      // and each warp polls its lines until all of their words carry this step's tag
      constexpr int kLinesPerPass = kPersistThreads / kLine;                   // 32
      constexpr int kPasses = kPersistMaxJp / kPersistRows / kLinesPerPass;    // G <= 128: 4
      const int w = tid & (kLine - 1), q0 = tid / kLine;
      const unsigned long long *base = wr + (size_t)(t & 1) * par;
      const uint32_t want = (uint32_t)(t + 1);
      unsigned long long wv[kPasses];
      const long long t0 = clock64();
      int spins = 0;
      for (;;) {
#pragma unroll
        for (int k = 0; k < kPasses; ++k) {
          const int q = q0 + kLinesPerPass * k;
          if (q < G) wv[k] = ld_relaxed_u64(base + (size_t)q * kLine + w);
        }
        bool mine = true;
#pragma unroll
        for (int k = 0; k < kPasses; ++k)
          if (q0 + kLinesPerPass * k < G) mine = mine && (uint32_t)(wv[k] >> 32) == want;
        if (__all_sync(0xffffffffu, mine)) break;
        if (__shfl_sync(0xffffffffu, (clock64() - t0 > ptx::kWaitCycles) ? 1 : 0, 0)) return false;
        if (++spins > 8) __nanosleep(32);
      }
#pragma unroll
      for (int k = 0; k < kPasses; ++k) {
        const int q = q0 + kLinesPerPass * k;
        if (q < G) xs[q * kLine + w] = __uint_as_float((uint32_t)wv[k]);
      }
      return true;
    }
  };
  publish(0);
  bool ok = true;
  float pump_next = a.steps > 0 ? a.pumps[0] : 0.0f;
  for (int t = 0; t < a.steps && ok; ++t) {
    const float pump = pump_next;
    if (t + 1 < a.steps) pump_next = a.pumps[t + 1];  // off the step's critical path
    ok = __syncthreads_and(gather(t) ? 1 : 0) != 0;
    if (!ok) break;
    // field of this warp's row over groups g = lane + 32 k (spins 4 g .. 4 g + 3)
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < kPersistGroups; ++k) {
      const int g = lane + 32 * k;
      if (g < ng) {
        const float4 jv = jr[k];
        const float4 xv = reinterpret_cast<const float4 *>(xs)[g];
        acc = __fmaf_rn(jv.x, xv.x, acc);
        acc = __fmaf_rn(jv.y, xv.y, acc);
        acc = __fmaf_rn(jv.z, xv.z, acc);
        acc = __fmaf_rn(jv.w, xv.w, acc);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (have) {
      if constexpr (VARIANT == 0) {
        // aSB: the coupling kick; the next step's local sub-steps follow below
        y = __fmaf_rn(a.coeff, acc, y);
      } else if constexpr (VARIANT == 3) {
        // NMFA sweep t (stage t / 2): the stage's first sweep draws its Gaussian pair
        float z;
        if ((t & 1) == 0)
          sbm::nmfa_gauss(wd, a.noise, z, z1);
        else
          z = z1;
        x = sbm::nmfa_update(acc, nv, z, pump, a.keep, a.mix, x);
      } else {
        sb_update(acc, hv, pump, a.c0, a.dt, a.dta0, x, y);
      }
    }
    if constexpr (VARIANT == 0) {
      if (t + 1 < a.steps) {
        // aSB: the next step's FP64 local sub-steps (none after the last) for the CTA's 16 rows in
        // 16 lanes of one warp, where one lane per row warp would issue 16 times the FP64 warp
        // instructions (FP64 is scarce on this part); rows past n run on x = y = 0 and stay 0
        if (lane == 0) {
          sx[warp] = x;
          sy[warp] = y;
        }
        __syncthreads();
        if (warp == 0 && lane < kPersistRows) {
          float lx = sx[lane], ly = sy[lane];
          asb_local(lx, ly, __fdiv_rn((float)(t + 1), (float)a.steps), a.m, a.mts_dt, a.detune, a.kerr);
          sx[lane] = lx;
          sy[lane] = ly;
        }
        __syncthreads();
        x = sx[warp];
        y = sy[warp];
      }
    }
    publish(t + 1);  // its barrier also ends this step's reads of xs (and sx, sy)
  }
  if (!ok) {
    if (tid == 0) atomicOr(a.status, kErrWaitTimeout);
    return;
  }
  if (have && lane == 0 && SB_BOUNDS(k_xy < (size_t)a.R * a.xp, a.status)) {
    a.x_out[k_xy] = x;
    if constexpr (VARIANT == 3) {
#pragma unroll
      for (int q = 0; q < 5; ++q) a.rng[q * plane + k_xy] = wd[q];
      if (a.samples) a.samples[(size_t)r * a.n + row] = x > 0.0f ? 1 : -1;
    } else {
      a.y[k_xy] = y;
    }
  }
}

}  // namespace

template <typename K>
void set_smem_once(K kernel, size_t bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct PlainAttrInit {
  PlainAttrInit() {
    set_smem_once(plain_step_kernel<0, false>, kSmemBytes);
    set_smem_once(plain_step_kernel<1, false>, kSmemBytes);
    set_smem_once(plain_step_kernel<2, false>, kSmemBytes);
    set_smem_once(plain_step_kernel<0, true>, kWideSmem);
    set_smem_once(plain_step_kernel<1, true>, kWideSmem);
    set_smem_once(plain_step_kernel<2, true>, kWideSmem);
    set_smem_once(plain_energy_kernel<float, false>, kSmemBytes);
    set_smem_once(plain_energy_kernel<double, false>, kSmemBytes);
    set_smem_once(plain_energy_kernel<float, true>, kWideSmem);
    set_smem_once(plain_energy_kernel<double, true>, kWideSmem);
    set_smem_once(nmfa_sweep_kernel<false>, kSmemBytes);
    set_smem_once(nmfa_sweep_kernel<true>, kWideSmem);
  }
};

void plain_attrs() { static PlainAttrInit once; }

void init_kernel_attributes() { plain_attrs(); }

// Ring depth for at most two replicas per CTA: as many stages as fit the budget (at least two), at
// most the number of chunks. A CTA with fewer replicas than the launch's (the last replica block)
// uses smaller stages inside the same ring.
size_t plain_smem(int rb, int stages) {
  return rb > 2 ? kWideSmem : (size_t)stages * (kRows + rb) * kChunk * sizeof(float);
}

int plain_stages(int jp, int rb) {
  const int nchunks = (jp + kChunk - 1) / kChunk;
  int s = kStageBudget / ((kRows + rb) * kChunk * (int)sizeof(float));
  s = s < 2 ? 2 : (s > kMaxStages ? kMaxStages : s);
  return s < nchunks ? s : nchunks;
}

template <int V, bool WIDE>
cudaError_t launch_step_variant(const PlainStep &a, dim3 grid, cudaStream_t st) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = plain_smem(a.rb, a.stages);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (a.overlap && !WIDE) ? 1 : 0;  // only the ring layout waits in grid_dep_wait
  return cudaLaunchKernelEx(&cfg, plain_step_kernel<V, WIDE>, a);
}

cudaError_t launch_plain_step(const PlainStep &a0, cudaStream_t st) {
  plain_attrs();
  if (a0.rb < 1 || a0.rb > kMaxRB || a0.jp % 4 || a0.xp % 4 || a0.jp > a0.xp || a0.jp < 4)
    return cudaErrorInvalidValue;
  PlainStep a = a0;
  a.stages = plain_stages(a.jp, a.rb);
  dim3 grid((a.n + kRows - 1) / kRows, (a.R + a.rb - 1) / a.rb);
  const bool wide = a.rb > 2;
  switch (a.variant) {
    case 0:
      return wide ? launch_step_variant<0, true>(a, grid, st) : launch_step_variant<0, false>(a, grid, st);
    case 1:
      return wide ? launch_step_variant<1, true>(a, grid, st) : launch_step_variant<1, false>(a, grid, st);
    case 2:
      return wide ? launch_step_variant<2, true>(a, grid, st) : launch_step_variant<2, false>(a, grid, st);
    default:
      return cudaErrorInvalidValue;
  }
}

int plain_persist_ctas(int n, int R, int jp) {
  if (n < 1 || R < 1 || jp < 4 || jp % 4 || jp > kPersistMaxJp) return 0;
  const int G = (n + kPersistRows - 1) / kPersistRows;
  if (jp / 4 > 4 * G) return 0;
  int dev = 0, sms = 0, per_sm = 1 << 30;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  // the variants differ in registers: the least co-resident one decides
  const void *ks[4] = {(const void *)plain_persist_kernel<0>, (const void *)plain_persist_kernel<1>,
                       (const void *)plain_persist_kernel<2>, (const void *)plain_persist_kernel<3>};
  for (const void *k : ks) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kPersistThreads, 0) != cudaSuccess) return 0;
    per_sm = b < per_sm ? b : per_sm;
  }
  const long long ctas = (long long)G * R;
  return ctas <= (long long)sms * per_sm ? (int)ctas : 0;
}

cudaError_t launch_plain_persist(const PlainPersist &a, cudaStream_t st) {
  if (plain_persist_ctas(a.n, a.R, a.jp) == 0 || a.xp < a.jp || a.steps < 0) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)((a.n + kPersistRows - 1) / kPersistRows), (unsigned)a.R);
  cfg.blockDim = dim3(kPersistThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every CTA waits on every other one's words
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  switch (a.variant) {
    case 0: return cudaLaunchKernelEx(&cfg, plain_persist_kernel<0>, a);
    case 1: return cudaLaunchKernelEx(&cfg, plain_persist_kernel<1>, a);
    case 2: return cudaLaunchKernelEx(&cfg, plain_persist_kernel<2>, a);
    case 3: return cudaLaunchKernelEx(&cfg, plain_persist_kernel<3>, a);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_plain_energy(const PlainEnergy &a0, bool fp64, cudaStream_t st) {
  plain_attrs();
  if (a0.rb < 1 || a0.rb > kMaxRB || a0.jp % 4 || a0.xp % 4 || a0.jp > a0.xp || a0.jp < 4)
    return cudaErrorInvalidValue;
  PlainEnergy a = a0;
  a.stages = plain_stages(a.jp, a.rb);
  dim3 grid((a.n + kRows - 1) / kRows, (a.R + a.rb - 1) / a.rb);
  const size_t smem = plain_smem(a.rb, a.stages);
  if (a.rb > 2) {
    if (fp64)
      plain_energy_kernel<double, true><<<grid, kThreads, smem, st>>>(a);
    else
      plain_energy_kernel<float, true><<<grid, kThreads, smem, st>>>(a);
  } else {
    if (fp64)
      plain_energy_kernel<double, false><<<grid, kThreads, smem, st>>>(a);
    else
      plain_energy_kernel<float, false><<<grid, kThreads, smem, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_nmfa_sweep(const NmfaSweep &a0, cudaStream_t st) {
  plain_attrs();
  if (a0.rb < 1 || a0.rb > kMaxRB || a0.jp % 4 || a0.xp % 4 || a0.jp > a0.xp || a0.jp < 4)
    return cudaErrorInvalidValue;
  NmfaSweep a = a0;
  a.stages = plain_stages(a.jp, a.rb);
  const bool wide = a.rb > 2;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((a.n + kRows - 1) / kRows, (a.R + a.rb - 1) / a.rb);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = plain_smem(a.rb, a.stages);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (a.overlap && !wide) ? 1 : 0;
  return wide ? cudaLaunchKernelEx(&cfg, nmfa_sweep_kernel<true>, a)
              : cudaLaunchKernelEx(&cfg, nmfa_sweep_kernel<false>, a);
}

cudaError_t launch_nmfa_norms(const float *J, int n, int jp, float *norm, bool integral, cudaStream_t st) {
  if (integral)
    nmfa_norms_int_kernel<<<(n + 7) / 8, 256, 0, st>>>(J, n, jp, norm);
  else
    nmfa_norms_kernel<<<(n + 127) / 128, 128, 0, st>>>(J, n, jp, norm);
  return cudaGetLastError();
}

cudaError_t launch_nmfa_signs(const float *s, int n, int R, int xp, int32_t *samples, cudaStream_t st) {
  nmfa_signs_kernel<<<grid_for((size_t)n * R), 256, 0, st>>>(s, n, R, xp, samples);
  return cudaGetLastError();
}

cudaError_t launch_nmfa_seed(uint32_t *rng, int n, int R, int xp, uint32_t seed, cudaStream_t st) {
  nmfa_seed_kernel<<<grid_for((size_t)n * R), 256, 0, st>>>(rng, n, R, xp, seed);
  return cudaGetLastError();
}

cudaError_t launch_init_uniform(float *x, float *y, int n, int R, int xp, uint64_t seed,
                                cudaStream_t st) {
  init_uniform_kernel<<<grid_for((size_t)n * R), 256, 0, st>>>(x, y, n, R, xp, seed);
  return cudaGetLastError();
}

cudaError_t launch_init_reference(float *x, float *y, int n, int R, int xp, cudaStream_t st) {
  init_reference_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, n, R, xp);
  return cudaGetLastError();
}

cudaError_t launch_asb_local(float *x, float *y, int n, int R, int xp, float amp, int m,
                             float mts_dt, float detune, float kerr, cudaStream_t st) {
  asb_local_kernel<<<grid_for((size_t)n * R), 256, 0, st>>>(x, y, n, R, xp, amp, m, mts_dt,
                                                            detune, kerr);
  return cudaGetLastError();
}

cudaError_t launch_pad_rows_f32(const float *src, float *dst, int n, int jp, cudaStream_t st) {
  pad_rows_f32_kernel<<<grid_for((size_t)n * jp), 256, 0, st>>>(src, dst, n, jp);
  return cudaGetLastError();
}

}  // namespace sbk
