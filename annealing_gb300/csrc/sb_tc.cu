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
//   * warps 2..9 (two per TMEM lane quadrant, each half of the replica columns) read the
//     accumulator, x and y with tcgen05.ld, apply the SB update with the exact operation order of
//     the CPU oracle, write x and y back to TMEM and the next step's operand V (sign as FP8/BF16,
//     or x as BF16 hi + lo) to global memory; the accumulator is double-buffered in TMEM so the
//     next contraction can start while the epilogue drains (split operands instead accumulate K in
//     segments, each folded by the epilogue into an FP32 sum rounded to nearest);
//   * steps are ordered by per-unit release/acquire flags instead of a grid barrier: a unit
//     publishes its V(t+1) chunk and the units of its replica column wait only for the chunks they
//     load (bounded spins).
// Operand dtypes: FP8 E4M3 holds +-1 and integers |J| <= 16 exactly; BF16 holds integers up to 256;
// BF16 hi + lo (J = Jh + Jl, x = xh + xl) gives ~16 bits for real values, with the three products
// Jh*xh + Jh*xl + Jl*xh accumulated in FP32. Integer fields are exact whenever every partial sum
// stays below 2^24 in magnitude, which holds for n * max|J| < 2^24.
// Every wait is bounded; a timeout sets a status bit, the kernel still frees its TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "sb_host.h"
#include "sb_tc_fp4.cuh"
#include "sb_tc_kernel.cuh"

namespace sbk {

// Kernel lookup by (variant, replica tile, epilogue mode); one definition per operand dtype, each
// in its own translation unit (sb_tc_fp8.cu, sb_tc_bf16.cu, sb_tc_split.cu).
bool tc_kernel_fp8(int variant, int nr, int emode, const void **k, size_t *smem);
bool tc_kernel_bf16(int variant, int nr, int emode, const void **k, size_t *smem);
bool tc_kernel_split(int variant, int nr, int emode, const void **k, size_t *smem);
bool tc_kernel_split16(int variant, int nr, int emode, const void **k, size_t *smem);
bool tc_kernel_fp4(int variant, int nr, int emode, int k_chunks, const void **k, size_t *smem, bool pair = false);

namespace {
using namespace tck;

// ---- operand preparation ----

// jscale: FP16 hi + lo, the power of two that brings max |J| into [2^12, 2^13)
__global__ void convert_j_kernel(const float *J, int n, int jp, uint8_t *a0, uint8_t *a1, int Np,
                                 int Kp, int dt, float jscale) {
  const size_t total = (size_t)Np * Kp;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / Kp, j = k % Kp;
    const float v = (i < (size_t)n && j < (size_t)n) ? J[i * jp + j] : 0.0f;
    if (dt == kTcFp16Split) {
      const float vs = __fmul_rn(v, jscale);
      const __half hi = __float2half_rn(vs);
      reinterpret_cast<__half *>(a0)[k] = hi;
      reinterpret_cast<__half *>(a1)[k] = __float2half_rn(__fsub_rn(vs, __half2float(hi)));
    } else if (dt == kTcFp8) {
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
                                 int Kp, int dt, int variant, float xscale) {
  const size_t total = (size_t)n * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / n, i = k % n;
    const float xv = x[r * xp + i];
    const size_t idx = r * Kp + i;
    if (dt == kTcFp8) {
      v0[idx] = xv > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;
    } else if ((dt == kTcBf16 && variant != 3) || variant == 2) {
      reinterpret_cast<uint16_t *>(v0)[idx] =
          dt == kTcFp16Split ? one16<kTcFp16Split>(!(xv > 0.0f)) : one16<kTcBf16>(!(xv > 0.0f));
    } else if (dt == kTcFp16Split) {
      const float xs = __fmul_rn(xv, xscale);
      const __half hi = __float2half_rn(xs);
      reinterpret_cast<__half *>(v0)[idx] = hi;
      reinterpret_cast<__half *>(v1)[idx] = __float2half_rn(__fsub_rn(xs, __half2float(hi)));
    } else {
      const __nv_bfloat16 hi = __float2bfloat16_rn(xv);
      reinterpret_cast<__nv_bfloat16 *>(v0)[idx] = hi;
      reinterpret_cast<__nv_bfloat16 *>(v1)[idx] = __float2bfloat16_rn(__fsub_rn(xv, __bfloat162float(hi)));
    }
  }
}

// Packed E2M1 operands: byte b of a row holds spins 2b (low nibble) and 2b + 1 (high nibble).
__global__ void convert_j_fp4_kernel(const float *J, int n, int jp, uint8_t *a, int Np, int Kb) {
  const size_t total = (size_t)Np * Kb;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / Kb, j = 2 * (k % Kb);
    const float v0 = (i < (size_t)n && j < (size_t)n) ? J[i * jp + j] : 0.0f;
    const float v1 = (i < (size_t)n && j + 1 < (size_t)n) ? J[i * jp + j + 1] : 0.0f;
    a[k] = (uint8_t)((e2m1_code(v0) & 0xFu) | ((e2m1_code(v1) & 0xFu) << 4));
  }
}

__global__ void prepare_v_fp4_kernel(const float *x, int n, int R, int xp, uint8_t *v, int Kb) {
  const size_t total = (size_t)R * Kb;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / Kb, i = 2 * (k % Kb);
    const uint32_t c0 = i < (size_t)n ? (x[r * xp + i] > 0.0f ? kE2m1Plus : kE2m1Minus) : 0u;
    const uint32_t c1 = i + 1 < (size_t)n ? (x[r * xp + i + 1] > 0.0f ? kE2m1Plus : kE2m1Minus) : 0u;
    v[k] = (uint8_t)(c0 | (c1 << 4));
  }
}

// max |J| over the n x n couplings, as the bits of a non-negative float (NaN ignored)
__global__ void absmax_kernel(const float *J, int n, int jp, unsigned int *out) {
  unsigned int m = 0;
  const size_t total = (size_t)n * n;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const float a = fabsf(J[(k / n) * jp + k % n]);
    const unsigned int u = __float_as_uint(a);
    if (a == a && u > m) m = u;
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
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

bool encode_2d(CUtensorMap *m, void *base, int elem, uint64_t inner, uint64_t outer, uint32_t box_rows,
               bool store_tile = false, uint32_t store_inner = kBM) {
  auto enc = get_encode();
  if (!enc) return false;
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {inner * (uint64_t)elem};
  // loads: one 128-byte swizzled K chunk; stores: the unit's whole 128-spin row, unswizzled
  const cuuint32_t box[2] = {(cuuint32_t)(store_tile ? store_inner : kChunkBytes / elem), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, elem == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                         base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         store_tile ? CU_TENSOR_MAP_SWIZZLE_NONE : CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

// ---------------------------------------------------------------------------------------------

struct TcEngine {
  TcSetup s{};
  int nr = 128, Np = 0, Kp = 0, Rp = 0, n_mtiles = 0, n_rtiles = 0, units = 0;
  uint8_t *a[2] = {nullptr, nullptr};
  uint8_t *v[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  uint32_t *flags = nullptr;
  TcArgs args{};
  const void *kernel[3] = {nullptr, nullptr, nullptr};  // by epilogue mode
  size_t smem = 0;
  int threads = kTcThreads;
  bool pair = false;  // E2M1 kernel in CTA pairs (clusters of two, launched with that attribute)
  float jscale = 1.0f, jinv = 1.0f;  // FP16 hi + lo: the coupling scale (a power of two) and its inverse
  int flag_stride = 1;  // words between consecutive units' step flags
};

namespace {

// Kp: K extent in spins (a multiple of 256 for packed E2M1 operands, of 128 otherwise).
int kp_for(int dt, int n) { return dt == kTcFp4 ? (n + 255) / 256 * 256 : (n + 127) / 128 * 128; }

bool pick(TcEngine *e, int dt, int variant, int nr, int n, bool pair = false) {
  size_t smem = 0;
  for (int m = 0; m < 3; ++m) {
    const void *k = nullptr;
    bool ok;
    if (dt == kTcFp4) ok = tc_kernel_fp4(variant, nr, m, kp_for(dt, n) / 256, &k, &smem, pair);
    else if (dt == kTcFp8) ok = tc_kernel_fp8(variant, nr, m, &k, &smem);
    else if (dt == kTcBf16) ok = tc_kernel_bf16(variant, nr, m, &k, &smem);
    else if (dt == kTcFp16Split) ok = tc_kernel_split16(variant, nr, m, &k, &smem);
    else ok = tc_kernel_split(variant, nr, m, &k, &smem);
    e->kernel[m] = ok ? k : nullptr;
  }
  e->smem = smem;
  return e->kernel[kEmodeStep] != nullptr;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Replica tile (MMA N): the smallest of {32, 64, 128} covering R when R <= 128 (no padded replicas
// to compute), else 128; every unit needs its own SM for the whole solve (cooperative launch), so
// 0 when the units outnumber the SMs.
int choose_nr(int n, int R, int sms) {
  const int mt = (n + kBM - 1) / kBM;
  const int nr = R <= 32 ? 32 : (R <= 64 ? 64 : 128);
  return mt * ((R + nr - 1) / nr) <= sms ? nr : 0;
}

// NMFA: the epilogue (noise draws, tanh) weighs as much as the contraction, so the smallest replica
// tile whose units still fit the SMs (more units, fewer elements per epilogue).
int choose_nr_nmfa(int n, int R, int sms) {
  const int mt = (n + kBM - 1) / kBM;
  for (int nr : {32, 64, 128})
    if (mt * ((R + nr - 1) / nr) <= sms) return nr;
  return 0;
}

}  // namespace

// one counter per unit (per unit and replica half for the E2M1 kernel)
size_t flag_bytes(const TcEngine *e) {
  return ((size_t)e->units * 2 * e->flag_stride * sizeof(uint32_t) + 255) / 256 * 256;
}

namespace {

// Tile geometry of an engine: the setup, the replica tile and the padded extents that follow.
void set_geometry(TcEngine *e, const TcSetup &s, int nr, bool pair = false) {
  e->s = s;
  e->nr = nr;
  e->pair = pair;
  if (s.dtype == kTcFp4) e->threads = kFp4Threads;
  // CTA pairs take spin tiles 2k and 2k + 1: an even number of them
  e->Np = pair ? (s.n + 2 * kBM - 1) / (2 * kBM) * (2 * kBM) : (s.n + kBM - 1) / kBM * kBM;
  e->Kp = kp_for(s.dtype, s.n);
  e->Rp = (s.R + nr - 1) / nr * nr;
  e->n_mtiles = e->Np / kBM;
  e->n_rtiles = e->Rp / nr;
  e->units = e->n_mtiles * e->n_rtiles;
  // the streamed-J kernel polls and publishes faster with each unit's flag on its own 128-byte line
  // (FP8 dSB N=2000 R=1024: 24.7 -> 23.4 ms per solve); the E2M1 kernel is indifferent (its two
  // halves' flags alternate) and keeps them packed. SB_FLAG_STRIDE overrides it (measurements).
  e->flag_stride = s.dtype == kTcFp4 ? 1 : 32;
  if (const char *fs = getenv("SB_FLAG_STRIDE")) {
    const int v = atoi(fs);
    if (v >= 1 && v <= 64) e->flag_stride = v;
  }
}

int elem_bytes(const TcEngine *e) { return (e->s.dtype == kTcFp8 || e->s.dtype == kTcFp4) ? 1 : 2; }
// operand row length in tensor-map elements: bytes of E2M1 pairs, else K elements
uint64_t row_elems(const TcEngine *e) { return e->s.dtype == kTcFp4 ? (uint64_t)e->Kp / 2 : (uint64_t)e->Kp; }
int a_parts(const TcEngine *e) { return tc_split(e->s.dtype) ? 2 : 1; }
int b_parts(const TcEngine *e) { return ((tc_split(e->s.dtype) && e->s.variant == 1) || e->s.variant == 3) ? 2 : 1; }
size_t a_part_bytes(const TcEngine *e) { return (size_t)e->Np * row_elems(e) * elem_bytes(e); }
size_t v_part_bytes(const TcEngine *e) { return (size_t)e->Rp * row_elems(e) * elem_bytes(e); }

// Tensor maps, kernel arguments and the shared-memory attribute of an engine whose operand and
// flag buffers are in place. Returns null, or the name of the call that failed (its CUDA error in
// *ce, cudaSuccess when the call is a tensor-map encoding).
const char *bind(TcEngine *e, cudaError_t *ce) {
  *ce = cudaSuccess;
  const bool fp4 = e->s.dtype == kTcFp4;
  const int elem = elem_bytes(e), nr = e->nr;
  // V boxes: the whole replica tile, or one replica half for the E2M1 kernel (half of that for each
  // CTA of a pair); stores: one replica half of the unit's own spins
  const uint32_t vrows = fp4 ? (uint32_t)(nr >= 64 ? nr / 2 : nr) : (uint32_t)nr;
  const uint32_t vload = e->pair ? vrows / 2 : vrows;
  const uint64_t rowe = row_elems(e);
  TcArgs &g = e->args;
  memset(&g, 0, sizeof(g));
  for (int a = 0; a < a_parts(e); ++a)
    if (!encode_2d(&g.tmA[a], e->a[a], elem, rowe, (uint64_t)e->Np, kBM)) return "cuTensorMapEncodeTiled(J)";
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < b_parts(e); ++pp) {
      if (!encode_2d(&g.tmB[b][pp], e->v[b][pp], elem, rowe, (uint64_t)e->Rp, vload))
        return "cuTensorMapEncodeTiled(V)";
      g.v[b][pp] = e->v[b][pp];
    }
  // the unit's V tile: 128 spins = 128 elements, or 64 bytes of E2M1 pairs
  for (int b = 0; b < 2; ++b)
    if (!encode_2d(&g.tmS[b], e->v[b][0], elem, rowe, (uint64_t)e->Rp, vrows, true, fp4 ? kBM / 2 : kBM))
      return "cuTensorMapEncodeTiled(V store)";
  g.flags = e->flags;
  g.flag_stride = e->flag_stride;
  g.n = e->s.n;
  g.R = e->s.R;
  g.xp = e->s.xp;
  g.Kp = e->Kp;
  g.Rp = e->Rp;
  g.n_mtiles = e->n_mtiles;
  g.n_rtiles = e->n_rtiles;
  g.k_chunks = (int)(rowe * elem / kChunkBytes);
  g.jinv = e->jinv;
  g.xscale = e->s.dtype == kTcFp16Split ? 16384.0f : 1.0f;  // |x| <= 1 -> [-2^14, 2^14]
  g.wait_cycles = ptx::kWaitCycles;
  // split operands: K chunks per accumulation segment (shorter segments take fewer roundings each
  // and cost more hand-offs). BF16 hi + lo: 8 (512 spins); its error is mostly the representation's
  // (16 bits per operand). FP16 hi + lo keeps 22 bits, so the accumulation's rounding is its error
  // and 2 chunks pay (~5 % more time per solve). SB_SPLIT_SEG_CHUNKS overrides both.
  g.seg_chunks = e->s.dtype == kTcFp16Split ? 2 : 8;
  if (const char *sc = getenv("SB_SPLIT_SEG_CHUNKS")) {
    const int v = atoi(sc);
    if (v > 0) g.seg_chunks = v;
  }
  g.skip_unit = -1;
  g.skip_step = -1;
  for (int m = 0; m < 3; ++m)
    if (e->kernel[m] &&
        (*ce = cudaFuncSetAttribute(e->kernel[m], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smem)) !=
            cudaSuccess)
      return "cudaFuncSetAttribute";
  return nullptr;
}

}  // namespace

namespace {
// The CTA-pair E2M1 kernel runs this dSB shape when asked for (SB_TC_PAIR=1): the 128-replica
// tile, its units (spin tiles rounded up to an even count) on distinct SMs, every pair co-resident
// as a cluster of two. It is bit-identical to the single-CTA kernel and measured slower on the
// batched dSB workload, so the single-CTA kernel is the default.
bool pair_fits(const TcSetup &s, int nr, int sms) {
  if (s.dtype != kTcFp4 || s.variant != 2 || nr != 128) return false;
  const char *v = getenv("SB_TC_PAIR");
  if (!v || v[0] != '1') return false;
  const int mt = (s.n + 2 * kBM - 1) / (2 * kBM) * 2;
  const int units = mt * ((s.R + nr - 1) / nr);
  if (units > sms) return false;
  const void *k = nullptr;
  size_t smem = 0;
  if (!tc_kernel_fp4(2, nr, kEmodeStep, kp_for(kTcFp4, s.n) / 256, &k, &smem, true)) return false;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)units);
  cfg.blockDim = dim3((unsigned)kFp4Threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return 2 * clusters >= units;
}
}  // namespace

bool tc_fp4_fits(int n, int R) {
  const int nr = choose_nr(n, R, sm_count());
  const void *k = nullptr;
  size_t smem = 0;
  return nr > 0 && tc_kernel_fp4(2, nr, kEmodeStep, kp_for(kTcFp4, n) / 256, &k, &smem);
}

int64_t tc_footprint(const TcSetup &s) {
  if (s.dtype == kTcFp4) {
    const int64_t Np = (s.n + 2 * kBM - 1) / (2 * kBM) * (2 * kBM), Kb = kp_for(kTcFp4, s.n) / 2;
    const int64_t Rp = (s.R + 127) / 128 * 128;
    return Np * Kb + 2 * Rp * Kb + 4096;
  }
  const int elem = s.dtype == kTcFp8 ? 1 : 2;
  const int64_t Np = (s.n + kBM - 1) / kBM * kBM, Kp = (s.n + 127) / 128 * 128;
  const int64_t Rp = (s.R + 127) / 128 * 128;
  const int ap = tc_split(s.dtype) ? 2 : 1;
  const int bp = ((tc_split(s.dtype) && s.variant == 1) || s.variant == 3) ? 2 : 1;
  return Np * Kp * elem * ap + 2 * Rp * Kp * elem * bp + 4096;
}

sb_status tc_create(TcEngine **out, const TcSetup &s, const float *dJ, int jp, std::string &err,
                    cudaStream_t st) {
  *out = nullptr;
  if (s.variant != 1 && s.variant != 2 && s.variant != 3) {
    err = "tensor-core path runs bSB, dSB and NMFA";
    return SB_ERR_UNSUPPORTED;
  }
  if (s.variant == 3 && s.dtype != kTcBf16) {
    err = "NMFA on tensor cores needs BF16 operands (integer couplings)";
    return SB_ERR_UNSUPPORTED;
  }
  if (s.variant == 1 && !tc_split(s.dtype)) {
    err = "bSB on tensor cores needs split (hi + lo) operands";
    return SB_ERR_UNSUPPORTED;
  }
  const int sms = sm_count();
  const int nr = s.variant == 3 ? choose_nr_nmfa(s.n, s.R, sms) : choose_nr(s.n, s.R, sms);
  if (nr == 0) {
    err = "problem too large for the single-pass tensor-core kernel (units > SMs)";
    return SB_ERR_UNSUPPORTED;
  }
  TcEngine *e = new TcEngine();
  const bool pair = pair_fits(s, nr, sms);
  if (!pick(e, s.dtype, s.variant, nr, s.n, pair)) {
    delete e;
    err = "no kernel for this dtype / variant / size";
    return SB_ERR_UNSUPPORTED;
  }
  set_geometry(e, s, nr, pair);
  auto fail = [&](const char *what, cudaError_t ce) {
    err = std::string(what) + (ce != cudaSuccess ? std::string(": ") + cudaGetErrorString(ce) : "");
    tc_destroy(e);
    return ce == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  };
  cudaError_t ce;
  const size_t abytes = a_part_bytes(e), vbytes = v_part_bytes(e);
  for (int a = 0; a < a_parts(e); ++a)
    if ((ce = cudaMalloc(&e->a[a], abytes)) != cudaSuccess) return fail("cudaMalloc(J operand)", ce);
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < b_parts(e); ++pp) {
      if ((ce = cudaMalloc(&e->v[b][pp], vbytes)) != cudaSuccess) return fail("cudaMalloc(V operand)", ce);
      if ((ce = cudaMemsetAsync(e->v[b][pp], 0, vbytes, st)) != cudaSuccess) return fail("memset", ce);
    }
  if ((ce = cudaMalloc(&e->flags, flag_bytes(e))) != cudaSuccess) return fail("cudaMalloc(flags)", ce);
  if ((ce = tc_reload(e, dJ, jp, st)) != cudaSuccess) return fail("convert_j_kernel", ce);
  const char *what = bind(e, &ce);
  if (what) return fail(what, ce);
  *out = e;
  return SB_OK;
}

void tc_destroy(TcEngine *e) {
  if (!e) return;
  cudaFree(e->a[0]);
  cudaFree(e->a[1]);
  for (int b = 0; b < 2; ++b)
    for (int pp = 0; pp < 2; ++pp) cudaFree(e->v[b][pp]);
  cudaFree(e->flags);
  delete e;
}

cudaError_t tc_reload(TcEngine *e, const float *dJ, int jp, cudaStream_t st) {
  if (e->s.dtype == kTcFp16Split) {
    // the scale that brings max |J| into [2^12, 2^13): the flag words serve as the reduction's cell
    cudaError_t ce = cudaMemsetAsync(e->flags, 0, sizeof(unsigned int), st);
    if (ce != cudaSuccess) return ce;
    absmax_kernel<<<grid_1d((size_t)e->s.n * e->s.n), 256, 0, st>>>(dJ, e->s.n, jp, e->flags);
    if ((ce = cudaGetLastError()) != cudaSuccess) return ce;
    unsigned int bits = 0;
    if ((ce = cudaMemcpyAsync(&bits, e->flags, sizeof(bits), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return ce;
    if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return ce;
    float m;
    memcpy(&m, &bits, sizeof(m));
    int ex = 0;
    if (m > 0.0f && m < 3.0e38f) frexpf(m, &ex);  // m = f 2^ex, f in [0.5, 1)
    const int sj = m > 0.0f ? std::max(-100, std::min(100, 13 - ex)) : 0;
    e->jscale = ldexpf(1.0f, sj);
    e->jinv = ldexpf(1.0f, -sj);
    e->args.jinv = e->jinv;
  }
  if (e->s.dtype == kTcFp4) {
    const int Kb = e->Kp / 2;
    convert_j_fp4_kernel<<<grid_1d((size_t)e->Np * Kb), 256, 0, st>>>(dJ, e->s.n, jp, e->a[0], e->Np, Kb);
    return cudaGetLastError();
  }
  convert_j_kernel<<<grid_1d((size_t)e->Np * e->Kp), 256, 0, st>>>(dJ, e->s.n, jp, e->a[0], e->a[1], e->Np, e->Kp,
                                                                   e->s.dtype, e->jscale);
  return cudaGetLastError();
}

int tc_dtype(const TcEngine *e) { return e ? e->s.dtype : 0; }

void tc_set_waits(TcEngine *e, long long wait_cycles, int skip_step) {
  e->args.wait_cycles = wait_cycles > 0 ? wait_cycles : ptx::kWaitCycles;
  e->args.skip_unit = skip_step >= 0 ? 0 : -1;
  e->args.skip_step = skip_step;
}
int tc_units(const TcEngine *e) { return e ? e->units : 0; }
int tc_replica_tile(const TcEngine *e) { return e ? e->nr : 0; }

cudaError_t tc_prepare(TcEngine *e, const float *x, cudaStream_t st) {
  if (e->s.dtype == kTcFp4) {
    const int Kb = e->Kp / 2;
    prepare_v_fp4_kernel<<<grid_1d((size_t)e->s.R * Kb), 256, 0, st>>>(x, e->s.n, e->s.R, e->s.xp, e->v[0][0], Kb);
    return cudaGetLastError();
  }
  prepare_v_kernel<<<grid_1d((size_t)e->s.n * e->s.R), 256, 0, st>>>(x, e->s.n, e->s.R, e->s.xp, e->v[0][0], e->v[0][1], e->Kp,
                                                                      e->s.dtype, e->s.variant, e->args.xscale);
  return cudaGetLastError();
}

static cudaError_t launch(TcEngine *e, int emode, const TcArgs &a, cudaStream_t st) {
  if (!e->kernel[emode]) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)e->units);
  cfg.blockDim = dim3((unsigned)e->threads);
  cfg.dynamicSmemBytes = e->smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = 2;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = e->pair ? 2 : 1;
  void *params[1] = {const_cast<TcArgs *>(&a)};
  return cudaLaunchKernelExC(&cfg, e->kernel[emode], params);
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
  a.buf0 = 0;
  a.pumps = pumps;
  a.c0 = c0;
  a.dt = dt;
  a.dta0 = dta0;
  cudaError_t ce = cudaMemsetAsync(e->flags, 0, flag_bytes(e), st);
  if (ce != cudaSuccess) return ce;
  return launch(e, energy_trace ? kEmodeStepTrace : kEmodeStep, a, st);
}

cudaError_t tc_run_nmfa(TcEngine *e, int sweeps, const float *betas, float *s, float *z1, const float *norm,
                        uint32_t *rng, float noise, float keep, float mix, uint32_t *status, cudaStream_t st) {
  if (sweeps <= 0) return cudaSuccess;
  if (e->s.variant != 3) return cudaErrorInvalidValue;
  TcArgs a = e->args;
  a.x = s;
  a.y = z1;
  a.h = norm;
  a.energy = nullptr;
  a.status = status;
  a.steps = sweeps;
  a.t0 = 0;
  a.buf0 = 0;
  a.pumps = betas;
  a.rng = rng;
  a.noise = noise;
  a.keep = keep;
  a.mix = mix;
  cudaError_t ce = cudaMemsetAsync(e->flags, 0, flag_bytes(e), st);
  if (ce != cudaSuccess) return ce;
  return launch(e, kEmodeStep, a, st);
}

cudaError_t tc_energy_signs(TcEngine *e, const float *x, const float *h, double *energy, uint32_t *status,
                            cudaStream_t st) {
  // the dSB energy contraction on the engine's couplings (BF16 or BF16 hi + lo): operand buffer 0
  // part 0 takes sign(x) (its padding is still zero) and the kernel adds -1/2 s_i (J s)_i - h_i s_i
  // per replica into energy
  const void *k = nullptr;
  size_t smem = 0;
  const bool have = e->s.dtype == kTcBf16        ? tc_kernel_bf16(2, e->nr, kEmodeEnergy, &k, &smem)
                    : e->s.dtype == kTcBf16Split ? tc_kernel_split(2, e->nr, kEmodeEnergy, &k, &smem)
                    : e->s.dtype == kTcFp16Split ? tc_kernel_split16(2, e->nr, kEmodeEnergy, &k, &smem)
                                                 : false;
  if (!have) return cudaErrorInvalidValue;
  cudaError_t ce = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (ce != cudaSuccess) return ce;
  prepare_v_kernel<<<grid_1d((size_t)e->s.n * e->s.R), 256, 0, st>>>(x, e->s.n, e->s.R, e->s.xp, e->v[0][0], nullptr,
                                                                      e->Kp, e->s.dtype, 2, 1.0f);
  if ((ce = cudaGetLastError()) != cudaSuccess) return ce;
  TcArgs a = e->args;
  a.x = const_cast<float *>(x);
  a.y = nullptr;
  a.h = h;
  a.energy = energy;
  a.status = status;
  a.steps = 1;
  a.t0 = 0;
  a.buf0 = 0;
  a.pumps = nullptr;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)e->units);
  cfg.blockDim = dim3((unsigned)e->threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void *params[1] = {&a};
  return cudaLaunchKernelExC(&cfg, k, params);
}

bool tc_external_sizes(int n, int R, bool fp4, size_t *a_bytes, size_t *v_bytes, size_t *flags_bytes) {
  const int nr = choose_nr(n, R, sm_count());
  *a_bytes = *v_bytes = *flags_bytes = 0;
  if (nr == 0 || (fp4 && !tc_fp4_fits(n, R))) return false;
  TcEngine e;
  set_geometry(&e, TcSetup{2, fp4 ? kTcFp4 : kTcFp8, n, R, n}, nr);
  e.flag_stride = 1;  // packed flags: the allocation-free caller's fixed control area
  *a_bytes = a_part_bytes(&e);
  *v_bytes = v_part_bytes(&e);
  *flags_bytes = flag_bytes(&e);
  return true;
}

cudaError_t tc_dsb_external(const TcExternal &ext, cudaStream_t st) {
  TcEngine e;  // on the stack: every buffer below belongs to the caller
  const int dt = ext.fp4 ? kTcFp4 : kTcFp8;
  const int nr = choose_nr(ext.n, ext.R, sm_count());
  if (nr == 0 || (ext.fp4 && !tc_fp4_fits(ext.n, ext.R)) || !pick(&e, dt, 2, nr, ext.n)) return cudaErrorInvalidValue;
  set_geometry(&e, TcSetup{2, dt, ext.n, ext.R, ext.xp}, nr);
  e.flag_stride = 1;  // packed flags (tc_external_sizes)
  e.a[0] = ext.a;
  e.v[0][0] = ext.v0;
  e.v[1][0] = ext.v1;
  e.flags = ext.flags;
  cudaError_t ce = cudaSuccess;
  if (bind(&e, &ce)) return ce != cudaSuccess ? ce : cudaErrorInvalidValue;
  if ((ce = tc_reload(&e, ext.J, ext.jp, st)) != cudaSuccess) return ce;
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
  a.buf0 = t & 1;
  return launch(e, kEmodeEnergy, a, st);
}

}  // namespace sbk
