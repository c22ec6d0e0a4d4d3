// Host side of the grouped tensor-core path: many dSB instances of uneven size advanced together.
// Used by sb_batch_* (a fixed batch, all instances run the same number of steps) and by the
// serving loop (instances admitted and retired while others run).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sb_grouped.cuh"
#include "sb_grouped.h"
#include "sb_host.h"

namespace sbk {
namespace {
using namespace tck;

__global__ void g_convert_kernel(const float *J, int n, uint8_t *a, int Np, int Kp) {
  const size_t total = (size_t)Np * Kp;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = k / Kp, j = k % Kp;
    const float v = (i < (size_t)n && j < (size_t)n) ? J[i * n + j] : 0.0f;
    a[k] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
  }
}

__global__ void g_signs_kernel(const float *x, int n, int R, int xp, uint8_t *v, int Kp) {
  const size_t total = (size_t)n * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / n, i = k % n;
    v[r * Kp + i] = x[r * xp + i] > 0.0f ? (uint8_t)0x38 : (uint8_t)0xB8;
  }
}

// packed E2M1 signs: byte b of replica r holds spins 2b (low nibble) and 2b + 1 (high nibble)
__global__ void g_signs_fp4_kernel(const float *x, int n, int R, int xp, uint8_t *v, int kb) {
  const int nb = (n + 1) / 2;
  const size_t total = (size_t)nb * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / nb, b = k % nb, i = 2 * b;
    const uint32_t c0 = x[r * xp + i] > 0.0f ? kE2m1Plus : kE2m1Minus;
    const uint32_t c1 = i + 1 < (size_t)n ? (x[r * xp + i + 1] > 0.0f ? kE2m1Plus : kE2m1Minus) : 0u;
    v[r * kb + b] = (uint8_t)(c0 | (c1 << 4));
  }
}

// packed E2M3 signs (+4: 0x18, -4: 0x38, padding 0): one thread per 16 spins of a replica, 12 bytes
// (value i of the group at bits 6 i .. 6 i + 5, little-endian)
__global__ void g_signs_fp6_kernel(const float *x, int n, int R, int xp, uint8_t *v, int kb) {
  const int ng = (n + 15) / 16;
  const size_t total = (size_t)ng * R;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t r = k / ng, g = k % ng;
    uint32_t w[3] = {0u, 0u, 0u};
    for (int i = 0; i < 16; ++i) {
      const size_t sp = 16 * g + i;
      if (sp >= (size_t)n) break;
      const uint32_t code = x[r * xp + sp] > 0.0f ? 0x18u : 0x38u;
      const int bit = 6 * i;
      w[bit >> 5] |= code << (bit & 31);
      if ((bit & 31) > 26) w[(bit >> 5) + 1] |= code >> (32 - (bit & 31));
    }
    uint32_t *dst = reinterpret_cast<uint32_t *>(v + r * kb + 12 * g);
    dst[0] = w[0];
    dst[1] = w[1];
    dst[2] = w[2];
  }
}

int grid1(size_t total) {
  size_t g = (total + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool encode_fp8(CUtensorMap *m, void *base, uint64_t inner, uint64_t outer, uint32_t rows) {
  auto enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {inner};
  const cuuint32_t box[2] = {(cuuint32_t)kChunkBytes, rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Packed E2M3 operand [rows][kelems] (six bits per value, rows of 3 kelems / 4 bytes): the tensor
// map spreads each 12 bytes (sixteen values) into a 16-byte shared-memory slot, 128 values per box
// row (kelems a multiple of 128, rows of a multiple of 32 bytes, base 32-byte aligned).
bool encode_fp6(CUtensorMap *m, void *base, uint64_t kelems, uint64_t rows, uint32_t box_rows) {
  auto enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {kelems, rows};
  const cuuint64_t strides[1] = {kelems * 3 / 4};
  const cuuint32_t box[2] = {128u, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_16U6_ALIGN16B, 2, base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the operand maps of an instance: J (box of 128 rows) or V (box of nr rows)
bool encode_operand(int op, CUtensorMap *m, void *base, int Kp, int kbytes, uint64_t rows, uint32_t box_rows) {
  return op == kGopE2m3 ? encode_fp6(m, base, (uint64_t)Kp, rows, box_rows)
                        : encode_fp8(m, base, (uint64_t)kbytes, rows, box_rows);
}

template <int NR, int OP>
const void *gk(int emode) {
  return emode == kEmodeEnergy ? reinterpret_cast<const void *>(&grouped_kernel<NR, grouped_stages<NR>(), kEmodeEnergy, OP>)
                               : reinterpret_cast<const void *>(&grouped_kernel<NR, grouped_stages<NR>(), kEmodeStep, OP>);
}

template <int NR>
const void *gk_op(int op, int emode) {
  return op == kGopE2m1 ? gk<NR, kGopE2m1>(emode) : (op == kGopE2m3 ? gk<NR, kGopE2m3>(emode) : gk<NR, kGopFp8>(emode));
}

bool grouped_kernel_for(int nr, int emode, int op, const void **k, size_t *smem) {
  switch (nr) {
    case 32: *k = gk_op<32>(op, emode); *smem = grouped_smem<32>(); return true;
    case 64: *k = gk_op<64>(op, emode); *smem = grouped_smem<64>(); return true;
    case 128: *k = gk_op<128>(op, emode); *smem = grouped_smem<128>(); return true;
  }
  return false;
}

// E4M3 code of the integer v, |v| <= 16: 1.m x 2^(e - 7) with a 3-bit mantissa (every integer up
// to 16 has at most 4 significant bits).
uint8_t fp8_code(int v) {
  if (v == 0) return 0;
  const uint8_t sign = v < 0 ? 0x80 : 0;
  int a = v < 0 ? -v : v;
  int e = 0;
  while ((2 << e) <= a) ++e;                // a in [2^e, 2^(e+1))
  const int m = ((a << 3) >> e) - 8;        // (a / 2^e - 1) * 8, exact for these integers
  return (uint8_t)(sign | ((e + 7) << 3) | m);
}

// Off-diagonal sums of J and J^2 over integer couplings, gathered while packing: the coupling
// statistics behind the default c0 (sbh::c0_from_sums gives the value sb_default_c0 computes).
struct CouplingSums {
  int64_t s = 0, s2 = 0;
};

// Rows [0, Np) of J packed by `nt` threads, `row(i, d, sum, sum2)` writing row i < n into d.
template <typename RowFn>
CouplingSums pack_rows(int n, uint8_t *dst, int Np, int row_bytes, int64_t elems_per_thread, RowFn row) {
  const unsigned want = (unsigned)std::max<int64_t>(1, (int64_t)Np * row_bytes / elems_per_thread);
  const unsigned nt = std::max(1u, std::min({std::thread::hardware_concurrency() / 2, want, 16u}));
  const int rows_per = (Np + (int)nt - 1) / (int)nt;
  std::vector<CouplingSums> part(nt);
  auto work = [&, rows_per](unsigned w) {
    const int r0 = (int)w * rows_per, r1 = std::min(Np, r0 + rows_per);
    int64_t a = 0, a2 = 0;
    for (int i = r0; i < r1; ++i) {
      uint8_t *d = dst + (size_t)i * row_bytes;
      if (i >= n) {
        memset(d, 0, row_bytes);
        continue;
      }
      int32_t rs = 0, rs2 = 0;  // |J| <= 16: at most 256 n per row
      row(i, d, rs, rs2);
      a += rs;
      a2 += rs2;
    }
    part[w].s = a;
    part[w].s2 = a2;
  };
  sbh::parallel_run((int)nt, [&](int w) { work((unsigned)w); });
  CouplingSums out;
  for (const auto &c : part) {
    out.s += c.s;
    out.s2 += c.s2;
  }
  return out;
}

// Couplings as FP8 E4M3 (integers |J| <= 16; fp8_code), rows of Kp bytes, zero padded.
CouplingSums pack_fp8(const float *J, int n, uint8_t *dst, int Np, int Kp) {
  uint8_t lut[33];
  for (int v = -16; v <= 16; ++v) lut[v + 16] = fp8_code(v);
  // about 2 M elements per thread; several admissions pack at once
  return pack_rows(n, dst, Np, Kp, 2 << 20, [&](int i, uint8_t *d, int32_t &rs, int32_t &rs2) {
    const float *Ji = J + (size_t)i * n;
    for (int j = 0; j < n; ++j) {
      const int v = (int)Ji[j];
      d[j] = lut[v + 16];
      rs += v;
      rs2 += v * v;
    }
    const int dg = (int)Ji[i];  // the diagonal does not count
    rs -= dg;
    rs2 -= dg * dg;
    memset(d + n, 0, Kp - n);
  });
}

// Couplings as packed E2M1 (integers |J| <= 4), rows of kb bytes, zero padded. The code of v is
// |v| + min(|v|, 2) with the sign in bit 3 (0, 1, 2, 3, 4 -> 0x0, 0x2, 0x4, 0x5, 0x6: e2m1_code),
// computed rather than looked up so that the loop vectorises.
CouplingSums pack_fp4(const float *J, int n, uint8_t *dst, int Np, int kb) {
  return pack_rows(n, dst, Np, kb, 1 << 20, [&](int i, uint8_t *d, int32_t &rs, int32_t &rs2) {
    const float *Ji = J + (size_t)i * n;
    auto code = [](int v) {
      const int a = v < 0 ? -v : v;
      return (a + (a < 2 ? a : 2)) | (v < 0 ? 8 : 0);
    };
    const int pairs = n >> 1;
    int32_t s1 = 0, s2 = 0;
    for (int b = 0; b < pairs; ++b) {
      const int v0 = (int)Ji[2 * b], v1 = (int)Ji[2 * b + 1];
      d[b] = (uint8_t)(code(v0) | (code(v1) << 4));
      s1 += v0 + v1;
      s2 += v0 * v0 + v1 * v1;
    }
    int used = pairs;
    if (n & 1) {
      const int v = (int)Ji[n - 1];
      d[pairs] = (uint8_t)code(v);
      s1 += v;
      s2 += v * v;
      used = pairs + 1;
    }
    memset(d + used, 0, kb - used);
    const int dg = (int)Ji[i];  // the diagonal does not count
    rs = s1 - dg;
    rs2 = s2 - dg * dg;
  });
}

// Couplings as packed E2M3 (integers |J| <= 16 held as J / 4), rows of 3 Kp / 4 bytes, sixteen
// values per 12 bytes (value i at bits 6 i .. 6 i + 5, little-endian), zero padded. E2M3 is
// (-1)^s 2^(e-1) (1 + m / 8) for e >= 1 and m / 8 for e = 0, so every quarter-integer up to 4 is exact:
// |J| < 4: e 0, m 2|J|; 4 <= |J| < 8: e 1, m 2|J| - 8; 8 <= |J| < 16: e 2, m |J| - 8; 16: e 3, m 0.
uint8_t fp6_code(int v) {
  const int a = v < 0 ? -v : v;
  int e, m;
  if (a < 4) e = 0, m = 2 * a;
  else if (a < 8) e = 1, m = 2 * a - 8;
  else if (a < 16) e = 2, m = a - 8;
  else e = 3, m = 0;
  return (uint8_t)((a == 0 ? 0 : (v < 0 ? 0x20 : 0)) | (e << 3) | m);
}

CouplingSums pack_fp6(const float *J, int n, uint8_t *dst, int Np, int Kp) {
  uint8_t lut[33];
  for (int v = -16; v <= 16; ++v) lut[v + 16] = fp6_code(v);
  const int kb = Kp / 4 * 3;
  return pack_rows(n, dst, Np, kb, 2 << 20, [&](int i, uint8_t *d, int32_t &rs, int32_t &rs2) {
    const float *Ji = J + (size_t)i * n;
    int32_t s1 = 0, s2 = 0;
    for (int g = 0; g < Kp / 16; ++g) {
      uint64_t lo = 0;  // bits 0..63 of the group
      uint32_t hi = 0;  // bits 64..95
      for (int t = 0; t < 16; ++t) {
        const int j = 16 * g + t;
        const int v = j < n ? (int)Ji[j] : 0;
        s1 += v;
        s2 += v * v;
        const uint64_t c = lut[v + 16];
        const int bit = 6 * t;
        if (bit < 64) {
          lo |= c << bit;
          if (bit > 58) hi |= (uint32_t)(c >> (64 - bit));
        } else {
          hi |= (uint32_t)(c << (bit - 64));
        }
      }
      uint8_t *q = d + 12 * g;
      for (int b = 0; b < 8; ++b) q[b] = (uint8_t)(lo >> (8 * b));
      for (int b = 0; b < 4; ++b) q[8 + b] = (uint8_t)(hi >> (8 * b));
    }
    const int dg = (int)Ji[i];  // the diagonal does not count
    rs = s1 - dg;
    rs2 = s2 - dg * dg;
  });
}

int device_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

// ---------------------------------------------------------------------------------------------

bool grouped_supports(const sb_problem *p, const sb_params *prm) {
  return prm->variant == SB_DSB && p->integer_valued && p->max_abs_j <= 16 && p->n <= 65536 &&
         prm->replicas <= 4096 && (int64_t)p->n * 16 < (1 << 24);
}

bool grouped_fp4_exact(const sb_problem *p) { return p->integer_valued && p->max_abs_j <= 4; }

int64_t grouped_instance_bytes(int n, int R, int steps, int nr, int op) {
  const int64_t Np = (n + 127) / 128 * 128, Rp = (R + nr - 1) / nr * nr, xp = (n + 3) / 4 * 4;
  const int64_t kb = op == kGopE2m1 ? (n + 255) / 256 * 128 : (op == kGopE2m3 ? Np / 4 * 3 : Np);
  return Np * kb + 2 * Rp * kb + 2 * (int64_t)R * xp * 4 + (int64_t)n * 4 + (int64_t)R * 8 + (int64_t)steps * 4 + 4096;
}

Grouped::~Grouped() { clear(); }

void Grouped::clear() {
  for (auto &g : insts) free_instance(g);
  insts.clear();
  cudaFree(d_insts);
  cudaFree(d_items);
  cudaFree(d_status);
  cudaFree(d_stage);
  cudaStreamSynchronize(st);
  cudaFreeHost(stg_.pin);
  stg_.pin = nullptr;
  stg_.bytes = 0;
  cudaFree(d_sub_items);
  d_sub_items = nullptr;
  cap_sub = 0;
  if (graph) cudaGraphExecDestroy(graph);
  d_insts = nullptr;
  d_items = nullptr;
  d_status = nullptr;
  d_stage = nullptr;
  graph = nullptr;
  stage_bytes = 0;
  cap_insts = cap_items = 0;
}

void Grouped::free_instance(GHost &g) { release(g, st); }

// Stream-ordered frees: the memory returns to the device pool once `s` passes this point, with no
// device-wide synchronisation (plain cudaFree would stall every stream).
void Grouped::release(GHost &g, cudaStream_t s) {
  for (void *ptr : {(void *)g.a, (void *)g.v[0], (void *)g.v[1], (void *)g.x, (void *)g.y, (void *)g.h,
                    (void *)g.energy, (void *)g.pumps})
    if (ptr) cudaFreeAsync(ptr, s);
  g.a = g.v[0] = g.v[1] = nullptr;
  g.x = g.y = g.h = g.pumps = nullptr;
  g.energy = nullptr;
}

sb_status Grouped::prepare(GHost &g, const sb_problem *p, const sb_params *prm, uint64_t seed, int tag, int nr,
                           cudaStream_t st, Staging &stg, std::string &err, int op) {
  g.tag = tag;
  g.prob = p;
  g.n = p->n;
  g.R = prm->replicas;
  g.steps = prm->steps;
  g.t0 = 0;
  g.Np = (g.n + 127) / 128 * 128;
  g.op = op;
  const bool fp4 = op == kGopE2m1;
  g.Kp = fp4 ? (g.n + 255) / 256 * 256 : g.Np;  // K extent in spins: whole 128-byte shared-memory chunks
  g.kbytes = fp4 ? g.Kp / 2 : (op == kGopE2m3 ? g.Kp / 4 * 3 : g.Kp);
  g.Rp = (g.R + nr - 1) / nr * nr;
  g.xp = (g.n + 3) / 4 * 4;
  g.c0 = prm->c0;  // or, when unset, the default from the coupling sums the packing gathers
  g.dt = prm->dt;
  g.dta0 = prm->dt * prm->a0;
  cudaError_t e;
  auto fail = [&](const char *what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    release(g, st);
    return e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA;
  };
  const size_t xs = (size_t)g.R * g.xp * sizeof(float), vb = (size_t)g.Rp * g.kbytes;
  if ((e = cudaMallocAsync(&g.a, (size_t)g.Np * g.kbytes, st)) != cudaSuccess) return fail("cudaMalloc(J operand)");
  if ((e = cudaMallocAsync(&g.v[0], vb, st)) != cudaSuccess) return fail("cudaMalloc(V)");
  if ((e = cudaMallocAsync(&g.v[1], vb, st)) != cudaSuccess) return fail("cudaMalloc(V)");
  if ((e = cudaMallocAsync(&g.x, xs, st)) != cudaSuccess) return fail("cudaMalloc(x)");
  if ((e = cudaMallocAsync(&g.y, xs, st)) != cudaSuccess) return fail("cudaMalloc(y)");
  if ((e = cudaMallocAsync(&g.energy, (size_t)g.R * sizeof(double), st)) != cudaSuccess) return fail("cudaMalloc(energy)");
  if ((e = cudaMallocAsync(&g.pumps, (size_t)(g.steps > 0 ? g.steps : 1) * sizeof(float), st)) != cudaSuccess)
    return fail("cudaMalloc(pumps)");
  if (p->h) {
    if ((e = cudaMallocAsync(&g.h, (size_t)g.n * sizeof(float), st)) != cudaSuccess) return fail("cudaMalloc(h)");
    if ((e = cudaMemcpyAsync(g.h, p->h, (size_t)g.n * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return fail("upload h");
  }
  // couplings: packed to FP8 E4M3 (integers |J| <= 16 are exact, see fp8_code), to E2M3 (J / 4,
  // six bits; fp6_code) or to E2M1 pairs (|J| <= 4) on the host threads into a pinned staging
  // buffer, then one copy into the padded operand layout.
  const size_t ab = (size_t)g.Np * g.kbytes;
  if (ab > stg.bytes) {
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("synchronize");
    cudaFreeHost(stg.pin);
    stg.pin = nullptr;
    stg.bytes = 0;
    if ((e = cudaMallocHost(&stg.pin, ab)) != cudaSuccess) return fail("cudaMallocHost(staging)");
    stg.bytes = ab;
  }
  const CouplingSums sums = fp4 ? pack_fp4(p->J, g.n, stg.pin, g.Np, g.kbytes)
                                : (op == kGopE2m3 ? pack_fp6(p->J, g.n, stg.pin, g.Np, g.Kp)
                                                  : pack_fp8(p->J, g.n, stg.pin, g.Np, g.Kp));
  if (!(g.c0 > 0.0f)) g.c0 = sbh::c0_from_sums(g.n, sums.s, sums.s2);
  if ((e = cudaMemcpyAsync(g.a, stg.pin, ab, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail("upload J");
  std::vector<float> pumps((size_t)(g.steps > 0 ? g.steps : 1), 0.0f);
  for (int t = 0; t < g.steps; ++t) pumps[t] = sb_pump(prm->a0, t, g.steps);
  if ((e = cudaMemcpyAsync(g.pumps, pumps.data(), pumps.size() * sizeof(float), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return fail("upload pumps");
  // the staging buffer and the pump vector are reused / freed: finish the copies now
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("synchronize");
  if ((e = cudaMemsetAsync(g.v[0], 0, vb, st)) != cudaSuccess) return fail("memset");
  if ((e = cudaMemsetAsync(g.v[1], 0, vb, st)) != cudaSuccess) return fail("memset");
  if ((e = cudaMemsetAsync(g.x, 0, xs, st)) != cudaSuccess) return fail("memset");
  if ((e = cudaMemsetAsync(g.y, 0, xs, st)) != cudaSuccess) return fail("memset");
  if (!encode_operand(op, &g.desc.tmA, g.a, g.Kp, g.kbytes, (uint64_t)g.Np, kBM) ||
      !encode_operand(op, &g.desc.tmB[0], g.v[0], g.Kp, g.kbytes, (uint64_t)g.Rp, (uint32_t)nr) ||
      !encode_operand(op, &g.desc.tmB[1], g.v[1], g.Kp, g.kbytes, (uint64_t)g.Rp, (uint32_t)nr)) {
    e = cudaErrorInvalidValue;
    return fail("cuTensorMapEncodeTiled");
  }
  g.desc.v[0] = g.v[0];
  g.desc.v[1] = g.v[1];
  g.desc.x = g.x;
  g.desc.y = g.y;
  g.desc.h = g.h;
  g.desc.energy = g.energy;
  g.desc.pumps = g.pumps;
  g.desc.n = g.n;
  g.desc.Kp = g.Kp;
  g.desc.kbytes = g.kbytes;
  g.desc.R = g.R;
  g.desc.Rp = g.Rp;
  g.desc.xp = g.xp;
  g.desc.t0 = 0;
  g.desc.c0 = g.c0;
  g.desc.dt = g.dt;
  g.desc.dta0 = g.dta0;
  g.seed = seed;
  sb_status s = init_state_on(g, seed, st, err);
  if (s != SB_OK) {
    release(g, st);
    return s;
  }
  // the instance is complete before another stream uses it
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("synchronize");
  return SB_OK;
}

void Grouped::attach(GHost &g, int t0) {
  g.t0 = t0;
  g.desc.t0 = t0;
  insts.push_back(g);
  dirty = true;
}

sb_status Grouped::add(const sb_problem *p, const sb_params *prm, uint64_t seed, int t0, int tag, std::string &err) {
  GHost g;
  sb_status s = prepare(g, p, prm, seed, tag, nr, st, stg_, err, op);
  if (s != SB_OK) return s;
  attach(g, t0);
  return SB_OK;
}


sb_status Grouped::init_state(GHost &g, uint64_t seed, std::string &err) { return init_state_on(g, seed, st, err); }

sb_status Grouped::init_state_on(GHost &g, uint64_t seed, cudaStream_t st, std::string &err) {
  cudaError_t e = launch_init_uniform(g.x, g.y, g.n, g.R, g.xp, seed, st);
  if (e == cudaSuccess) {
    if (g.op == kGopE2m1)
      g_signs_fp4_kernel<<<grid1((size_t)g.n * g.R), 256, 0, st>>>(g.x, g.n, g.R, g.xp, g.v[0], g.kbytes);
    else if (g.op == kGopE2m3)
      g_signs_fp6_kernel<<<grid1((size_t)(g.n + 15) / 16 * g.R), 256, 0, st>>>(g.x, g.n, g.R, g.xp, g.v[0], g.kbytes);
    else
      g_signs_kernel<<<grid1((size_t)g.n * g.R), 256, 0, st>>>(g.x, g.n, g.R, g.xp, g.v[0], g.Kp);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    err = std::string("initial state: ") + cudaGetErrorString(e);
    return SB_ERR_CUDA;
  }
  // step t of the instance reads buffer t & 1 (t = tick - t0), so V(0) goes to buffer 0
  return SB_OK;
}

sb_status Grouped::retile(int new_nr, std::string &err) {
  if (new_nr == nr) return SB_OK;
  nr = new_nr;
  for (auto &g : insts) {
    cudaFreeAsync(g.v[0], st);
    cudaFreeAsync(g.v[1], st);
    g.v[0] = g.v[1] = nullptr;
    g.Rp = (g.R + nr - 1) / nr * nr;
    const size_t vb = (size_t)g.Rp * g.kbytes;
    cudaError_t e;
    if ((e = cudaMallocAsync(&g.v[0], vb, st)) != cudaSuccess || (e = cudaMallocAsync(&g.v[1], vb, st)) != cudaSuccess) {
      err = "cudaMalloc(V)";
      return SB_ERR_OOM;
    }
    cudaMemsetAsync(g.v[0], 0, vb, st);
    cudaMemsetAsync(g.v[1], 0, vb, st);
    if (!encode_operand(g.op, &g.desc.tmB[0], g.v[0], g.Kp, g.kbytes, (uint64_t)g.Rp, (uint32_t)nr) ||
        !encode_operand(g.op, &g.desc.tmB[1], g.v[1], g.Kp, g.kbytes, (uint64_t)g.Rp, (uint32_t)nr)) {
      err = "cuTensorMapEncodeTiled";
      return SB_ERR_CUDA;
    }
    g.desc.v[0] = g.v[0];
    g.desc.v[1] = g.v[1];
    g.desc.Rp = g.Rp;
  }
  dirty = true;
  return SB_OK;
}

void Grouped::remove(int idx) {
  free_instance(insts[idx]);
  insts.erase(insts.begin() + idx);
  dirty = true;
}

sb_status Grouped::sync_tables(std::string &err) {
  if (!dirty) return SB_OK;
  cudaError_t e;
  if ((int)insts.size() > cap_insts) {
    cudaFree(d_insts);
    cap_insts = std::max<int>((int)insts.size(), 2 * cap_insts);
    if ((e = cudaMalloc(&d_insts, (size_t)cap_insts * sizeof(GInst))) != cudaSuccess) {
      cap_insts = 0;
      err = "cudaMalloc(instance table)";
      return SB_ERR_OOM;
    }
  }
  std::vector<GInst> descs(insts.size());
  std::vector<GItem> items;
  for (size_t i = 0; i < insts.size(); ++i) {
    descs[i] = insts[i].desc;
    const GHost &g = insts[i];
    for (int m0 = 0; m0 < g.Np; m0 += kBM)
      for (int r0 = 0; r0 < g.Rp; r0 += nr) items.push_back(GItem{(int)i, m0, r0, grouped_kchunks(g.Kp, g.op)});
  }
  if (order == 0) {
    // longest first, dealt round-robin to the persistent CTAs
    std::stable_sort(items.begin(), items.end(), [](const GItem &a, const GItem &b) { return a.kchunks > b.kchunks; });
  }
  if ((int)items.size() > cap_items) {
    cudaFree(d_items);
    cap_items = std::max<int>((int)items.size(), 2 * cap_items);
    if ((e = cudaMalloc(&d_items, (size_t)cap_items * sizeof(GItem))) != cudaSuccess) {
      cap_items = 0;
      err = "cudaMalloc(item table)";
      return SB_ERR_OOM;
    }
  }
  n_items = (int)items.size();
  if (!d_status) {
    if ((e = cudaMalloc(&d_status, sizeof(uint32_t))) != cudaSuccess) return SB_ERR_OOM;
    cudaMemsetAsync(d_status, 0, sizeof(uint32_t), st);
  }
  if (!descs.empty() &&
      (e = cudaMemcpyAsync(d_insts, descs.data(), descs.size() * sizeof(GInst), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
    err = "upload instance table";
    return SB_ERR_CUDA;
  }
  if (!items.empty() &&
      (e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(GItem), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
    err = "upload item table";
    return SB_ERR_CUDA;
  }
  // the host vectors go out of scope: make the copies complete first
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
    err = std::string("synchronize: ") + cudaGetErrorString(e);
    return SB_ERR_CUDA;
  }
  if (graph) {
    cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
  dirty = false;
  return SB_OK;
}

cudaError_t Grouped::launch(int tick, int emode) { return launch_items(d_items, n_items, tick, emode); }

cudaError_t Grouped::launch_items(const GItem *items_ptr, int count, int tick, int emode) {
  const void *k = nullptr;
  size_t smem = 0;
  if (!grouped_kernel_for(nr, emode, op, &k, &smem)) return cudaErrorInvalidValue;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lk(mu);
    static std::map<const void *, bool> done;
    if (!done[k]) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      done[k] = true;
    }
  }
  if (count == 0) return cudaSuccess;
  const int grid = std::min(count, device_sms());
  const GInst *pi = d_insts;
  const GItem *pit = items_ptr;
  int ni = count;
  uint32_t *ps = d_status;
  void *args[] = {(void *)&pi, (void *)&pit, (void *)&ni, (void *)&tick, (void *)&ps};
  ++launches;
  return cudaLaunchKernel(k, dim3(grid), dim3(kTcThreads), args, smem, st);
}

cudaError_t Grouped::run_steps(int tick0, int count, bool use_graph) {
  if (count <= 0) return cudaSuccess;
  if (!use_graph) {
    for (int s = 0; s < count; ++s) {
      cudaError_t e = launch(tick0 + s, kEmodeStep);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  if (!graph || graph_tick0 != tick0 || graph_count != count) {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    // kernel attributes are set before the capture starts
    const void *k = nullptr;
    size_t smem = 0;
    grouped_kernel_for(nr, kEmodeStep, op, &k, &smem);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const int64_t l0 = launches;
    for (int s = 0; s < count && e == cudaSuccess; ++s) e = launch(tick0 + s, kEmodeStep);
    cudaError_t e2 = cudaStreamEndCapture(st, &gr);
    launches = l0;
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (gr) cudaGraphDestroy(gr);
      return e != cudaSuccess ? e : e2;
    }
    e = cudaGraphInstantiate(&graph, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
      graph = nullptr;
      return e;
    }
    graph_tick0 = tick0;
    graph_count = count;
  }
  launches += count;
  return cudaGraphLaunch(graph, st);
}

cudaError_t Grouped::energy_pass(int tick) {
  for (auto &g : insts) {
    cudaError_t e = cudaMemsetAsync(g.energy, 0, (size_t)g.R * sizeof(double), st);
    if (e != cudaSuccess) return e;
  }
  return launch(tick, kEmodeEnergy);
}

cudaError_t Grouped::energy_pass_for(const std::vector<int> &idx, int tick) {
  std::vector<GItem> items;
  for (int i : idx) {
    const GHost &g = insts[i];
    cudaError_t e = cudaMemsetAsync(g.energy, 0, (size_t)g.R * sizeof(double), st);
    if (e != cudaSuccess) return e;
    for (int m0 = 0; m0 < g.Np; m0 += kBM)
      for (int r0 = 0; r0 < g.Rp; r0 += nr) items.push_back(GItem{i, m0, r0, grouped_kchunks(g.Kp, g.op)});
  }
  if (items.empty()) return cudaSuccess;
  if ((int)items.size() > cap_sub) {
    cudaFree(d_sub_items);
    cap_sub = std::max<int>((int)items.size(), 2 * cap_sub);
    cudaError_t e = cudaMalloc(&d_sub_items, (size_t)cap_sub * sizeof(GItem));
    if (e != cudaSuccess) {
      cap_sub = 0;
      return e;
    }
  }
  cudaError_t e = cudaMemcpyAsync(d_sub_items, items.data(), items.size() * sizeof(GItem), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  e = launch_items(d_sub_items, (int)items.size(), tick, kEmodeEnergy);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);  // `items` is a host temporary
}

// ---- autotuning: replica tile and item order, timed on the batch itself ----

std::string Grouped::tune_key() const {
  int64_t chunks = 0;
  int rmax = 0;
  for (const auto &g : insts) {
    chunks += (int64_t)(g.Np / kBM) * grouped_kchunks(g.Kp, g.op);
    rmax = std::max(rmax, g.R);
  }
  // bucket by total work (log2) and replica count
  int b = 0;
  while ((int64_t(1) << b) < chunks) ++b;
  return std::to_string(rmax) + ":" + std::to_string(b) + ":" + std::to_string(insts.size() > 64 ? 2 : insts.size() > 8 ? 1 : 0) +
         (op == kGopE2m1 ? ":e2m1" : (op == kGopE2m3 ? ":e2m3" : ":e4m3"));
}

std::vector<std::pair<int, int>> Grouped::candidates(int R) {
  std::vector<std::pair<int, int>> c;
  std::vector<int> nrs;
  if (R <= 32) nrs = {32};
  else if (R <= 64) nrs = {64, 32};
  else nrs = {128, 64};
  for (int v : nrs)
    for (int o : {0, 1}) c.push_back({v, o});
  return c;
}

}  // namespace sbk
