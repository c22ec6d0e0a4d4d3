// sb_dsb_solve_noalloc: the tensor-core dSB solve for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs under a device-memory budget owned by its
// host process (a plugin handed buffers by an application's own pool), code that must not risk the
// implicit device-wide synchronisation and unbounded latency of cudaMalloc / cudaFree (real-time
// loops, callbacks), or code that must not fail with an out-of-memory error half-way through.
// For them this entry point takes every input and output as a device buffer the caller owns and
// keeps its own scratch in one fixed array in the library's device memory (below), so it calls no
// allocator at all.
//
// The scratch array is a file-scope __device__ object: every GPU that loads the library holds its
// kNoAllocScratchBytes until the process exits. Host code cannot use the array's name as a device
// address (on the host it names a stand-in object; a kernel given it would fault or silently use
// the wrong memory), so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current, and later calls reuse it. Every call shares
// the one array and the array keeps the last
// call's contents: the parts that must start at zero are cleared by each call, and calls that
// overlap on the GPU (different streams or threads at the same time) race on it.
//
// The call is synchronous: it reads the coupling scan back before the solve (couplings that no
// operand type holds exactly are rejected without running a step) and the device status after it,
// waiting for `stream` each time, so no call can run under stream capture. Integer couplings with |J| <= 4 run on packed E2M1 operands when
// the kernel that keeps J in shared memory fits the shape, others (|J| <= 16) on FP8; both give the
// same bits as sb_solve's tensor-core dSB.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "sb.h"
#include "sb_host.h"
#include "sb_internal.h"

namespace {

constexpr int kMaxN = 2048;
constexpr int kMaxReplicas = 1024;
constexpr int kMaxSteps = 16384;
// J operand (FP8 2048 x 2048; packed E2M1 needs half) + two operand buffers (1024 x 2048) + pump
// table + control words: [0, 2048) per-unit step flags (the solve clears what it uses), then the
// status word and the coupling-scan word.
constexpr size_t kOffA = 0;
constexpr size_t kOffV0 = kOffA + (size_t)kMaxN * kMaxN;
constexpr size_t kOffV1 = kOffV0 + (size_t)kMaxReplicas * kMaxN;
constexpr size_t kOffPump = kOffV1 + (size_t)kMaxReplicas * kMaxN;
constexpr size_t kOffCtl = kOffPump + (size_t)kMaxSteps * sizeof(float);
constexpr size_t kFlagBytes = 2048;
constexpr size_t kCtlBytes = 4096;
constexpr size_t kNoAllocScratchBytes = kOffCtl + kCtlBytes;
static_assert(kNoAllocScratchBytes == 8458240, "the size stated in sb.h");

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

// coupling-scan bits
constexpr uint32_t kNotFp8Exact = 1u;   // a coupling is not an integer with |J| <= 16
constexpr uint32_t kNotE2m1Exact = 2u;  // a coupling is not an integer with |J| <= 4

std::mutex g_mu;
void *g_scratch_ptr[64] = {nullptr};

// pumps[t] = a0 - a0 * t / steps rounded as the host's sb_pump does (double, then float).
__global__ void noalloc_pumps_kernel(float *pumps, float a0, int steps) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= steps) return;
  const double a = __ddiv_rn(__dmul_rn((double)a0, (double)t), (double)steps);
  pumps[t] = __fsub_rn(a0, __double2float_rn(a));
}

// Which operand types hold the couplings exactly: FP8 E4M3 every integer |J| <= 16, E2M1 every
// integer |J| <= 4.
__global__ void noalloc_scan_kernel(const float *J, size_t count, uint32_t *scan) {
  uint32_t bits = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count;
       k += (size_t)gridDim.x * blockDim.x) {
    const float v = J[k], a = fabsf(v);
    if (!(a <= 16.0f) || v != truncf(v)) {
      bits = kNotFp8Exact | kNotE2m1Exact;
      break;
    }
    if (a > 4.0f) bits |= kNotE2m1Exact;
  }
  bits = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && bits) atomicOr(scan, bits);
}

sb_status fail(sb_status s, const std::string &msg) {
  sbh::set_thread_error(msg);
  return s;
}

}  // namespace

extern "C" sb_status sb_dsb_solve_noalloc(const float *d_J, const float *d_h, int32_t n,
                                          int32_t replicas, int32_t steps, uint64_t seed, float dt,
                                          float a0, float c0, float *d_x, float *d_y,
                                          double *d_energies, void *stream) {
  if (!d_J || !d_x || !d_y || !d_energies)
    return fail(SB_ERR_INVALID_ARG, "sb_dsb_solve_noalloc: J, x, y and energies must be device buffers");
  if (n < 1 || n > kMaxN || replicas < 1 || replicas > kMaxReplicas || steps < 0 || steps > kMaxSteps)
    return fail(SB_ERR_INVALID_ARG,
                "sb_dsb_solve_noalloc: limits are n <= 2048, replicas <= 1024, steps <= 16384 (got n=" +
                    std::to_string(n) + ", replicas=" + std::to_string(replicas) + ", steps=" +
                    std::to_string(steps) + ")");
  if (!(c0 > 0.0f) || !(dt > 0.0f) || !isfinite(a0))
    return fail(SB_ERR_INVALID_ARG, "sb_dsb_solve_noalloc: c0 and dt must be positive, a0 finite");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(SB_ERR_NO_DEVICE, "sb_dsb_solve_noalloc: no current CUDA device");
  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
      cudaDeviceProp prop;
      if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || !(prop.major == 10 && prop.minor == 3))
        return fail(SB_ERR_NO_DEVICE, "sb_dsb_solve_noalloc: kernels are built for sm_103a");
      sbk::init_kernel_attributes();
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail(SB_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t *sc = (uint8_t *)base;
  uint32_t *flags = (uint32_t *)(sc + kOffCtl);
  uint32_t *status = (uint32_t *)(sc + kOffCtl + kFlagBytes);
  uint32_t *scan = status + 1;
  float *pumps = (float *)(sc + kOffPump);
  cudaError_t e;
  std::string where;
  uint32_t scan_bits = 0, hstatus = 0;
  bool fp4 = false;
  size_t a_bytes = 0, v_bytes = 0, f_bytes = 0;
#define NA_CUDA(call)                       \
  if ((e = (call)) != cudaSuccess) {        \
    where = #call;                          \
    goto cuda_fail;                         \
  }
  // The coupling scan comes first, so that couplings no operand type holds exactly are rejected
  // before any solve work; it also picks the operand type (packed E2M1 when every coupling allows
  // it and the kernel that keeps J in shared memory fits this shape, else FP8).
  NA_CUDA(cudaMemsetAsync(sc + kOffCtl, 0, kCtlBytes, st));
  noalloc_scan_kernel<<<152, 256, 0, st>>>(d_J, (size_t)n * n, scan);
  NA_CUDA(cudaGetLastError());
  NA_CUDA(cudaMemcpyAsync(&scan_bits, scan, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  NA_CUDA(cudaStreamSynchronize(st));
  if (scan_bits & kNotFp8Exact)
    return fail(SB_ERR_UNSUPPORTED, "sb_dsb_solve_noalloc: couplings must be integers with |J| <= 16");
  fp4 = !(scan_bits & kNotE2m1Exact) && sbk::tc_external_sizes(n, replicas, true, &a_bytes, &v_bytes, &f_bytes);
  if (!fp4 && !sbk::tc_external_sizes(n, replicas, false, &a_bytes, &v_bytes, &f_bytes))
    return fail(SB_ERR_UNSUPPORTED, "sb_dsb_solve_noalloc: no single-pass tensor-core kernel for this shape");
  if (a_bytes > kOffV0 - kOffA || v_bytes > kOffV1 - kOffV0 || f_bytes > kFlagBytes)
    return fail(SB_ERR_UNSUPPORTED, "sb_dsb_solve_noalloc: shape does not fit the scratch tiling");
  // what must start at zero: both operand buffers (their padding is never written) and the
  // caller's energy accumulators; the solve clears its own flags
  NA_CUDA(cudaMemsetAsync(sc + kOffV0, 0, v_bytes, st));
  NA_CUDA(cudaMemsetAsync(sc + kOffV1, 0, v_bytes, st));
  NA_CUDA(cudaMemsetAsync(d_energies, 0, (size_t)replicas * sizeof(double), st));
  if (steps > 0) {
    noalloc_pumps_kernel<<<(steps + 255) / 256, 256, 0, st>>>(pumps, a0, steps);
    NA_CUDA(cudaGetLastError());
  }
  NA_CUDA(sbk::launch_init_uniform(d_x, d_y, n, replicas, n, seed, st));
  {
    sbk::TcExternal ext;
    ext.J = d_J;
    ext.jp = n;
    ext.h = d_h;
    ext.n = n;
    ext.R = replicas;
    ext.xp = n;
    ext.x = d_x;
    ext.y = d_y;
    ext.fp4 = fp4;
    ext.a = sc + kOffA;
    ext.v0 = sc + kOffV0;
    ext.v1 = sc + kOffV1;
    ext.flags = flags;
    ext.status = status;
    ext.pumps = pumps;
    ext.steps = steps;
    ext.c0 = c0;
    ext.dt = dt;
    ext.dta0 = dt * a0;
    ext.energy = d_energies;
    NA_CUDA(sbk::tc_dsb_external(ext, st));
  }
  NA_CUDA(cudaMemcpyAsync(&hstatus, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  NA_CUDA(cudaStreamSynchronize(st));
  if (hstatus & sbk::kErrWaitTimeout) return fail(SB_ERR_TIMEOUT, "sb_dsb_solve_noalloc: a device wait timed out");
  if (hstatus) return fail(SB_ERR_CUDA, "sb_dsb_solve_noalloc: " + sbh::device_status_text(hstatus));
#undef NA_CUDA
  return SB_OK;
cuda_fail:
  return fail(e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA,
              std::string("sb_dsb_solve_noalloc: ") + where + ": " + cudaGetErrorString(e));
}
