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
// cudaGetSymbolAddress while that device is current, and later calls reuse it. Make that first
// call before any stream capture. Every call shares the one array and the array keeps the last
// call's contents: the parts that must start at zero are cleared by each call, and calls that
// overlap on the GPU (different streams or threads at the same time) race on it.
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
// FP8 J operand (2048 x 2048) + two operand buffers (1024 x 2048) + pump table + control words.
constexpr size_t kOffA = 0;
constexpr size_t kOffV0 = kOffA + (size_t)kMaxN * kMaxN;
constexpr size_t kOffV1 = kOffV0 + (size_t)kMaxReplicas * kMaxN;
constexpr size_t kOffPump = kOffV1 + (size_t)kMaxReplicas * kMaxN;
constexpr size_t kOffCtl = kOffPump + (size_t)kMaxSteps * sizeof(float);
constexpr size_t kNoAllocScratchBytes = kOffCtl + 1024;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr uint32_t kErrNotFp8Exact = 0x100u;  // a coupling is not an integer with |J| <= 16

std::mutex g_mu;
void *g_scratch_ptr[64] = {nullptr};

// pumps[t] = a0 - a0 * t / steps rounded as the host's sb_pump does (double, then float).
__global__ void noalloc_pumps_kernel(float *pumps, float a0, int steps) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= steps) return;
  const double a = __ddiv_rn(__dmul_rn((double)a0, (double)t), (double)steps);
  pumps[t] = __fsub_rn(a0, __double2float_rn(a));
}

// FP8 E4M3 holds the couplings exactly only when each is an integer with |J| <= 16.
__global__ void noalloc_check_kernel(const float *J, size_t count, uint32_t *status) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count;
       k += (size_t)gridDim.x * blockDim.x) {
    const float v = J[k];
    if (!(fabsf(v) <= 16.0f) || v != truncf(v)) {
      atomicOr(status, kErrNotFp8Exact);
      return;
    }
  }
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
  int nr = 0;
  size_t a_bytes = 0, v_bytes = 0;
  sbk::tc_external_sizes(n, replicas, &nr, &a_bytes, &v_bytes);
  if (nr == 0 || a_bytes > kOffV0 - kOffA || v_bytes > kOffV1 - kOffV0)
    return fail(SB_ERR_UNSUPPORTED, "sb_dsb_solve_noalloc: shape does not fit the scratch tiling");
  uint32_t *ctl = (uint32_t *)(sc + kOffCtl);  // [0, 128): per-unit step flags, [192]: status
  uint32_t *status = ctl + 192;
  float *pumps = (float *)(sc + kOffPump);
  cudaError_t e;
  std::string where;
#define NA_CUDA(call)                       \
  if ((e = (call)) != cudaSuccess) {        \
    where = #call;                          \
    goto cuda_fail;                         \
  }
  // what must start at zero: control words, both operand buffers (their padding is never
  // written), the caller's energy accumulators
  NA_CUDA(cudaMemsetAsync(ctl, 0, 1024, st));
  NA_CUDA(cudaMemsetAsync(sc + kOffV0, 0, v_bytes, st));
  NA_CUDA(cudaMemsetAsync(sc + kOffV1, 0, v_bytes, st));
  NA_CUDA(cudaMemsetAsync(d_energies, 0, (size_t)replicas * sizeof(double), st));
  noalloc_check_kernel<<<152, 256, 0, st>>>(d_J, (size_t)n * n, status);
  NA_CUDA(cudaGetLastError());
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
    ext.a = sc + kOffA;
    ext.v0 = sc + kOffV0;
    ext.v1 = sc + kOffV1;
    ext.flags = ctl;
    ext.status = status;
    ext.pumps = pumps;
    ext.steps = steps;
    ext.c0 = c0;
    ext.dt = dt;
    ext.dta0 = dt * a0;
    ext.energy = d_energies;
    NA_CUDA(sbk::tc_dsb_fp8_external(ext, st));
  }
  {
    uint32_t hstatus = 0;
    NA_CUDA(cudaMemcpyAsync(&hstatus, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    if (hstatus & kErrNotFp8Exact)
      return fail(SB_ERR_UNSUPPORTED, "sb_dsb_solve_noalloc: couplings must be integers with |J| <= 16");
    if (hstatus & sbk::kErrWaitTimeout) return fail(SB_ERR_TIMEOUT, "sb_dsb_solve_noalloc: a device wait timed out");
    if (hstatus) return fail(SB_ERR_CUDA, "sb_dsb_solve_noalloc: " + sbh::device_status_text(hstatus));
  }
#undef NA_CUDA
  return SB_OK;
cuda_fail:
  return fail(e == cudaErrorMemoryAllocation ? SB_ERR_OOM : SB_ERR_CUDA,
              std::string("sb_dsb_solve_noalloc: ") + where + ": " + cudaGetErrorString(e));
}
