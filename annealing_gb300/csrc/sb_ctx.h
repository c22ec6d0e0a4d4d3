// The context behind the opaque sb_ctx handle (shared by the solve, batch and serving code).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "sb.h"

namespace sbs {
struct Server;
}
struct NmfaCache;  // sb_nmfa.cpp

struct sb_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::mutex mu;
  std::string last_error;
  int64_t hbm_budget = 0;
  int max_inflight = 64;
  sb_plan *cached = nullptr;  // most recent sb_solve plan, reused when the shape matches
  sbs::Server *server = nullptr;
  NmfaCache *nmfa = nullptr;  // device buffers of the last NMFA shape
  int64_t wait_cycles = 0;    // bounded-wait limit of the tensor-core kernels (0: the default)
  int32_t debug_skip_step = -1;  // sb_debug_skip_publish: consumed by the next tensor-core solve
};
