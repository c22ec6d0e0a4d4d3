// Internal host-side declarations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "sb.h"

namespace sbh {
void problem_scan(sb_problem *p);
sb_status load_graph(const char *path, const sb_graph_opts *opts, sb_problem *out,
                     std::string &err);
void set_thread_error(const std::string &e);
const char *thread_error();
}  // namespace sbh

namespace sbk {

// Tensor-core field engine for one dense instance with R replicas (sb_tc.cu).
struct TcEngine;

struct TcSetup {
  int variant;  // 1 bSB, 2 dSB
  int dtype;    // TcDtype
  int n, R;
  int xp;       // pitch of the x / y state rows (floats)
};

// Builds the tensor-core operand form of J from the padded FP32 J on the device ([n][jp]).
sb_status tc_create(TcEngine **out, const TcSetup &s, const float *dJ, int jp, std::string &err,
                    cudaStream_t st);
void tc_destroy(TcEngine *e);
int64_t tc_footprint(const TcSetup &s);
// Builds the step-0 operand (sign(x) or x hi/lo) from the initial state.
cudaError_t tc_prepare(TcEngine *e, const float *x, cudaStream_t st);
// One SB step: field from operand buffer (t & 1), in-place x / y update, next operand into
// buffer ((t + 1) & 1). energy (may be null): += energy of s(t) per replica (dSB only).
cudaError_t tc_step(TcEngine *e, int t, float *x, float *y, const float *h, float pump, float c0,
                    float dt, float dta0, double *energy, uint32_t *status, cudaStream_t st);
// Field-only pass on operand buffer (t & 1): energy of s(t) per replica (dSB, integer J).
cudaError_t tc_energy(TcEngine *e, int t, const float *x, const float *h, double *energy,
                      uint32_t *status, cudaStream_t st);
int tc_dtype(const TcEngine *e);

}  // namespace sbk
