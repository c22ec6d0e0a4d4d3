// Host-side state of the grouped tensor-core path (sb_grouped.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "sb.h"

namespace sbk {

// Operand types of the grouped kernel: FP8 E4M3 (integer |J| <= 16), packed E2M1 (|J| <= 4), or
// packed E2M3, six bits per value (|J| <= 16 held as J / 4 against signs of +-4, exact products).
enum GOperand : int { kGopFp8 = 0, kGopE2m1 = 1, kGopE2m3 = 2 };

// Per-instance descriptor read by the grouped kernel (device memory, 64-byte aligned for the
// tensor maps).
struct alignas(64) GInst {
  CUtensorMap tmA;       // J operand [Np][Kp], 128 x 128-byte shared-memory boxes, 128B swizzle
  CUtensorMap tmB[2];    // V operand [Rp][Kp] buffers, 128-byte x NR boxes
  uint8_t *v[2];         // the V buffers
  float *x, *y;          // state [R][xp]
  const float *h;        // fields or null
  double *energy;        // [R] energies (energy pass)
  const float *pumps;    // [steps] a0 - a(t)
  int n, Kp, R, Rp, xp;
  int t0;                // the instance's step t = tick - t0
  float c0, dt, dta0;
  int kbytes;            // bytes of one operand row in global memory: Kp (FP8), Kp / 2 (E2M1), 3 Kp / 4 (E2M3)
};

// One work item: a 128-spin x NR-replica tile of one instance.
struct GItem {
  int inst, m0, r0, kchunks;
};

// dSB with integer |J| <= 16 (exact E2M3 and FP8 operands) and n * 16 < 2^24 (exact FP32 accumulation).
bool grouped_supports(const sb_problem *p, const sb_params *prm);
// ... and integer |J| <= 4: exact as packed E2M1 operands (half the bytes of FP8)
bool grouped_fp4_exact(const sb_problem *p);
// device bytes one instance holds while resident
int64_t grouped_instance_bytes(int n, int R, int steps, int nr, int op = kGopFp8);
// K chunks (128 bytes of shared memory each) of an instance's operand rows
inline int grouped_kchunks(int Kp, int op) { return op == kGopE2m1 ? Kp / 256 : Kp / 128; }

struct GHost {
  int tag = 0;                  // caller's index / ticket
  const sb_problem *prob = nullptr;
  int n = 0, R = 0, steps = 0, t0 = 0, Np = 0, Kp = 0, Rp = 0, xp = 0;
  int kbytes = 0;  // operand row bytes in global memory (Kp, Kp / 2 for E2M1, 3 Kp / 4 for E2M3)
  int op = kGopFp8;
  float c0 = 0, dt = 0, dta0 = 0;
  uint64_t seed = 0;
  uint8_t *a = nullptr, *v[2] = {nullptr, nullptr};
  float *x = nullptr, *y = nullptr, *h = nullptr, *pumps = nullptr;
  double *energy = nullptr;
  GInst desc;
};

// Pinned host staging for packed couplings (one per thread that prepares instances).
struct Staging {
  uint8_t *pin = nullptr;
  size_t bytes = 0;
  ~Staging() {
    if (pin) cudaFreeHost(pin);
  }
};

class Grouped {
 public:
  // operand: the type every instance's couplings are held in (GOperand)
  explicit Grouped(cudaStream_t s, int replica_tile, int item_order, int operand = kGopFp8)
      : st(s), nr(replica_tile), order(item_order), op(operand) {}
  ~Grouped();
  // Uploads p (host) with J packed to the operand type, seeds the state. t0: the tick at which its
  // step 0 runs.
  sb_status add(const sb_problem *p, const sb_params *prm, uint64_t seed, int t0, int tag, std::string &err);
  // The two halves of add: prepare builds a complete instance on stream `st` (any thread; memory
  // from the stream-ordered pool), attach makes it resident from tick t0 (the engine's thread).
  static sb_status prepare(GHost &g, const sb_problem *p, const sb_params *prm, uint64_t seed, int tag, int nr,
                           cudaStream_t st, Staging &stg, std::string &err, int op = kGopFp8);
  void attach(GHost &g, int t0);
  static void release(GHost &g, cudaStream_t s);
  static sb_status init_state_on(GHost &g, uint64_t seed, cudaStream_t st, std::string &err);
  void remove(int idx);
  // Changes the replica tile (reallocates the operand buffers; the state must be re-initialised).
  sb_status retile(int new_nr, std::string &err);
  void clear();
  // Re-uploads the instance / item tables after add / remove (synchronous).
  sb_status sync_tables(std::string &err);
  // Steps ticks [tick0, tick0 + count) for every resident instance (a CUDA graph when use_graph).
  cudaError_t run_steps(int tick0, int count, bool use_graph);
  // Energies of every resident instance's current spins (instances must be at step t = tick - t0).
  cudaError_t energy_pass(int tick);
  // The same for a subset of resident instances (indices into insts).
  cudaError_t energy_pass_for(const std::vector<int> &idx, int tick);
  // Index of the resident instance with this tag, or -1.
  int find(int tag) const {
    for (size_t i = 0; i < insts.size(); ++i)
      if (insts[i].tag == tag) return (int)i;
    return -1;
  }
  sb_status init_state(GHost &g, uint64_t seed, std::string &err);
  std::string tune_key() const;
  static std::vector<std::pair<int, int>> candidates(int R);
  void set_order(int o) {
    if (o != order) {
      order = o;
      dirty = true;
    }
  }

  cudaStream_t st;
  int nr, order;
  int op;
  std::vector<GHost> insts;
  int64_t launches = 0;
  int n_items = 0;
  uint32_t *d_status = nullptr;

 private:
  cudaError_t launch(int tick, int emode);
  cudaError_t launch_items(const GItem *items, int count, int tick, int emode);
  GItem *d_sub_items = nullptr;
  int cap_sub = 0;
  void free_instance(GHost &g);
  GInst *d_insts = nullptr;
  GItem *d_items = nullptr;
  int cap_insts = 0, cap_items = 0;
  float *d_stage = nullptr;
  size_t stage_bytes = 0;
  Staging stg_;
  bool dirty = true;
  cudaGraphExec_t graph = nullptr;
  int graph_tick0 = -1, graph_count = -1;
};

}  // namespace sbk
