/*
 * sb.h — C ABI of the GB300 simulated-bifurcation (SB) Ising solver.
 *
 * The reference program (strongshih/Annealing, SB/CUDA_GPU/m2_opt.cu) has no library
 * interface: its contract is `./opt <graph>` -> output.txt (one energy per trial).
 * Every entry point below names the piece of that program it replaces:
 *
 *   sb_load_graph   <- the graph reader in main()           SB/CUDA_GPU/m2_opt.cu:111-123
 *   sb_solve        <- the trial loop + step loop + energy   SB/CUDA_GPU/m2_opt.cu:152-203
 *                      (prepare_points :48-56, UpdateTwice :58-75, cublasSgemv :169,
 *                       host energy :192-202)
 *   sb_energy_i64 / sb_energy_f64
 *                   <- the host energy loop                  SB/CUDA_GPU/m2_opt.cu:192-202
 *   sb_params.trace <- print_energy (per-step energy trace)  SB/CUDA_GPU/m2_opt.cu:77-91
 *                      (filled into sb_result.energy_trace)
 *   sb_sqa_solve    <- the SQA program SQA_fully/fully_test/pre_calculate.cu (main :158-257;
 *                      preapare_spins :38-51, reduce :99-149, update_spins :53-84)
 *   sb_nmfa_solve / sb_gpu_nmfa
 *                   <- gpu_nmfa (NMFA/CUDA_GPU/src/cuda_nmfa.h:10-14, nmfa.cu:142-199) and its
 *                      kernel gpu_nmfa_kernel (nmfa.cu:54-140); sb_nmfa_schedule <- the beta
 *                      schedule of NMFA/CUDA_GPU/Ising.cpp:37-43
 *   sb_time_to_target
 *                   <- the trace analysis of plot_energy_decrease/plot.r:88-240 and the
 *                      success-probability time of SA_naive/CUDA_GPU/tests/test.sh:26-32
 *   sb_create / sb_destroy
 *                   <- cublasCreate + the cudaMalloc block   SB/CUDA_GPU/m2_opt.cu:106-145
 *
 * The one library-style precedent in the reference repository is
 *   float gpu_nmfa(int N, float* J, std::vector<float> betas, ...)   NMFA/CUDA_GPU/src/cuda_nmfa.h:10-14
 * (caller-owned J, returns elapsed ms). This ABI keeps that shape — caller-owned host buffers,
 * plain pointers and sizes — but reports errors as status codes instead of exit()/assert
 * (SB/CUDA_GPU/m2_opt.cu:24-36, :113). Nothing here throws or exits.
 *
 * Threading: one CUDA stream per context; every call on a context is serialised by the context's
 * own mutex, so a context may be shared by threads. Different contexts run concurrently.
 *
 * Energy convention (the reference project's README.md:9-13): H(s) = -sum_{i<j} J_ij s_i s_j - sum_i h_i s_i, with
 * s_i = (x_i > 0) ? +1 : -1 (SB/CUDA_GPU/m2_opt.cu:197-198). With h = 0 this is exactly the value
 * the reference writes to output.txt (it stores -E, m2_opt.cu:202).
 */
#ifndef SB_H
#define SB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SB_ABI_VERSION 3  /* 3: sb_problem gained stats_valid / sum_j / sum_j2 */

typedef enum sb_status {
  SB_OK = 0,
  SB_ERR_INVALID_ARG = 1,   /* a NULL pointer, a size out of range, an unknown enum value */
  SB_ERR_IO = 2,            /* the graph file cannot be opened or read */
  SB_ERR_PARSE = 3,         /* malformed line, index out of range, non-numeric weight */
  SB_ERR_CUDA = 4,          /* a CUDA runtime call failed; sb_last_error() has the text */
  SB_ERR_OOM = 5,           /* device or host allocation failed / over the context's HBM budget */
  SB_ERR_UNSUPPORTED = 6,   /* the requested field mode cannot represent this problem exactly */
  SB_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up (kernel returned a status) */
  SB_ERR_BUSY = 8,          /* serving queue is full */
  SB_ERR_NOT_FOUND = 9,     /* unknown ticket */
  SB_ERR_CANCELLED = 10,    /* the request was cancelled before it finished */
  SB_ERR_NO_DEVICE = 11,    /* no CUDA device, or the device is not sm_103 */
  SB_ERR_PENDING = 12       /* sb_poll: request not finished yet */
} sb_status;

/* SB variants.
 *  SB_ASB: the reference's adiabatic SB with multiple-time-step (MTS) integration:
 *          M local sub-steps  x += detune*y*deltaT; y -= deltaT*(K x^3 + (detune - p) x)
 *          then the coupling kick  y += DeltaT*xi * J x   (m2_opt.cu:58-75, :169), p = s/steps.
 *  SB_BSB: ballistic SB (Goto et al., Sci. Adv. 7, eabe7953, 2021):
 *          y += dt*(-(a0 - a(t)) x + c0 (J x + h)); x += dt*a0*y; |x|>1 -> x = sign x, y = 0.
 *  SB_DSB: discrete SB: the same with J*sign(x) in place of J*x. */
typedef enum sb_variant { SB_ASB = 0, SB_BSB = 1, SB_DSB = 2 } sb_variant;

/* How the field J*v is computed.
 *  SB_FIELD_AUTO: tensor cores when replicas >= 32 and the problem allows an exact/declared
 *                 precision, otherwise the plain FP32 kernel.
 *  SB_FIELD_FP32: the plain fused FP32 kernel (the drop-in form): the whole solve in one cooperative
 *                 launch when the rows fit one co-resident grid (n <= 2048, ceil(n / 16) x replicas
 *                 CTAs on the SMs, no energy trace), else one launch per step; the same bits either
 *                 way (environment SB_PLAIN_PERSIST=0 keeps one launch per step).
 *  SB_FIELD_TC:   tcgen05 tensor cores. dSB with integer |J| <= 4 and n <= ~2300: packed E2M1
 *                 operands with J resident in shared memory, FP32 accumulation (bit-exact).
 *                 dSB with integer |J| <= 16: FP8 E4M3 operands (grouped batches and serving:
 *                 packed E2M3, J / 4 in six bits), FP32 accumulation (bit-exact).
 *                 dSB with integer |J| <= 256: BF16 operands (bit-exact).
 *                 dSB with real J: BF16 hi+lo split of J. bSB: BF16 hi+lo split of J and of x
 *                 (three products), FP32 accumulation. aSB is not offered on tensor cores. */
typedef enum sb_field_mode { SB_FIELD_AUTO = 0, SB_FIELD_FP32 = 1, SB_FIELD_TC = 2 } sb_field_mode;

/* Tensor-core operand type (sb_params.operand_dtype, sb_result.field_dtype_used). AUTO takes the
 * narrowest exact type the couplings allow; a forced type must be exact for them as well
 * (SB_ERR_UNSUPPORTED otherwise). */
typedef enum sb_operand_dtype {
  SB_OPERAND_AUTO = 0,
  SB_OPERAND_FP8 = 1,    /* E4M3, integer |J| <= 16 */
  SB_OPERAND_BF16 = 2,   /* integer |J| <= 256 */
  SB_OPERAND_BF16X2 = 3, /* BF16 hi + lo, real J */
  SB_OPERAND_FP4 = 4,    /* packed E2M1, integer |J| <= 4, single-instance dSB */
  SB_OPERAND_FP16X2 = 5, /* FP16 hi + lo, real J scaled by powers of two: 22 bits per operand (opt-in) */
  SB_OPERAND_FP6 = 6     /* packed E2M3 (6 bits), integer |J| <= 16 held as J/4 against signs of +-4:
                            the grouped path (batches, serving); the same products as FP8 */
} sb_operand_dtype;

/* Initial x, y.
 *  SB_INIT_UNIFORM:   x, y iid uniform in [-0.1, 0.1) from a counter-based hash of (seed, replica,
 *                     spin); identical on the device and in the CPU oracle.
 *  SB_INIT_REFERENCE: the reference's prepare_points (m2_opt.cu:48-56): per-spin xorshift32 state
 *                     seeded with the spin index (m2_opt.cu:136-137), values in [0, 0.1);
 *                     replica r takes the values trial r would get. */
typedef enum sb_init_mode { SB_INIT_UNIFORM = 0, SB_INIT_REFERENCE = 1 } sb_init_mode;

/* Graph-file options (sb_load_graph_ex). The reference format is: first integer N, then
 * "i j w" lines with 0-based i != j (m2_opt.cu:115-121). Extensions accepted here:
 * "i i h" lines give the field h_i (the SA_king/CUDA_GPU/tests/king.py:27-28 convention),
 * a header "N E" (rudy / Gset), real-valued weights, and '#' comment lines. */
typedef struct sb_graph_opts {
  int32_t index_base;      /* 0 (reference) or 1 (rudy / Gset); -1 = autodetect: 1 if any index == N
                              and none == 0 */
  int32_t n_override;      /* > 0: use this N instead of the header (the reference ignores the header
                              and uses its compile-time N, m2_opt.cu:10,115) */
  int32_t strict;          /* 1: a repeated edge with a different weight is an error; 0: the last line
                              wins, as in the reference */
} sb_graph_opts;

/* A dense problem instance. J is N*N row-major, symmetric, zero diagonal. */
typedef struct sb_problem {
  int32_t n;
  float *J;                /* n*n */
  float *h;                /* n, or NULL for h = 0 */
  int32_t integer_valued;  /* 1 if every J_ij and h_i is an integer */
  int32_t max_abs_j;       /* max |J_ij| rounded up (valid when integer_valued) */
  int64_t n_edges;         /* number of nonzero J_ij with i < j */
  int32_t lib_owned;       /* 1 when J/h were allocated by sb_load_graph (free with sb_problem_free) */
  int32_t stats_valid;     /* 1 when sum_j / sum_j2 hold the exact off-diagonal sums (set by the scan
                              of sb_problem_init / wrap / load / random, for integer couplings whose
                              sums stay below 2^53): the default c0 then needs no pass over J */
  int64_t sum_j;           /* sum of J_ij over i != j */
  int64_t sum_j2;          /* sum of J_ij^2 over i != j */
} sb_problem;

typedef struct sb_params {
  int32_t variant;         /* sb_variant */
  int32_t field_mode;      /* sb_field_mode */
  int32_t init_mode;       /* sb_init_mode */
  int32_t steps;           /* SB time steps (reference STEP, m2_opt.cu:22) */
  int32_t replicas;        /* independent trajectories run together (reference TIMES runs them
                              one after another, m2_opt.cu:12,152) */
  uint64_t seed;
  /* bSB / dSB */
  float dt;                /* 1.25 */
  float a0;                /* 1.0; a(t) = a0 * t / steps, t = 0 .. steps-1 (m2_opt.cu:158 form) */
  float c0;                /* <= 0: 0.5 / (sqrt(N) * std(J_offdiag)) */
  /* aSB (reference constants, m2_opt.cu:15-22) */
  int32_t mts_m;           /* M = 2 */
  float mts_dt;            /* deltaT = 0.5 */
  float coupling_dt;       /* DeltaT = 1.0 */
  float xi;                /* 0.01565 (m2_opt.cu:18); <= 0: 0.7 * detune / sqrt(N) (its comment, rho = 1) */
  float detune;            /* 1.0 */
  float kerr;              /* K = 1.0 */
  int32_t trace;           /* 1: record the per-step energy trace (min over replicas) */
  int32_t trace_all;       /* 1: record every replica's energy at every step */
  int32_t profile;         /* 1: run the step loop launch by launch (no CUDA graph) with a CUDA
                              event pair around every step kernel; fills kernel_ms_avg */
  int32_t operand_dtype;   /* sb_operand_dtype for the tensor-core field (0: auto) */
} sb_params;

/* Results. The caller owns every array; any of them may be NULL. */
typedef struct sb_result {
  int8_t *best_spins;          /* [n]  +1 / -1 of the lowest-energy replica (final state) */
  double *replica_energies;    /* [replicas] final-state energy of each replica: exact for integer
                                  couplings; for real couplings from the FP32 field, except the 8
                                  lowest, which are recomputed in FP64 (best_energy is FP64) */
  double *energy_trace;        /* [steps + 1] min-over-replicas energy of s(t), t = 0..steps (trace) */
  double *energy_trace_all;    /* [(steps + 1) * replicas] (trace_all) */
  float *final_x;              /* [replicas * n] final positions, replica-major */
  float *final_y;              /* [replicas * n] final momenta */
  /* scalar outputs */
  double best_energy;          /* energy of best_spins */
  int64_t best_energy_i64;     /* exact host re-check (integer problems); 0 otherwise */
  int32_t best_replica;
  int32_t field_mode_used;     /* SB_FIELD_FP32 or SB_FIELD_TC */
  int32_t field_dtype_used;    /* 0 fp32, else the sb_operand_dtype used */
  int32_t energy_check_ok;     /* 1 when the host re-check agrees with the device energy */
  double device_ms;            /* CUDA-event time of init + step loop + final energy */
  double kernel_ms_avg;        /* profile == 1: average device time of one launch of the step kernel
                                  (the tensor-core kernel runs every step in one launch), else 0 */
  int32_t steps_per_launch;    /* SB steps one step-kernel launch advances (1 for the per-step plain
                                  kernel, steps for the one-launch plain solve and the TC kernel) */
  int64_t kernel_launches;     /* kernels this call launched on the device */
  double total_ms;             /* host wall time of the call, copies included */
  double spin_updates_per_s;   /* n * replicas * steps / (device_ms / 1e3) */
} sb_result;

typedef struct sb_device_opts {
  int32_t device;              /* CUDA ordinal */
  void *stream;                /* cudaStream_t to run on, or NULL for a stream the context owns */
  int64_t hbm_budget_bytes;    /* serving admission budget; <= 0: 80% of free memory at create */
  int32_t max_inflight;        /* serving: most requests resident at once (<= 0: 64) */
} sb_device_opts;

typedef struct sb_ctx sb_ctx;
typedef struct sb_plan sb_plan;

/* ---- library ---- */
const char *sb_status_string(sb_status s);
int32_t sb_abi_version(void);
void sb_params_default(sb_params *p, int32_t variant);
void sb_graph_opts_default(sb_graph_opts *o);

/* ---- problems (host only, no GPU needed) ---- */
sb_status sb_load_graph(const char *path, sb_problem *out);
sb_status sb_load_graph_ex(const char *path, const sb_graph_opts *opts, sb_problem *out);
sb_status sb_problem_init(sb_problem *p, int32_t n, const float *J, const float *h);
/* Zero-copy form of sb_problem_init: p refers to the caller's J / h (which must stay alive and
 * unchanged while p is used; J must already be symmetric with a zero diagonal). */
sb_status sb_problem_wrap(sb_problem *p, int32_t n, float *J, float *h);
void sb_problem_free(sb_problem *p);
/* Seeded random instance, generated on the host threads: each pair i < j is an edge with
 * probability `density`; an edge's coupling is +-1 (jmax == 1) or uniform in [-jmax, jmax];
 * field_max > 0 adds fields h_i uniform in [-field_max, field_max]. The same seed gives the same
 * instance on any machine and thread count (the generators of SA_naive/CUDA_GPU/tests/fully.py
 * and NMFA/CUDA_GPU/tests/fully.py play this role in the reference, unseeded). */
sb_status sb_problem_random(sb_problem *p, int32_t n, double density, int32_t jmax,
                            int32_t field_max, uint64_t seed);
/* std of the off-diagonal couplings and the default c0 for that problem */
double sb_coupling_std(const sb_problem *p);
float sb_default_c0(const sb_problem *p);
/* pump term a0 - a(t) for step t (shared by every kernel and the host) */
float sb_pump(float a0, int32_t t, int32_t steps);
/* exact energies: int64 when every J, h is integral (else SB_ERR_UNSUPPORTED), double otherwise */
sb_status sb_energy_i64(const sb_problem *p, const int8_t *spins, int64_t *out);
double sb_energy_f64(const sb_problem *p, const int8_t *spins);
/* the int64 energies of `count` spin vectors (count x n int8, row after row) into out[count]; for
 * couplings in {-1, 0, +1} or |J| <= 127 the matrix is first copied into bit planes / int8, so each
 * vector reads 16x / 4x fewer bytes than sb_energy_i64 does; the same integers either way */
sb_status sb_energies_i64(const sb_problem *p, const int8_t *spins, int32_t count, int64_t *out);

/* ---- time to target (host only, no GPU needed) ----
 * Replaces the reference's trace analysis: per trial, the first time its energy trace goes below
 * a target, summarised over the trials that reach it (SB/CUDA_GPU/plot_figure/
 * plot_energy_decrease/plot.r:88-240), and the time to reach the target with probability P from
 * the success rate p_s of single runs, run_ms * ln(1 - P) / ln(1 - p_s)
 * (SA_naive/CUDA_GPU/tests/test.sh:26-32). energies is laid out as sb_result.energy_trace_all:
 * [rows * trials], row-major (row = step 0..steps); times_ms holds the time at which each row was
 * reached, [rows] shared by all trials (times_per_trial = 0, replicas run together) or
 * [rows * trials] (1, trials run one after another). "Below" is strict, as in both scripts. */
typedef struct sb_tts {
  int32_t trials;
  int32_t reached;      /* trials whose trace went below the target at some row */
  int32_t succeeded;    /* trials whose final row is below the target (the success test) */
  double best_ms;       /* first-passage time: least, mean and greatest over the trials that */
  double mean_ms;       /* reached the target; NaN when none did */
  double worst_ms;
  double success_rate;  /* succeeded / trials */
  double tts_ms;        /* run_ms * ln(1 - p_target) / ln(1 - success_rate); run_ms when the
                           success rate is >= p_target; +inf when no trial succeeded */
} sb_tts;
sb_status sb_time_to_target(const double *energies, const double *times_ms, int32_t rows,
                            int32_t trials, int32_t times_per_trial, double threshold,
                            double run_ms, double p_target, sb_tts *out);

/* ---- contexts ---- */
sb_status sb_create(sb_ctx **out, const sb_device_opts *opts);
sb_status sb_destroy(sb_ctx *ctx);
const char *sb_last_error(sb_ctx *ctx);
/* Bounded device waits. Every wait inside the persistent tensor-core kernels (a dataflow flag of
 * another unit, an mbarrier of a copy or a contraction) gives up after `cycles` SM clock cycles;
 * the kernel then lets the copies and contractions it started finish, frees its tensor memory,
 * returns, and the call returns SB_ERR_TIMEOUT with the context still usable. 0 restores the
 * default (2e9 cycles, about one second at the maximum SM clock). Replaces the reference's
 * gpuErrchk, which ends the program on any CUDA error (m2_opt.cu:24-36). */
sb_status sb_set_wait_limit(sb_ctx *ctx, int64_t cycles);
/* Test hook for the timeout path above, a host-side fault injection: the next tensor-core solve of
 * this context runs with unit 0 (spins 0..127 of the first replica tile) leaving out its
 * published flag of SB step `step`, so the units of its replica column wait for a flag that
 * nothing sets and give up at the wait limit. Nothing faults; no counterpart in the reference. */
sb_status sb_debug_skip_publish(sb_ctx *ctx, int32_t step);

/* One blocking solve from host buffers: upload J, run, copy results back. */
sb_status sb_solve(sb_ctx *ctx, const sb_problem *p, const sb_params *params, sb_result *res);

/* Device-resident form: sb_plan_create uploads J once (converted to the field dtype) and allocates
 * the state; sb_plan_run runs one solve on it (init + steps + final energy) and copies the results
 * out. Used for repeated solves and for timing with inputs resident in HBM. */
sb_status sb_plan_create(sb_ctx *ctx, const sb_problem *p, const sb_params *params, sb_plan **out);
sb_status sb_plan_run(sb_plan *plan, uint64_t seed, sb_result *res);
sb_status sb_plan_destroy(sb_plan *plan);
/* bytes of HBM a plan for (p, params) would hold */
int64_t sb_plan_footprint(const sb_problem *p, const sb_params *params);

/* ---- batches: many instances of uneven size, solved together ----
 * The reference runs one instance per program run and its trials one after another
 * (SB/CUDA_GPU/m2_opt.cu:152). A batch advances every instance, with all of its replicas, by
 * grouped tensor-core launches, the step loop replayed from a CUDA graph (dSB, integer |J| <= 16).
 * Instances whose couplings are integers |J| <= 4 run on packed E2M1 operands (half the bytes), the
 * others on FP8 (params->operand_dtype SB_OPERAND_FP8 / SB_OPERAND_FP4 forces one type); each operand
 * bucket has one grouped launch per SB step, with its replica tile and work order chosen by timing
 * the candidates on the bucket itself (cached per shape). params is shared; instance k uses seed
 * seed + k; results[k] is filled as sb_solve would fill it (arrays sized for instance k). The
 * problems must stay alive until sb_batch_destroy. */
typedef struct sb_batch sb_batch;
sb_status sb_batch_create(sb_ctx *ctx, const sb_problem *problems, int32_t count,
                          const sb_params *params, sb_batch **out);
sb_status sb_batch_run(sb_batch *batch, uint64_t seed, sb_result *results);
sb_status sb_batch_destroy(sb_batch *batch);
sb_status sb_solve_batch(sb_ctx *ctx, const sb_problem *problems, int32_t count,
                         const sb_params *params, sb_result *results);

/* ---- serving: continuous batching ----
 * sb_submit queues a request and returns a ticket at once; the problem (and its J / h) must stay
 * alive until sb_poll has returned the request's final status. A worker thread admits queued
 * requests in arrival order while the context's HBM budget and in-flight limit allow, and
 * advances every admitted request together (one grouped tensor-core launch per step over all
 * resident requests, each on its own schedule), so requests that arrive while others run join
 * them at the next step. Each request retires at its own step budget (energies, best spins, exact
 * host re-check) and its device memory goes to the next. dSB requests with integer |J| <= 16 use
 * the grouped engine; others are solved one at a time between steps. Results equal those of
 * sb_solve with the same parameters (field_mode SB_FIELD_TC for the grouped ones). */
sb_status sb_submit(sb_ctx *ctx, const sb_problem *p, const sb_params *params, uint64_t *ticket);
/* SB_OK when finished (res filled; the ticket is released), SB_ERR_PENDING otherwise, or the
 * request's error (SB_ERR_CANCELLED after sb_cancel). res->best_spins / replica_energies must hold
 * n / replicas entries; res->total_ms is the latency from sb_submit to the result, device_ms the
 * time from admission to retirement. wait_ms < 0 blocks until done. */
sb_status sb_poll(sb_ctx *ctx, uint64_t ticket, sb_result *res, int32_t wait_ms);
sb_status sb_cancel(sb_ctx *ctx, uint64_t ticket);
/* latency of every finished request in submission order: arrival->result ms, and queue stats */
typedef struct sb_serving_stats {
  int64_t submitted, finished, cancelled, inflight, queued;
  int64_t grouped_launches;     /* device steps run by the serving loop */
  double busy_ms;               /* time the worker had work resident */
  int64_t peak_inflight;
  int64_t ticks;                /* SB steps the resident set advanced */
  double admit_ms;              /* summed time spent preparing requests (several threads) */
} sb_serving_stats;
sb_status sb_serving_stats_get(sb_ctx *ctx, sb_serving_stats *out);

/* ---- simulated quantum annealing (SQA), fully connected ----
 * Replaces the reference's GPU SQA program SQA_fully/fully_test/pre_calculate.cu (its main,
 * :158-257): M Trotter slices of the N spins, a diagonal wavefront of M + N - 1 Metropolis updates
 * per slice and annealing step (slice m updates spin (a - m) mod N at iteration a, :63, :221-224),
 * the energy change 2 M s (f - M J_perp (s[m-1] + s[m+1])) with f the exact integer local field
 * (:68-77), acceptance when -log(u) / beta > delta (:79-81), and the schedule
 * Gamma = 8 (1 - p / steps), J_perp = -0.5 log(tanh(Gamma / M * beta)) / beta, beta from 1/16
 * rising by (8 - 1/16) / steps per step (:206-225; sb_sqa_schedule returns it). Couplings: integers
 * with |J| <= 127 (the reference stores char, :164-179), no fields (:176). Replicas are the
 * reference's TIMES trials, run side by side. Energies are those of slice 0, as the reference
 * reports (:230-236), exact (int64). */
enum { SB_SQA_RNG_REFERENCE = 0, /* the reference's random numbers: per-spin xorshift32 seeded with
                                    the spin index, M calls per trial for the initial slices
                                    (:38-51, :186-191), and one fixed random word per spin for every
                                    acceptance test of the run (update_spins never advances it, :71) */
       SB_SQA_RNG_HASH = 1 };     /* initial slices and one uniform per (replica, step, iteration,
                                    slice) from counter hashes of the seed */
typedef struct sb_sqa_params {
  int32_t trotter;    /* M, Trotter slices: 1 <= M <= min(n, 128) (reference: pre_calculate.cu:16) */
  int32_t steps;      /* annealing steps (:15) */
  int32_t replicas;   /* independent runs (:12 TIMES) */
  int32_t rng_mode;   /* SB_SQA_RNG_REFERENCE or SB_SQA_RNG_HASH */
  uint64_t seed;      /* hash mode */
  int32_t trace;      /* 1: every replica's slice-0 energy after every step */
} sb_sqa_params;
typedef struct sb_sqa_result {
  int8_t *best_spins;         /* [n] slice 0 of the lowest-energy replica */
  double *replica_energies;   /* [replicas] final slice-0 energy of each replica */
  double *energy_trace;       /* [replicas * steps] replica-major (trace) */
  int8_t *final_spins;        /* [replicas * trotter * n] every slice of every replica, or NULL */
  double best_energy;
  int64_t best_energy_i64;    /* host re-check of best_spins */
  int32_t best_replica;
  int32_t energy_check_ok;
  double device_ms;           /* CUDA-event time of set-up kernels + the anneal + energies */
  double total_ms;            /* host wall time of the call, copies included */
  double spin_updates_per_s;  /* replicas * trotter * (n + trotter - 1) * steps / device time */
  int64_t kernel_launches;
} sb_sqa_result;
void sb_sqa_params_default(sb_sqa_params *p);
/* beta[p] and J_perp[p] for p = 0 .. steps - 1 (host only) */
void sb_sqa_schedule(int32_t steps, int32_t trotter, float *beta, float *jperp);
sb_status sb_sqa_solve(sb_ctx *ctx, const sb_problem *p, const sb_sqa_params *params, sb_sqa_result *res);

/* ---- dSB without any device allocation ----
 * No counterpart in the reference (its program allocates everything itself, m2_opt.cu:106-145).
 * For callers that cannot call cudaMalloc: code that lives inside a host process which owns the
 * device memory budget (and hands out buffers from its own pool), or that must not pay the
 * implicit synchronisation, latency or out-of-memory risk of cudaMalloc / cudaFree in the middle
 * of its work. It runs the same solve as sb_solve with variant SB_DSB on the tensor-core path
 * (packed E2M1 operands when every coupling is an integer with |J| <= 4 and the shape fits the
 * kernel that keeps J in shared memory, else FP8; the same bits either way), with a uniform initial
 * state from `seed` and the schedule a(t) = a0 t / steps, on device buffers the caller owns:
 * d_J [n*n] row-major (symmetric, zero diagonal, integers |J| <= 16), d_h [n] or NULL, outputs
 * d_x, d_y [replicas*n] (final state, replica-major) and d_energies [replicas] (final energies),
 * all on `stream` (a cudaStream_t, NULL = legacy default stream) of the current device. c0 must be
 * given (> 0; sb_default_c0 on the host problem gives the usual value). The call is synchronous:
 * it waits for `stream` once after scanning the couplings (other couplings return
 * SB_ERR_UNSUPPORTED before any step runs) and again when the solve has finished.
 * Scratch is one fixed array of 8,458,240 bytes in the library's device memory, held by every GPU
 * that loads the library until the process exits; hence the limits n <= 2048, replicas <= 1024,
 * steps <= 16384 (larger sizes return SB_ERR_INVALID_ARG). The first call on a device looks up
 * the array's device address. No call can run under stream capture (each one waits for `stream`
 * and reads its status back into host memory). All calls share the array: calls that overlap on
 * the GPU (other streams or threads at the same time) race. */
sb_status sb_dsb_solve_noalloc(const float *d_J, const float *d_h, int32_t n, int32_t replicas,
                               int32_t steps, uint64_t seed, float dt, float a0, float c0,
                               float *d_x, float *d_y, double *d_energies, void *stream);

/* ---- NMFA: noisy mean-field annealing (NMFA/CUDA_GPU/src/nmfa.cu:54-199) ----
 * Per sample, from s = 0, for each stage (inverse temperature beta) two Gaussian samples z0, z1 are
 * drawn (a per-(sample, spin) XORWOW stream seeded as nmfa.cu:62-76, Box-Muller as :103-109) and two
 * sweeps run, the first with z0 and the second with z1 (:114-134):
 *     s_i <- (1 - alpha) s_i + alpha tanh(beta (norm_i sum_j J_ij s_j + z)),
 *     norm_i = -1 / sqrt(sum_j |J_ij|)   (:93; 0 for a row without couplings),
 * and the sample is sign(s) (s > 0 ? +1 : -1, :139). NMFA minimises E(s) = sum_{i<j} J_ij s_i s_j
 * (its field is -J s); energies below are in that convention (the opposite sign to H above). A
 * sweep reads the states of the previous sweep: the reference's two sweeps of a stage have no
 * barrier between warps, which for up to 32 spins (one warp) is exactly this and beyond that depends
 * on warp timing. The transcendental functions are this library's own FP32 ones (the same
 * operations in the CPU oracle), the reference's are CUDA fast-math intrinsics. */
typedef struct sb_nmfa_params {
  int32_t samples;          /* independent samples (the reference's num_samples, one CTA each there) */
  int32_t stages;           /* number of betas (the reference's SWEEP, Ising.cpp:10) */
  const float *betas;       /* [stages], or NULL for sb_nmfa_schedule(stages) */
  float noise;              /* Gaussian noise scale sigma (Ising.cpp:12, SIGMA = 0.15) */
  float recombination;      /* alpha (Ising.cpp:11, ALPHA = 0.15) */
  uint32_t seed;            /* Ising.cpp:13, SEED = 1234 */
  int32_t field_mode;       /* sb_field_mode. SB_FIELD_FP32: the fused FP32 kernel, every sweep in one
                               cooperative launch when the rows fit one co-resident grid, else one launch
                               per sweep (bit-exact with the oracle either way). SB_FIELD_TC: one persistent tcgen05 launch,
                               the state as BF16 hi + lo against exact BF16 couplings (integer |J| <= 256),
                               FP32 accumulation; within a stated tolerance of the FP32 path.
                               SB_FIELD_AUTO: TC for 32 samples or more when it applies, else FP32. */
} sb_nmfa_params;

typedef struct sb_nmfa_result {
  int8_t *samples;          /* [samples][n] +-1, or NULL */
  float *states;            /* [samples][n] final mean-field states, or NULL */
  double *energies;         /* [samples] E of each sample (NMFA's convention), or NULL */
  int8_t *best_spins;       /* [n] the sample of lowest E, or NULL */
  double best_energy;       /* its E */
  int32_t best_sample;
  int32_t energy_check_ok;  /* 1 when the host re-evaluation of the best sample agrees */
  double device_ms;         /* seeding + all sweeps + the energy pass, CUDA events */
  double total_ms;          /* the whole call, host clock */
  double spin_updates_per_s;  /* n * samples * 2 * stages / device time */
  int64_t kernel_launches;
  int32_t field_mode_used;  /* SB_FIELD_FP32 or SB_FIELD_TC: the path that ran */
} sb_nmfa_result;

/* samples 1, stages 100 with the reference schedule, noise 0.15, recombination 0.15, seed 1234
 * (NMFA/CUDA_GPU/Ising.cpp:8-13), field_mode SB_FIELD_AUTO */
sb_status sb_nmfa_params_default(sb_nmfa_params *p);
/* betas[k] = 1/16 + k (8 - 1/16) / stages, accumulated in FP32 as Ising.cpp:37-43 does */
sb_status sb_nmfa_schedule(int32_t stages, float *betas);
/* NMFA on one problem (no fields h: the reference has none). */
sb_status sb_nmfa_solve(sb_ctx *ctx, const sb_problem *p, const sb_nmfa_params *params, sb_nmfa_result *res);
/* The reference's entry point (cuda_nmfa.h:10-14: float gpu_nmfa(int N, float *J, std::vector<float>
 * betas, int num_samples, int *samples, float noise, float recombination, uint32_t seed)) with C
 * types: J dense n x n row-major on the host, betas[num_betas], samples[num_samples][n] receives
 * +-1, *elapsed_ms the device time (the reference's return value). The reference throws
 * std::invalid_argument when N differs from its compile-time size; here any n >= 1 runs and bad
 * arguments return SB_ERR_INVALID_ARG. */
sb_status sb_gpu_nmfa(sb_ctx *ctx, int32_t n, const float *J, const float *betas, int32_t num_betas,
                      int32_t num_samples, int32_t *samples, float noise, float recombination, uint32_t seed,
                      float *elapsed_ms);

#ifdef __cplusplus
}
#endif
#endif /* SB_H */
