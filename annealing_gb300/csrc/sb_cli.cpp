// `sb` — drop-in command line for the reference program `./opt <graph>` (SB/CUDA_GPU/Makefile:
// 8-12, m2_opt.cu:100-221).
//
// With no options it runs what m2_opt.cu runs: aSB, STEP = 100, one trial (TIMES = 1), the
// reference's xorshift initial state, xi = 0.01565, and writes output.txt with one energy per trial
// (m2_opt.cu:206-210). Options select bSB / dSB, replicas, schedule and field precision, and add
// best_spins.txt (one +1/-1 per line) and a JSON summary on stdout. --target E adds the
// time-to-target summary of the run's replica traces (plot_energy_decrease/plot.r:88-240,
// SA_naive/CUDA_GPU/tests/test.sh:26-32). --variant sqa runs simulated quantum annealing, the
// drop-in for the reference's SQA program (SQA_fully/fully_test/pre_calculate.cu: output.txt holds
// each trial's final slice-0 energy, :242-246; --trace prints each step's energy, :236).
// --variant nmfa runs noisy mean-field annealing, the drop-in for NMFA/CUDA_GPU/Ising.cpp (100
// stages of its beta schedule, alpha = sigma = 0.15, seed 1234, one sample; the first line of stdout
// is the elapsed ms it prints, Ising.cpp:48); --steps sets the stages, --replicas the samples,
// --noise / --recombination sigma and alpha, --field fp32|tc the field; output.txt holds each
// sample's energy E = sum_{i<j} J_ij s_i s_j and best_spins.txt the best sample.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "sb.h"

static void usage() {
  printf(
      "Usage:\n"
      "  sb <graph> [--variant asb|bsb|dsb|sqa|nmfa] [--steps S] [--replicas R] [--seed X]\n"
      "             [--dt DT] [--a0 A0] [--c0 C0] [--xi XI] [--mts-m M]\n"
      "             [--field auto|fp32|tc] [--init uniform|reference]\n"
      "             [--n N] [--index-base 0|1] [--strict] [--trace] [--device D]\n"
      "             [--out output.txt] [--spins best_spins.txt] [--json]\n"
      "             [--target E [--p-target P]] [--trotter M] [--noise S] [--recombination A]\n"
      "Graph file: N [E] then lines 'i j J_ij' (i != j) and optional 'i i h_i'.\n");
}

// --variant sqa: one sb_sqa_solve; output.txt gets each trial's final energy
static int run_sqa(sb_ctx *ctx, const sb_problem *prob, const sb_sqa_params &q, const std::string &out_path,
                   const std::string &spins_path, bool json) {
  std::vector<int8_t> spins((size_t)prob->n);
  std::vector<double> energies((size_t)q.replicas);
  std::vector<double> trace(q.trace ? (size_t)q.replicas * q.steps : 0);
  sb_sqa_result r;
  memset(&r, 0, sizeof(r));
  r.best_spins = spins.data();
  r.replica_energies = energies.data();
  r.energy_trace = q.trace ? trace.data() : nullptr;
  const sb_status s = sb_sqa_solve(ctx, prob, &q, &r);
  if (s != SB_OK) {
    fprintf(stderr, "sb: sqa failed: %s (%s)\n", sb_status_string(s), sb_last_error(ctx));
    return 1;
  }
  if (q.trace)
    for (int k = 0; k < q.replicas; ++k)
      for (int t = 0; t < q.steps; ++t)
        printf("trial %d step %d energy %lld\n", k, t, (long long)trace[(size_t)k * q.steps + t]);
  FILE *f = fopen(out_path.c_str(), "w");
  if (f) {
    for (int k = 0; k < q.replicas; ++k) fprintf(f, "%lld\n", (long long)energies[k]);
    fclose(f);
  }
  f = fopen(spins_path.c_str(), "w");
  if (f) {
    for (int i = 0; i < prob->n; ++i) fprintf(f, "%d\n", (int)spins[i]);
    fclose(f);
  }
  if (json)
    printf("{\"n\": %d, \"trotter\": %d, \"replicas\": %d, \"steps\": %d, \"best_energy\": %lld, "
           "\"energy_check_ok\": %d, \"device_ms\": %.6f, \"total_ms\": %.6f, \"spin_updates_per_s\": %.6e}\n",
           prob->n, q.trotter, q.replicas, q.steps, (long long)r.best_energy, r.energy_check_ok, r.device_ms,
           r.total_ms, r.spin_updates_per_s);
  else
    printf("best energy %lld (replica %d), %.3f ms on device, %.4e spin-updates/s\n", (long long)r.best_energy,
           r.best_replica, r.device_ms, r.spin_updates_per_s);
  return 0;
}

// --variant nmfa: one sb_nmfa_solve
static int run_nmfa(sb_ctx *ctx, const sb_problem *prob, const sb_nmfa_params &q, const std::string &out_path,
                    const std::string &spins_path, bool json) {
  std::vector<int8_t> spins((size_t)prob->n);
  std::vector<double> energies((size_t)q.samples);
  sb_nmfa_result r;
  memset(&r, 0, sizeof(r));
  r.best_spins = spins.data();
  r.energies = energies.data();
  const sb_status s = sb_nmfa_solve(ctx, prob, &q, &r);
  if (s != SB_OK) {
    fprintf(stderr, "sb: nmfa failed: %s (%s)\n", sb_status_string(s), sb_last_error(ctx));
    return 1;
  }
  printf("%g\n", r.device_ms);
  FILE *f = fopen(out_path.c_str(), "w");
  if (f) {
    for (int k = 0; k < q.samples; ++k) fprintf(f, "%.17g\n", energies[k]);
    fclose(f);
  }
  f = fopen(spins_path.c_str(), "w");
  if (f) {
    for (int i = 0; i < prob->n; ++i) fprintf(f, "%d\n", (int)spins[i]);
    fclose(f);
  }
  if (json)
    printf("{\"n\": %d, \"samples\": %d, \"stages\": %d, \"best_energy\": %.17g, \"best_sample\": %d, "
           "\"energy_check_ok\": %d, \"device_ms\": %.6f, \"total_ms\": %.6f, \"spin_updates_per_s\": %.6e}\n",
           prob->n, q.samples, q.stages, r.best_energy, r.best_sample, r.energy_check_ok, r.device_ms, r.total_ms,
           r.spin_updates_per_s);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    usage();
    return 0;
  }
  const char *path = nullptr;
  std::string out_path = "output.txt", spins_path = "best_spins.txt";
  bool json = false, have_target = false;
  double target = 0.0, p_target = 0.99;
  int device = 0;
  sb_graph_opts go;
  sb_graph_opts_default(&go);
  int variant = SB_ASB;
  bool sqa = false, nmfa = false;
  // first pass: variant (it sets the defaults)
  for (int i = 1; i < argc; ++i)
    if (!strcmp(argv[i], "--variant") && i + 1 < argc) {
      const char *v = argv[i + 1];
      variant = !strcmp(v, "bsb") ? SB_BSB : !strcmp(v, "dsb") ? SB_DSB : SB_ASB;
      sqa = !strcmp(v, "sqa");
      nmfa = !strcmp(v, "nmfa");
    }
  sb_params p;
  sb_params_default(&p, variant);
  sb_sqa_params q;
  sb_sqa_params_default(&q);
  if (sqa) p.steps = q.steps;
  sb_nmfa_params nq;
  sb_nmfa_params_default(&nq);
  if (nmfa) {
    p.steps = nq.stages;
    p.replicas = nq.samples;
    p.seed = nq.seed;
  }
  for (int i = 1; i < argc; ++i) {
    const char *a = argv[i];
    auto next = [&](void) -> const char * {
      if (i + 1 >= argc) {
        fprintf(stderr, "missing value for %s\n", a);
        exit(2);
      }
      return argv[++i];
    };
    if (!strcmp(a, "--variant")) next();
    else if (!strcmp(a, "--steps")) p.steps = atoi(next());
    else if (!strcmp(a, "--replicas") || !strcmp(a, "--trials")) p.replicas = atoi(next());
    else if (!strcmp(a, "--seed")) p.seed = strtoull(next(), nullptr, 10);
    else if (!strcmp(a, "--dt")) p.dt = (float)atof(next());
    else if (!strcmp(a, "--a0")) p.a0 = (float)atof(next());
    else if (!strcmp(a, "--c0")) p.c0 = (float)atof(next());
    else if (!strcmp(a, "--xi")) p.xi = (float)atof(next());
    else if (!strcmp(a, "--mts-m")) p.mts_m = atoi(next());
    else if (!strcmp(a, "--field")) {
      const char *v = next();
      p.field_mode = !strcmp(v, "fp32") ? SB_FIELD_FP32 : !strcmp(v, "tc") ? SB_FIELD_TC : SB_FIELD_AUTO;
    } else if (!strcmp(a, "--init")) {
      p.init_mode = !strcmp(next(), "reference") ? SB_INIT_REFERENCE : SB_INIT_UNIFORM;
    } else if (!strcmp(a, "--n")) go.n_override = atoi(next());
    else if (!strcmp(a, "--index-base")) go.index_base = atoi(next());
    else if (!strcmp(a, "--strict")) go.strict = 1;
    else if (!strcmp(a, "--trace")) p.trace = 1;
    else if (!strcmp(a, "--device")) device = atoi(next());
    else if (!strcmp(a, "--out")) out_path = next();
    else if (!strcmp(a, "--spins")) spins_path = next();
    else if (!strcmp(a, "--json")) json = true;
    else if (!strcmp(a, "--target")) {
      target = atof(next());
      have_target = true;
    } else if (!strcmp(a, "--p-target")) p_target = atof(next());
    else if (!strcmp(a, "--trotter")) q.trotter = atoi(next());
    else if (!strcmp(a, "--noise")) nq.noise = (float)atof(next());
    else if (!strcmp(a, "--recombination")) nq.recombination = (float)atof(next());
    else if (!strcmp(a, "-h") || !strcmp(a, "--help")) {
      usage();
      return 0;
    } else if (a[0] == '-') {
      fprintf(stderr, "unknown option %s\n", a);
      return 2;
    } else path = a;
  }
  if (!path) {
    usage();
    return 2;
  }
  sb_problem prob;
  sb_status s = sb_load_graph_ex(path, &go, &prob);
  if (s != SB_OK) {
    fprintf(stderr, "sb: %s: %s (%s)\n", path, sb_status_string(s), sb_last_error(nullptr));
    return 1;
  }
  sb_device_opts dopt;
  memset(&dopt, 0, sizeof(dopt));
  dopt.device = device;
  sb_ctx *ctx = nullptr;
  s = sb_create(&ctx, &dopt);
  if (s != SB_OK) {
    fprintf(stderr, "sb: %s (%s)\n", sb_status_string(s), sb_last_error(nullptr));
    sb_problem_free(&prob);
    return 1;
  }
  if (sqa) {
    q.steps = p.steps;
    q.replicas = p.replicas;
    q.seed = p.seed;
    q.rng_mode = p.init_mode == SB_INIT_REFERENCE ? SB_SQA_RNG_REFERENCE : SB_SQA_RNG_HASH;
    q.trace = p.trace;
    const int rc = run_sqa(ctx, &prob, q, out_path, spins_path, json);
    sb_destroy(ctx);
    sb_problem_free(&prob);
    return rc;
  }
  if (nmfa) {
    nq.stages = p.steps;
    nq.samples = p.replicas;
    nq.seed = (uint32_t)p.seed;
    nq.field_mode = p.field_mode;
    const int rc = run_nmfa(ctx, &prob, nq, out_path, spins_path, json);
    sb_destroy(ctx);
    sb_problem_free(&prob);
    return rc;
  }
  std::vector<int8_t> spins((size_t)prob.n);
  std::vector<double> energies((size_t)p.replicas);
  std::vector<double> trace(p.trace ? (size_t)p.steps + 1 : 0);
  if (have_target) p.trace_all = 1;
  std::vector<double> trace_all(have_target ? ((size_t)p.steps + 1) * (size_t)p.replicas : 0);
  sb_result r;
  memset(&r, 0, sizeof(r));
  r.best_spins = spins.data();
  r.replica_energies = energies.data();
  r.energy_trace = p.trace ? trace.data() : nullptr;
  r.energy_trace_all = have_target ? trace_all.data() : nullptr;
  s = sb_solve(ctx, &prob, &p, &r);
  if (s != SB_OK) {
    fprintf(stderr, "sb: solve failed: %s (%s)\n", sb_status_string(s), sb_last_error(ctx));
    sb_destroy(ctx);
    sb_problem_free(&prob);
    return 1;
  }
  if (p.trace)
    for (int t = 0; t <= p.steps; ++t) printf("%d %.17g\n", t, trace[t]);
  FILE *f = fopen(out_path.c_str(), "w");
  if (f) {
    for (int k = 0; k < p.replicas; ++k) {
      if (prob.integer_valued)
        fprintf(f, "%lld\n", (long long)energies[k]);
      else
        fprintf(f, "%.17g\n", energies[k]);
    }
    fclose(f);
  }
  f = fopen(spins_path.c_str(), "w");
  if (f) {
    for (int i = 0; i < prob.n; ++i) fprintf(f, "%d\n", (int)spins[i]);
    fclose(f);
  }
  // every replica is one run; row t of its trace is reached at t / steps of the device time
  sb_tts tts;
  memset(&tts, 0, sizeof(tts));
  if (have_target) {
    std::vector<double> times((size_t)p.steps + 1);
    for (int t = 0; t <= p.steps; ++t) times[t] = p.steps > 0 ? r.device_ms * t / p.steps : 0.0;
    s = sb_time_to_target(trace_all.data(), times.data(), p.steps + 1, p.replicas, 0, target, r.device_ms,
                          p_target, &tts);
    if (s != SB_OK) {
      fprintf(stderr, "sb: time to target: %s (%s)\n", sb_status_string(s), sb_last_error(nullptr));
      have_target = false;
    }
  }
  auto num = [](double v) -> std::string {
    char b[64];
    if (isnan(v)) return "null";
    if (isinf(v)) return v > 0 ? "\"inf\"" : "\"-inf\"";
    snprintf(b, sizeof(b), "%.9g", v);
    return b;
  };
  if (have_target) {
    const std::string line =
        "{\"target\": " + num(target) + ", \"p_target\": " + num(p_target) + ", \"trials\": " +
        std::to_string(tts.trials) + ", \"reached\": " + std::to_string(tts.reached) + ", \"best_ms\": " +
        num(tts.best_ms) + ", \"mean_ms\": " + num(tts.mean_ms) + ", \"worst_ms\": " + num(tts.worst_ms) +
        ", \"succeeded\": " + std::to_string(tts.succeeded) + ", \"success_rate\": " + num(tts.success_rate) +
        ", \"tts_ms\": " + num(tts.tts_ms) + "}";
    printf("time_to_target %s\n", line.c_str());
  }
  if (json) {
    printf(
        "{\"n\": %d, \"replicas\": %d, \"steps\": %d, \"variant\": %d, \"best_energy\": %.17g, "
        "\"best_energy_i64\": %lld, \"energy_check_ok\": %d, \"field_mode\": %d, \"field_dtype\": %d, "
        "\"device_ms\": %.6f, \"total_ms\": %.6f, \"spin_updates_per_s\": %.6e}\n",
        prob.n, p.replicas, p.steps, p.variant, r.best_energy, (long long)r.best_energy_i64,
        r.energy_check_ok, r.field_mode_used, r.field_dtype_used, r.device_ms, r.total_ms,
        r.spin_updates_per_s);
  } else {
    printf("best energy %.17g (replica %d), %.3f ms on device, %.4e spin-updates/s\n",
           r.best_energy, r.best_replica, r.device_ms, r.spin_updates_per_s);
  }
  sb_destroy(ctx);
  sb_problem_free(&prob);
  return 0;
}
