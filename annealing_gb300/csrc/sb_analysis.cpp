// Time-to-target analysis of energy traces (host only).
//
// The reference judges its SB programs by their energy traces (print_energy, SB/CUDA_GPU/
// m2_opt.cu:77-91, saved as plot_figure/plot_energy_decrease/*_stats.csv): for every trial the
// first time its trace goes below a target energy, summarised as best / mean / worst over the
// trials that get there (plot_figure/plot_energy_decrease/plot.r:88-240, targets -62059 and
// -60278); and its test script turns a success rate into the time needed to reach the target with
// probability P, t * ln(1 - P) / ln(1 - p_s) (SA_naive/CUDA_GPU/tests/test.sh:26-32, P = 0.99).
// sb_time_to_target computes both from a trace laid out as sb_result.energy_trace_all.
#include <math.h>

#include <limits>

#include "sb.h"
#include "sb_host.h"

extern "C" sb_status sb_time_to_target(const double *energies, const double *times_ms, int32_t rows,
                                       int32_t trials, int32_t times_per_trial, double threshold,
                                       double run_ms, double p_target, sb_tts *out) {
  if (!energies || !times_ms || !out || rows < 1 || trials < 1 || (times_per_trial != 0 && times_per_trial != 1) ||
      !(p_target > 0.0 && p_target < 1.0) || !(run_ms >= 0.0)) {
    sbh::set_thread_error("sb_time_to_target: energies, times and out are required; rows, trials >= 1; "
                          "times_per_trial 0 or 1; 0 < p_target < 1; run_ms >= 0");
    return SB_ERR_INVALID_ARG;
  }
  const double nan = std::numeric_limits<double>::quiet_NaN();
  const double inf = std::numeric_limits<double>::infinity();
  int32_t reached = 0, final_ok = 0;
  double best = inf, worst = -inf, sum = 0.0;
  for (int32_t k = 0; k < trials; ++k) {
    // first passage: the first row whose energy is strictly below the target (plot.r:94-104)
    for (int32_t r = 0; r < rows; ++r) {
      const size_t at = (size_t)r * trials + k;
      if (energies[at] < threshold) {
        const double t = times_ms[times_per_trial ? at : (size_t)r];
        best = t < best ? t : best;
        worst = t > worst ? t : worst;
        sum += t;
        ++reached;
        break;
      }
    }
    // success of the run: its final energy below the target (test.sh:29, `$1 < par`)
    if (energies[(size_t)(rows - 1) * trials + k] < threshold) ++final_ok;
  }
  out->trials = trials;
  out->reached = reached;
  out->succeeded = final_ok;
  out->best_ms = reached ? best : nan;
  out->worst_ms = reached ? worst : nan;
  out->mean_ms = reached ? sum / reached : nan;
  const double ps = (double)final_ok / (double)trials;
  out->success_rate = ps;
  // test.sh:32; its edges (ln 0 when every run succeeds, division by ln 1 = 0 when none does) are
  // taken as: one run when the success rate already reaches p_target, never when it is zero
  if (final_ok == 0)
    out->tts_ms = inf;
  else if (ps >= p_target)
    out->tts_ms = run_ms;
  else
    out->tts_ms = run_ms * log1p(-p_target) / log1p(-ps);
  return SB_OK;
}
