"""Restatement of the reference's time-to-target analysis — TEST INFRASTRUCTURE ONLY.

Pure-Python loops over small traces, written to follow the reference scripts step by step:

* first_passage: SB/CUDA_GPU/plot_figure/plot_energy_decrease/plot.r:88-157 (and the same loop
  for the second target, :159-240). For each trial, walk its rows in order; at the first row whose
  energy is below the target (strict `<`, :94) take that row's time into best (least, :95-97),
  worst (greatest, :98-100), the running sum (:101) and the count (:102), then stop (:103).
  avg = sum / count (:107). plot.r starts best at 10000 and worst at 0 (:89-90) and divides by a
  zero count when no trial gets there; here those cases give None.
* success_cut / success_rate / annealing_time: SA_naive/CUDA_GPU/tests/test.sh:26-32.
  partial = small + (big - small) / 5 in shell integer arithmetic (:26-28); a run succeeds when
  its energy is below partial (`$1 < par`, :29, :38); success_rate = successes / runs (:31);
  annealing_time = time * l(1 - P) / l(1 - success_rate) (:32), P = 0.99 (:22).
"""
from __future__ import annotations

import math


def first_passage(rows_by_trial, threshold):
    """rows_by_trial: per trial a list of (time, energy) rows in step order.
    Returns (count, best, avg, worst); best/avg/worst are None when count is 0."""
    best = None
    worst = None
    total = 0.0
    count = 0
    for rows in rows_by_trial:
        for time, energy in rows:
            if energy < threshold:
                if best is None or time < best:
                    best = time
                if worst is None or time > worst:
                    worst = time
                total = total + time
                count = count + 1
                break
    if count == 0:
        return 0, None, None, None
    return count, best, total / count, worst


def success_cut(energies):
    """test.sh:26-28 on integer energies: small + (big - small) / 5 (integer division)."""
    big = max(energies)
    small = min(energies)
    difference = big - small
    return small + difference // 5


def success_rate(energies, partial):
    successes = 0
    for e in energies:
        if e < partial:
            successes += 1
    return successes / len(energies)


def annealing_time(time, rate, p=0.99):
    """test.sh:32 for 0 < rate < 1."""
    return time * math.log(1.0 - p) / math.log(1.0 - rate)
