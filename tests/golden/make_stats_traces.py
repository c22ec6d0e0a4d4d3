"""Pack the reference's published energy traces into a fixture for the time-to-target tests.

Reads SB/CUDA_GPU/plot_figure/plot_energy_decrease/{m1,m2,opt}_stats.csv from a checkout of the
reference (rows "trial cumulative_seconds energy", STEP rows per trial, written by print_energy,
SB/CUDA_GPU/m2_opt.cu:77-91) and writes ref_stats_traces.npz with, per file, the energies as
int32 [trials, steps] and the times as float64 seconds [trials, steps], unchanged.
Usage: python tests/golden/make_stats_traces.py <reference checkout root>
"""
import os
import sys

import numpy as np


def main(root):
    d = os.path.join(root, "SB/CUDA_GPU/plot_figure/plot_energy_decrease")
    out = {}
    for name, steps in (("m1", 40), ("m2", 20), ("opt", 20)):
        rows = np.loadtxt(os.path.join(d, f"{name}_stats.csv"))
        trials = rows.shape[0] // steps
        assert np.array_equal(rows[:, 0].reshape(trials, steps), np.repeat(np.arange(trials), steps).reshape(trials, steps))
        out[f"{name}_energy"] = rows[:, 2].astype(np.int32).reshape(trials, steps)
        out[f"{name}_time_s"] = rows[:, 1].reshape(trials, steps)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_stats_traces.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
