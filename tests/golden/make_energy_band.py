"""Summarise the reference's published per-step energies into a small fixture.

Reads SB/CUDA_GPU/plot_figure/plot_energy_decrease/{opt,m2,m1}_stats.csv from a checkout of the
reference (rows "trial cumulative_seconds energy", STEP rows per trial; written by print_energy,
SB/CUDA_GPU/m2_opt.cu:77-91) and writes ref_energy_band.json: per file the mean, standard
deviation and best of the final-step energies, and the per-step mean energy.
Usage: python tests/golden/make_energy_band.py <reference checkout root>
"""
import json
import os
import sys

import numpy as np


def summarise(path, steps):
    rows = np.loadtxt(path)
    e = rows[:, 2].reshape(-1, steps)
    fin = e[:, -1]
    return {"trials": int(e.shape[0]), "steps": steps, "mean": float(fin.mean()),
            "std": float(fin.std()), "best": float(fin.min()),
            "step_mean": [float(v) for v in e.mean(axis=0)],
            "first_row_energy": float(e[0, 0])}


def main(root):
    d = os.path.join(root, "SB/CUDA_GPU/plot_figure/plot_energy_decrease")
    out = {"source": "SB/CUDA_GPU/plot_figure/plot_energy_decrease/*_stats.csv",
           "opt": summarise(os.path.join(d, "opt_stats.csv"), 20),
           "m2": summarise(os.path.join(d, "m2_stats.csv"), 20),
           "m1": summarise(os.path.join(d, "m1_stats.csv"), 40)}
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_energy_band.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
