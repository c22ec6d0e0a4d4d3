"""Final energies of 1000 trials of the reference's own SB program, for the two-sample test.

Loads oracle/_ref/m2_opt.cubin through oracle/ref_gpu.py (prepare_points and UpdateTwice compiled from the reference's
SB/CUDA_GPU/m2_opt.cu by oracle/build_ref.py) and drives it with cuBLAS SGEMV exactly as
m2_opt.cu:main does for TIMES = 1000 trials of STEP = 100 steps (m2_opt.cu:152-203): per-spin
xorshift states initRand[i] = i that every trial continues, prepare_points, then per step
UpdateTwice with amplitude s / STEP and the SGEMV kick. The instance is the seeded +-1 complete
graph of 2000 spins in the first rows / columns of a 2048 x 2048 matrix (the reference's N must be
a multiple of 64; the padding couplings are 0). After each trial the energy
H = -sum_{i<j} J_ij s_i s_j of s = (x > 0 ? 1 : -1) over the 2000 spins is recorded: the value the
reference writes to output.txt (it stores -E, m2_opt.cu:192-210).

Usage (on a machine with a GB300):  python tests/golden/make_ref_energy_dist.py <out_dir>
Writes ref_m2opt_energies_n2000.npz into out_dir.
"""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402
from oracle.ref_gpu import M2opt  # noqa: E402

N, SPINS, TRIALS, STEPS, SEED = 2048, 2000, 1000, 100, 4321


def main(out_dir):
    Js = instances.complete_pm1(SPINS, seed=SEED)
    Jh = np.zeros((N, N), np.float32)
    Jh[:SPINS, :SPINS] = Js
    ref = M2opt(Jh)
    Jd = torch.from_numpy(Js.astype(np.float64)).cuda()
    energies = np.zeros(TRIALS, np.int64)
    for t in range(TRIALS):
        ref.prepare()
        for s in range(STEPS):
            ref.step(s, STEPS)
        spins = torch.where(ref.x[:SPINS] > 0, 1.0, -1.0).double()
        energies[t] = int(round(-0.5 * float(spins @ (Jd @ spins))))
    torch.cuda.synchronize()
    ref.close()
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "ref_m2opt_energies_n2000.npz")
    np.savez_compressed(path, energies=energies, spins=SPINS, seed=SEED, steps=STEPS, trials=TRIALS)
    print("wrote", path, "mean", energies.mean(), "std", energies.std(), "best", energies.min())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <out_dir>")
    main(sys.argv[1])
