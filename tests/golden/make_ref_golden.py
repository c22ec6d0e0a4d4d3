"""Generate golden SB trajectories by running the reference's own kernels on a GPU.

Loads oracle/_ref/m2_opt.cubin (prepare_points and UpdateTwice compiled from the reference's
SB/CUDA_GPU/m2_opt.cu by oracle/build_ref.py) through the CUDA driver API (oracle/ref_gpu.py) and drives it exactly as
m2_opt.cu:main does (m2_opt.cu:130-187): per-spin xorshift seeds initRand[i] = i, for each trial
prepare_points<<<N/64, 64>>>, then per step amplitude = s/(float)STEP, UpdateTwice<<<N/64, 64>>>
and cublasSgemv(OP_N, N, N, coeff1 = DeltaT*xi, J, N, x, 1, 1, y, 1). Records x, y after the
initialisation and after every step. The instance is a seeded +-1 complete graph on n_spins spins
stored in the first rows/columns of the N x N matrix, as the reference stores a file with fewer
spins than its compile-time N.

Usage (on a machine with a GB300):  python tests/golden/make_ref_golden.py <out_dir>
Writes ref_m2opt_n{N}.npz per case into out_dir.
"""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402
from oracle.ref_gpu import DELTA_T, XI, M2opt  # noqa: E402


def run_case(N, n_spins, trials, steps, seed):
    Jh = np.zeros((N, N), np.float32)
    Jh[:n_spins, :n_spins] = instances.complete_pm1(n_spins, seed=seed)
    ref = M2opt(Jh)
    x0 = np.zeros((trials, N), np.float32)
    y0 = np.zeros((trials, N), np.float32)
    xs = np.zeros((trials, steps, N), np.float32)
    ys = np.zeros((trials, steps, N), np.float32)
    for t in range(trials):
        ref.prepare()
        torch.cuda.synchronize()
        x0[t], y0[t] = ref.x.cpu().numpy(), ref.y.cpu().numpy()
        for s in range(steps):
            ref.step(s, steps)
            torch.cuda.synchronize()
            xs[t, s], ys[t, s] = ref.x.cpu().numpy(), ref.y.cpu().numpy()
    ref.close()
    return dict(N=N, n_spins=n_spins, seed=seed, steps=steps, x0=x0, y0=y0, xs=xs, ys=ys,
                coeff1=np.float32(DELTA_T * XI))


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    for N, n_spins, trials, steps in ((256, 250, 3, 20), (2048, 2000, 1, 20)):
        d = run_case(N, n_spins, trials, steps, seed=1234)
        path = os.path.join(out_dir, f"ref_m2opt_n{N}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <out_dir>")
    main(sys.argv[1])
