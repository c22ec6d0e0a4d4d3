"""Golden NMFA results from the reference's own kernel, run on a GB300 — TEST INFRASTRUCTURE.

Loads oracle/_ref/nmfa_states_n{N}.cubin through oracle/ref_gpu.py (gpu_nmfa_kernel of NMFA/CUDA_GPU/src/nmfa.cu, template
expanded for N by oracle/build_ref.py, its last store changed to write the final mean-field state
instead of its sign) and launches it the way gpu_nmfa does (nmfa.cu:161-184): one CTA of N threads
per sample, N floats of dynamic shared memory, the betas of NMFA/CUDA_GPU/Ising.cpp:37-43, noise =
recombination = 0.15 (Ising.cpp:11-12), seed 1234 (Ising.cpp:13). Instances: the seeded graphs of
annealing_gb300.instances.nmfa_fully (the distribution of NMFA/CUDA_GPU/tests/fully.py).

Writes into out_dir:
  ref_nmfa_n32.npz     N=32 (one warp: the reference's sweeps are then race-free), 256 samples:
                       the states after the first K stages of the 100-stage anneal, K in KS
  ref_nmfa_n128.npz    N=128, 1000 samples, 100 stages: each sample's energy
                       E = sum_{i<j} J_ij s_i s_j (NMFA's objective) and the first 16 final states
  ref_nmfa_n1024.npz   N=1024 (Ising.cpp's size), 1000 samples, 100 stages: energies, and the
                       kernel's event time for 1 and 1000 samples
Usage (on a machine with a GB300):  python tests/golden/make_nmfa_golden.py <out_dir>
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402
from oracle.ref_gpu import NmfaKernel as RefKernel  # noqa: E402
from oracle.ref_gpu import nmfa_schedule as schedule  # noqa: E402

KS = (1, 2, 5, 10, 20, 100)


def energies(J, states):
    s = np.where(states > 0, 1, -1).astype(np.int64)
    Ji = np.rint(J).astype(np.int64)
    return np.einsum("ri,ij,rj->r", s, Ji, s) // 2


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    full = schedule(100)
    # one warp
    n, seed = 32, 4242
    J = instances.nmfa_fully(n, seed)
    k = RefKernel(n)
    st = {f"states_k{K}": k.run(J, full[:K], 256) for K in KS}
    np.savez_compressed(os.path.join(out_dir, "ref_nmfa_n32.npz"), J=J.astype(np.int8), seed=seed, samples=256,
                        ks=np.array(KS), **st)
    # four warps
    n, seed = 128, 4343
    J = instances.nmfa_fully(n, seed)
    s128 = RefKernel(n).run(J, full, 1000)
    np.savez_compressed(os.path.join(out_dir, "ref_nmfa_n128.npz"), seed=seed, energies=energies(J, s128),
                        states16=s128[:16])
    # the reference program's size
    n, seed = 1024, 4444
    J = instances.nmfa_fully(n, seed)
    k = RefKernel(n)
    k.run(J, full, 1)  # warm-up
    _, ms1 = k.run(J, full, 1, timed=True)
    s1024, ms1000 = k.run(J, full, 1000, timed=True)
    np.savez_compressed(os.path.join(out_dir, "ref_nmfa_n1024.npz"), seed=seed, energies=energies(J, s1024),
                        kernel_ms_1=ms1, kernel_ms_1000=ms1000)
    print("n32 K=100 first states", st["states_k100"][0, :4])
    print("n128 mean E", energies(J=instances.nmfa_fully(128, 4343), states=s128).mean())
    print("n1024 mean E", energies(J, s1024).mean(), "kernel ms (1 sample)", ms1, "(1000 samples)", ms1000)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <out_dir>")
    main(sys.argv[1])
