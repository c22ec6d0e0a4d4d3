"""Golden NMFA results from the reference's own kernel, run on a GB300 — TEST INFRASTRUCTURE.

Loads oracle/_ref/nmfa_states_n{N}.cubin (gpu_nmfa_kernel of NMFA/CUDA_GPU/src/nmfa.cu, template
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
import ctypes as C
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402

KERNEL = b"_Z15gpu_nmfa_kernelPfPiS_iffj"
NOISE, RECOMB, SEED = 0.15, 0.15, 1234
KS = (1, 2, 5, 10, 20, 100)


def schedule(stages):
    """Ising.cpp:37-43 in FP32."""
    inc = np.float32((np.float32(8) - np.float32(1) / np.float32(16)) / np.float32(stages))
    b, out = np.float32(1) / np.float32(16), []
    for _ in range(stages):
        out.append(b)
        b = np.float32(b + inc)
    return np.array(out, np.float32)


class RefKernel:
    def __init__(self, n):
        self.cu = C.CDLL("libcuda.so.1")
        torch.zeros(1, device="cuda")
        assert self.cu.cuInit(0) == 0
        self.n = n
        self.mod = C.c_void_p()
        path = os.path.join(ROOT, "oracle", "_ref", f"nmfa_states_n{n}.cubin")
        if self.cu.cuModuleLoad(C.byref(self.mod), path.encode()) != 0:
            raise RuntimeError("cuModuleLoad failed: build " + path + " with oracle/build_ref.py")
        self.fn = C.c_void_p()
        assert self.cu.cuModuleGetFunction(C.byref(self.fn), self.mod, KERNEL) == 0

    def run(self, J, betas, samples, timed=False):
        """Final states [samples, n] (and the kernel's event time in ms)."""
        n = self.n
        dJ = torch.from_numpy(np.ascontiguousarray(J, np.float32)).cuda()
        db = torch.from_numpy(np.ascontiguousarray(betas, np.float32)).cuda()
        out = torch.zeros(samples * n, dtype=torch.int32, device="cuda")
        args = [C.c_void_p(dJ.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(db.data_ptr()),
                C.c_int(len(betas)), C.c_float(NOISE), C.c_float(RECOMB), C.c_uint32(SEED)]
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        if self.cu.cuLaunchKernel(self.fn, samples, 1, 1, n, 1, 1, n * 4, None, arr, None) != 0:
            raise RuntimeError("cuLaunchKernel failed")
        b.record()
        b.synchronize()
        states = out.cpu().numpy().view(np.float32).reshape(samples, n).copy()
        return (states, a.elapsed_time(b)) if timed else states


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
    main(sys.argv[1] if len(sys.argv) > 1 else "gpurun_out/golden")
