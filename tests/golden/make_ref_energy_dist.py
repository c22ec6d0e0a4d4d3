"""Final energies of 1000 trials of the reference's own SB program, for the two-sample test.

Loads oracle/_ref/m2_opt.cubin (prepare_points and UpdateTwice compiled from the reference's
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
import ctypes as C
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from annealing_gb300 import instances  # noqa: E402
from make_ref_golden import CUBIN, DELTA_T, XI, _cublas  # noqa: E402

N, SPINS, TRIALS, STEPS, SEED = 2048, 2000, 1000, 100, 4321


def main(out_dir):
    cu = C.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")
    assert cu.cuInit(0) == 0
    mod = C.c_void_p()
    if cu.cuModuleLoad(C.byref(mod), CUBIN.encode()) != 0:
        raise RuntimeError("cuModuleLoad failed")
    f_prep, f_upd = C.c_void_p(), C.c_void_p()
    assert cu.cuModuleGetFunction(C.byref(f_prep), mod, b"_Z14prepare_pointsPfS_Pj") == 0
    assert cu.cuModuleGetFunction(C.byref(f_upd), mod, b"_Z11UpdateTwicePfS_f") == 0
    cb = _cublas()
    handle = C.c_void_p()
    assert cb.cublasCreate_v2(C.byref(handle)) == 0
    Js = instances.complete_pm1(SPINS, seed=SEED)
    Jh = np.zeros((N, N), np.float32)
    Jh[:SPINS, :SPINS] = Js
    J = torch.from_numpy(Jh).cuda()
    Jd = torch.from_numpy(Js.astype(np.float64)).cuda()
    rand = torch.arange(N, dtype=torch.int32, device="cuda")
    x = torch.zeros(N, device="cuda")
    y = torch.zeros(N, device="cuda")
    coeff1, coeff2 = C.c_float(np.float32(DELTA_T * XI)), C.c_float(1.0)
    px, py, pr = C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(rand.data_ptr())

    def launch(fn, args):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        if cu.cuLaunchKernel(fn, N // 64, 1, 1, 64, 1, 1, 0, None, arr, None) != 0:
            raise RuntimeError("cuLaunchKernel failed")

    energies = np.zeros(TRIALS, np.int64)
    for t in range(TRIALS):
        launch(f_prep, [px, py, pr])
        for s in range(STEPS):
            launch(f_upd, [px, py, C.c_float(np.float32(s) / np.float32(STEPS))])
            if cb.cublasSgemv_v2(handle, 0, N, N, C.byref(coeff1), C.c_void_p(J.data_ptr()), N, px, 1,
                                 C.byref(coeff2), py, 1) != 0:
                raise RuntimeError("cublasSgemv failed")
        spins = torch.where(x[:SPINS] > 0, 1.0, -1.0).double()
        energies[t] = int(round(-0.5 * float(spins @ (Jd @ spins))))
    torch.cuda.synchronize()
    cb.cublasDestroy_v2(handle)
    cu.cuModuleUnload(mod)
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "ref_m2opt_energies_n2000.npz")
    np.savez_compressed(path, energies=energies, spins=SPINS, seed=SEED, steps=STEPS, trials=TRIALS)
    print("wrote", path, "mean", energies.mean(), "std", energies.std(), "best", energies.min())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "gpurun_out/golden")
