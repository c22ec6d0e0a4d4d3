"""Generate golden SB trajectories by running the reference's own kernels on a GPU.

Loads oracle/_ref/m2_opt.cubin (prepare_points and UpdateTwice compiled from the reference's
SB/CUDA_GPU/m2_opt.cu by oracle/build_ref.py) through the CUDA driver API and drives it exactly as
m2_opt.cu:main does (m2_opt.cu:130-187): per-spin xorshift seeds initRand[i] = i, for each trial
prepare_points<<<N/64, 64>>>, then per step amplitude = s/(float)STEP, UpdateTwice<<<N/64, 64>>>
and cublasSgemv(OP_N, N, N, coeff1 = DeltaT*xi, J, N, x, 1, 1, y, 1). Records x, y after the
initialisation and after every step. The instance is a seeded +-1 complete graph on n_spins spins
stored in the first rows/columns of the N x N matrix, as the reference stores a file with fewer
spins than its compile-time N.

Usage (on a machine with a GB300):  python tests/golden/make_ref_golden.py <out_dir>
Writes ref_m2opt_n{N}.npz per case into out_dir.
"""
import ctypes as C
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402

CUBIN = os.path.join(ROOT, "oracle", "_ref", "m2_opt.cubin")
XI, DELTA_T = 0.01565, 1.0  # m2_opt.cu:18, :20


def _cublas():
    torch.mv(torch.ones(4, 4, device="cuda"), torch.ones(4, device="cuda"))
    torch.cuda.synchronize()
    for line in open("/proc/self/maps"):
        if "libcublas.so" in line and "Lt" not in line:
            return C.CDLL(line.split()[-1])
    for cand in ("libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so.13"):
        try:
            return C.CDLL(cand)
        except OSError:
            pass
    raise RuntimeError("libcublas not found")


def run_case(N, n_spins, trials, steps, seed):
    cu = C.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")
    assert cu.cuInit(0) == 0
    mod = C.c_void_p()
    rc = cu.cuModuleLoad(C.byref(mod), CUBIN.encode())
    if rc != 0:
        raise RuntimeError(f"cuModuleLoad failed: {rc}")
    f_prep, f_upd = C.c_void_p(), C.c_void_p()
    assert cu.cuModuleGetFunction(C.byref(f_prep), mod, b"_Z14prepare_pointsPfS_Pj") == 0
    assert cu.cuModuleGetFunction(C.byref(f_upd), mod, b"_Z11UpdateTwicePfS_f") == 0
    cb = _cublas()
    handle = C.c_void_p()
    assert cb.cublasCreate_v2(C.byref(handle)) == 0

    Jh = np.zeros((N, N), np.float32)
    Jh[:n_spins, :n_spins] = instances.complete_pm1(n_spins, seed=seed)
    J = torch.from_numpy(Jh).cuda()
    rand = torch.arange(N, dtype=torch.int32, device="cuda")
    x = torch.zeros(N, device="cuda")
    y = torch.zeros(N, device="cuda")
    coeff1 = C.c_float(np.float32(DELTA_T * XI))
    coeff2 = C.c_float(1.0)

    def launch(fn, args):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        rc = cu.cuLaunchKernel(fn, N // 64, 1, 1, 64, 1, 1, 0, None, arr, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel: {rc}")

    px, py, pr = C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(rand.data_ptr())
    x0 = np.zeros((trials, N), np.float32)
    y0 = np.zeros((trials, N), np.float32)
    xs = np.zeros((trials, steps, N), np.float32)
    ys = np.zeros((trials, steps, N), np.float32)
    for t in range(trials):
        launch(f_prep, [px, py, pr])
        torch.cuda.synchronize()
        x0[t], y0[t] = x.cpu().numpy(), y.cpu().numpy()
        for s in range(steps):
            amp = C.c_float(np.float32(s) / np.float32(steps))
            launch(f_upd, [px, py, amp])
            rc = cb.cublasSgemv_v2(handle, 0, N, N, C.byref(coeff1), C.c_void_p(J.data_ptr()), N,
                                   px, 1, C.byref(coeff2), py, 1)
            if rc != 0:
                raise RuntimeError(f"cublasSgemv: {rc}")
            torch.cuda.synchronize()
            xs[t, s], ys[t, s] = x.cpu().numpy(), y.cpu().numpy()
    cb.cublasDestroy_v2(handle)
    cu.cuModuleUnload(mod)
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
    main(sys.argv[1] if len(sys.argv) > 1 else "gpurun_out/golden")
