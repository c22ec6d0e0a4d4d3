"""Generate golden SQA runs by executing the reference's own SQA kernels on a GPU.

Loads oracle/_ref/sqa_pre_calculate_n{N}_m{M}.cubin (preapare_spins, reduce<64> and update_spins
compiled from the reference's SQA_fully/fully_test/pre_calculate.cu by oracle/build_ref.py) through
the CUDA driver API and drives them as pre_calculate.cu:main does (:183-237): per-spin xorshift
states initRand[i] = i, per trial preapare_spins<<<N/64, 64>>>, then per annealing step p the
M + N - 1 wavefront iterations reduce<64><<<N/128, 64, M*64*4>>>(a, ...) and
update_spins<<<1, M>>>(a, ..., J_perp, beta, ...), with beta and J_perp from the schedule of
:206-225 (restated by the oracle, oracle_sqa_schedule, and stored with the run). Records the
initial slices, the per-spin random words and every slice after every step. The instances are
seeded graphs written into the reference's char coupling matrix.

Usage (on a machine with a GB300):  python tests/golden/make_sqa_golden.py <out_dir>
Writes ref_sqa_n{N}_m{M}.npz per case into out_dir.
"""
import ctypes as C
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from annealing_gb300 import instances  # noqa: E402
from oracle import binding as orc  # noqa: E402

THREADS = 64  # pre_calculate.cu:11

CASES = (
    # N, M, steps, trials, instance
    (256, 8, 10, 2, "complete_pm1"),
    (512, 16, 6, 2, "er_jmax3"),
)


def instance(kind, n, seed=1234):
    if kind == "complete_pm1":
        return instances.complete_pm1(n, seed=seed)
    return instances.erdos_renyi(n, 0.5, seed, jmax=3)


def run_case(N, M, steps, trials, kind):
    cu = C.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")
    assert cu.cuInit(0) == 0
    mod = C.c_void_p()
    path = os.path.join(ROOT, "oracle", "_ref", f"sqa_pre_calculate_n{N}_m{M}.cubin")
    rc = cu.cuModuleLoad(C.byref(mod), path.encode())
    if rc != 0:
        raise RuntimeError(f"cuModuleLoad({path}) failed: {rc}")
    f_prep, f_red, f_upd = C.c_void_p(), C.c_void_p(), C.c_void_p()
    assert cu.cuModuleGetFunction(C.byref(f_prep), mod, b"_Z14preapare_spinsPcPj") == 0
    assert cu.cuModuleGetFunction(C.byref(f_red), mod, b"_Z6reduceILj64EEviPcPiS0_") == 0
    assert cu.cuModuleGetFunction(C.byref(f_upd), mod, b"_Z12update_spinsiPcS_ffPjPi") == 0

    J = instance(kind, N)
    Jc = torch.from_numpy(J.astype(np.int8)).cuda()
    rand = torch.arange(N, dtype=torch.int32, device="cuda")
    s_buf = torch.zeros(N * M, dtype=torch.int8, device="cuda")
    out_buf = torch.zeros(M * (N // THREADS // 2), dtype=torch.int32, device="cuda")
    beta, jperp = orc.sqa_schedule(steps, M)

    def launch(fn, grid, block, shmem, args):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        rc = cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, shmem, None, arr, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel: {rc}")

    ps, pr = C.c_void_p(s_buf.data_ptr()), C.c_void_p(rand.data_ptr())
    pj, po = C.c_void_p(Jc.data_ptr()), C.c_void_p(out_buf.data_ptr())
    init = np.zeros((trials, N, M), np.int8)
    rnd = np.zeros((trials, N), np.uint32)
    spins = np.zeros((trials, steps, N, M), np.int8)
    energy = np.zeros((trials, steps), np.int64)
    for t in range(trials):
        launch(f_prep, N // THREADS, THREADS, 0, [ps, pr])
        torch.cuda.synchronize()
        init[t] = s_buf.cpu().numpy().reshape(N, M)
        rnd[t] = rand.cpu().numpy().view(np.uint32)
        for p in range(steps):
            jp, bt = C.c_float(float(jperp[p])), C.c_float(float(beta[p]))
            for a in range(M + N - 1):
                ai = C.c_int(a)
                launch(f_red, N // THREADS // 2, THREADS, M * THREADS * 4, [ai, ps, po, pj])
                launch(f_upd, 1, M, 0, [ai, ps, pj, jp, bt, pr, po])
            torch.cuda.synchronize()
            spins[t, p] = s_buf.cpu().numpy().reshape(N, M)
            s0 = spins[t, p][:, 0].astype(np.int64)
            energy[t, p] = -int(np.triu(np.outer(s0, s0) * J.astype(np.int64), 1).sum())
    cu.cuModuleUnload(mod)
    return dict(N=N, M=M, steps=steps, kind=kind, J=J.astype(np.int8), beta=beta, jperp=jperp, init=init,
                rnd=rnd, spins=spins, energy=energy)


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    for N, M, steps, trials, kind in CASES:
        d = run_case(N, M, steps, trials, kind)
        path = os.path.join(out_dir, f"ref_sqa_n{N}_m{M}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, "energies", d["energy"].tolist())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <out_dir>")
    main(sys.argv[1])
