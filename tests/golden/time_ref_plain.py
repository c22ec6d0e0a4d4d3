"""Time the reference's own plain SB method on a GPU, next to this library's plain path.

The reference program m2_opt.cu runs, per SB step, UpdateTwice<<<N/64, 64>>> and cublasSgemv on the
default stream, with a CUDA event pair around the two and a cudaEventSynchronize (m2_opt.cu:156-185).
This script loads oracle/_ref/m2_opt.cubin (its kernels, compiled from its source by
oracle/build_ref.py), drives them with cuBLAS exactly so on an N = 2048 matrix holding the seeded
+-1 complete graph of 2000 spins (the reference's N is a multiple of 64; the padding couplings are
0), and reports two rates in spin-updates/s (2000 spins per step):
  * as_program: wall time of the loop as the program runs it (events and a sync every step);
  * device_only: the same launches enqueued back to back, one event pair around all steps.
Then it times this library's plain FP32 path on the same instance (aSB, the reference's update,
and dSB), one fused launch per step replayed from a CUDA graph (device time of sb_plan_run).

Usage (on a machine with a GB300):  python tests/golden/time_ref_plain.py [steps]
Prints one JSON line.
"""
import ctypes as C
import json
import os
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import annealing_gb300 as sb  # noqa: E402
from annealing_gb300 import instances  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_ref_golden import CUBIN, DELTA_T, XI, _cublas  # noqa: E402

N, SPINS = 2048, 2000


def time_reference(steps):
    cu = C.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")
    assert cu.cuInit(0) == 0
    mod = C.c_void_p()
    if cu.cuModuleLoad(C.byref(mod), CUBIN.encode()) != 0:
        raise RuntimeError("cuModuleLoad failed: build oracle/_ref/m2_opt.cubin with oracle/build_ref.py")
    f_prep, f_upd = C.c_void_p(), C.c_void_p()
    assert cu.cuModuleGetFunction(C.byref(f_prep), mod, b"_Z14prepare_pointsPfS_Pj") == 0
    assert cu.cuModuleGetFunction(C.byref(f_upd), mod, b"_Z11UpdateTwicePfS_f") == 0
    cb = _cublas()
    handle = C.c_void_p()
    assert cb.cublasCreate_v2(C.byref(handle)) == 0
    Jh = np.zeros((N, N), np.float32)
    Jh[:SPINS, :SPINS] = instances.complete_pm1(SPINS, seed=1234)
    J = torch.from_numpy(Jh).cuda()
    rand = torch.arange(N, dtype=torch.int32, device="cuda")
    x = torch.zeros(N, device="cuda")
    y = torch.zeros(N, device="cuda")
    coeff1, coeff2 = C.c_float(np.float32(DELTA_T * XI)), C.c_float(1.0)
    px, py, pr = C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(rand.data_ptr())

    def launch(fn, args):
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        if cu.cuLaunchKernel(fn, N // 64, 1, 1, 64, 1, 1, 0, None, arr, None) != 0:
            raise RuntimeError("cuLaunchKernel failed")

    def step(s):
        launch(f_upd, [px, py, C.c_float(np.float32(s) / np.float32(steps))])
        if cb.cublasSgemv_v2(handle, 0, N, N, C.byref(coeff1), C.c_void_p(J.data_ptr()), N, px, 1,
                             C.byref(coeff2), py, 1) != 0:
            raise RuntimeError("cublasSgemv failed")

    launch(f_prep, [px, py, pr])
    for s in range(20):  # warm-up
        step(s)
    torch.cuda.synchronize()
    # as the program runs it: an event pair and a synchronize around every step (m2_opt.cu:159-185)
    t0 = time.perf_counter()
    for s in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        step(s)
        b.record()
        b.synchronize()
        a.elapsed_time(b)
    as_program = time.perf_counter() - t0
    # device only: the same launches back to back
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for s in range(steps):
        step(s)
    b.record()
    b.synchronize()
    device_ms = a.elapsed_time(b)
    cb.cublasDestroy_v2(handle)
    cu.cuModuleUnload(mod)
    return as_program * 1e3 / steps, device_ms / steps


def time_ours(steps, variant):
    J = instances.complete_pm1(SPINS, seed=1234)
    ctx = sb.Context(0)
    prm = sb.Params.default(variant, steps=steps, replicas=1, field_mode=sb.FIELD_FP32)
    plan = ctx.plan(sb.Problem.from_dense(J), prm)
    plan.run(seed=1)
    best = min(plan.run(seed=2 + k).device_ms for k in range(3))
    plan.close()
    ctx.close()
    return best / steps


def main(steps=1000):
    ref_prog_ms, ref_dev_ms = time_reference(steps)
    ours_asb = time_ours(steps, sb.ASB)
    ours_dsb = time_ours(steps, sb.DSB)
    rate = lambda ms: SPINS / (ms * 1e-3)  # noqa: E731
    print(json.dumps({
        "instance": f"complete +-1 graph, {SPINS} spins (reference matrix N={N}), 1 replica, {steps} steps",
        "reference_m2opt_as_program": {"ms_per_step": ref_prog_ms, "spin_updates_per_s": rate(ref_prog_ms)},
        "reference_m2opt_device_only": {"ms_per_step": ref_dev_ms, "spin_updates_per_s": rate(ref_dev_ms)},
        "ours_plain_asb": {"ms_per_step": ours_asb, "spin_updates_per_s": rate(ours_asb)},
        "ours_plain_dsb": {"ms_per_step": ours_dsb, "spin_updates_per_s": rate(ours_dsb)},
        "gpu": torch.cuda.get_device_name(0),
    }))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1000)
