"""Benchmark: SB spin-updates/s on the batched dSB workload (and the other workloads on request).

Default workload (one GB300): complete graph N = 2000 with J_ij iid in {-1, +1}, R = 1024
replicas, 2000 SB steps, dSB with the field J*sign(x) on the tensor cores (packed E2M1 operands,
FP32 accumulation, bit-exact; FP8 E4M3 with --operand fp8), x and y in FP32. One bench "step" is
one full solve (init, 2000 SB steps, final energies, best spins back to the host).

  value  spin-updates/s = N * R * sb_steps / solve time, J resident in HBM (sb_plan_run), device
         time from CUDA events on the solver's stream; L2 is flushed (256 MB write) between solves
  e2e    the same metric through the public call a user makes: sb_problem_wrap of pinned host
         memory (its O(N^2) coupling scan decides the operand type and c0) and sb_solve (H2D of J,
         the solve, D2H of the results), all inside the timed region
  roofline  the persistent tensor-core kernel: algorithmic FLOPs (2 N^2 R per SB step) per launch
         over its event-timed launch duration, against the E2M1 rate (6 x the measured dense BF16
         burst, the nominal 13.5 / 2.25 ratio; 2 x for FP8), and as a fraction of the BF16 burst
  latency  a bounded serving run after the timed region: Poisson requests of the serving
         workload's distribution through sb_submit / sb_poll, p50 / p99 latency and served rate
  cpu_baseline  the multithreaded FP32 CPU port of the same step loop (oracle/sb_cpu_baseline.c)
         on this host's cores, on a bounded sample of the workload
  plain_same_instance_as_reference_gpu  after the timed region: the plain FP32 path (aSB, the
         reference's update, and dSB) on the instance the reference arm's reference_gpu_plain
         times the reference program on (2000 spins, 1 replica, 1000 SB steps)

Multi-GPU: the path shards by replicas / instances only; each rank runs its own solve (weak
scaling) and the value is the total over ranks divided by the slowest rank's time.
`--impl reference` times the CPU port of the reference step loop (the reference has no CPU
implementation of its own) on the same workload and prints its line; each bench step is a bounded
sample (its wall time is the line's ms_per_step, its SB steps config.sb_steps_timed). The line also
carries the reference SB program itself on the GPU (its kernels compiled from its sources by
oracle/build_ref.py, with cuBLAS SGEMV for the field, as m2_opt.cu runs them), untimed by the
line's value.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (variant, n, replicas, sb_steps, field, description)
    "batched-dsb": ("dsb", 2000, 1024, 2000, "tc",
                    "batched dSB: complete N=2000, J iid +-1, R=1024, 2000 steps, tensor-core field "
                    "(packed E2M1 operands; FP8 with --operand fp8)"),
    "plain-dsb": ("dsb", 2000, 1, 1000, "fp32",
                  "plain dSB: complete N=2000, J iid +-1, R=1, 1000 steps, fused FP32 kernel"),
    "batched-bsb": ("bsb", 8192, 256, 3000, "tc",
                    "batched bSB: complete N=8192, J ~ N(0,1/N), h ~ N(0,0.1), R=256, 3000 steps, "
                    "BF16 hi+lo tensor-core field"),
    "uneven-batch": ("dsb", 0, 64, 1500, "grouped",
                     "uneven batch: 512 instances, N ~ U[64,4096], Erdos-Renyi density ~ U[0.05,1], "
                     "J = +-1, R=64, 1500 steps, one grouped tensor-core launch per step"),
    "sqa": ("sqa", 4096, 304, 100, "sqa",
            "SQA: complete N=4096, J iid +-1, M=64 Trotter slices, 100 annealing steps (the sizes of "
            "SQA_fully/fully_test/pre_calculate.cu), 304 replicas (two per SM)"),
    "nmfa": ("nmfa", 1024, 1024, 100, "nmfa",
             "NMFA: N=1024 (the size of NMFA/CUDA_GPU/Ising.cpp), J drawn as NMFA/CUDA_GPU/tests/fully.py "
             "(edge probability 1/2, weight in {-1,0,+1}), 100 stages x 2 sweeps of its beta schedule, "
             "1024 samples"),
    "serving": ("dsb", 0, 32, 0, "serving",
                "serving stream: Poisson arrivals at 200/s, N log-uniform in [128,16384], density "
                "~ U[0.01,1], J ~ U{-8..8}, R=32, step budget ~ U[500,4000]"),
}


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu capture of
# each dominant kernel; the summaries, with the commands, are the files named here.
NCU_TRAFFIC = {
    # batched dSB, N=2000, R=1024, E2M1 kernel: bytes per launch, the same for 30 and 240 steps
    # (everything after the first step is L2-resident)
    "batched-dsb": (19.58e6, "profiles/tc_fp4_kernel_batched_dsb_n2000_r1024.md"),
    # plain dSB, N=2000, R=1: bytes per launch (ncu runs the launch with cold caches)
    "plain-dsb": (16.03e6, "profiles/plain_step_kernel_plain_dsb_n2000.md"),
    # the same in one cooperative launch per solve: DRAM read + write per launch from a one-pass
    # capture (J read once; 16.06 MB read, 15.9 KB written)
    "plain-dsb-persist": (16.07e6, "profiles/plain_persist_kernel_plain_dsb_n2000.md"),
    # batched bSB, N=8192, R=256, BF16 hi+lo with the field accumulated in K segments: bytes per SB
    # step (8-step capture of the step launch: 2.587 GB; 4 steps: 1.146 GB), times the launch's steps
    "batched-bsb": (2.587e9 / 8, "profiles/tc_sb_kernel_batched_bsb_n8192_r256.md"),
    # uneven batch: measured bytes per algorithmic byte on a 48-instance batch (441.2 MB of
    # 451.8 MB); the launch of the full batch is scaled by its algorithmic bytes
    "uneven-batch": (441.2 / 451.8, "profiles/grouped_kernel_uneven_batch_48_instances.md"),
    # the same with E2M1 couplings (255.2 MB of 284.0 MB)
    "uneven-batch-e2m1": (255.2 / 284.0, "profiles/grouped_kernel_uneven_batch_48_instances.md"),
    # the same with packed E2M3 couplings (349.6 MB of 366.7 MB)
    "uneven-batch-e2m3": (349.6 / 366.75, "profiles/grouped_kernel_uneven_batch_48_instances.md"),
}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def reduce_max(value: float, world: int) -> float:
    """Max of a per-rank number over all ranks (NCCL on CUDA tensors, gloo on CPU tensors)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_scaling_value(units_per_rank: float, world: int, steps: int, max_total_ms: float) -> float:
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return world * units_per_rank * steps / (max_total_ms * 1e-3)


# bytes of one grouped operand row (couplings as stored on the device) and of one sign per spin and
# replica, by operand type: FP8 E4M3 [Np][Np]; packed E2M3, 3/4 byte per value [Np][3 Np / 4];
# packed E2M1 pairs [Np][Kp / 2] with Kp = N rounded up to 256
SIGN_BYTES = {"fp8e4m3": 1.0, "fp6e2m3": 0.75, "fp4e2m1": 0.5}


def operand_row_bytes(n, dtype):
    np_ = (n + 127) // 128 * 128
    if dtype == "fp4e2m1":
        return (n + 255) // 256 * 128
    return np_ * 3 // 4 if dtype == "fp6e2m3" else np_


def make_problem(name):
    from annealing_gb300 import instances

    variant, n, R, steps, field, desc = WORKLOADS[name]
    if variant == "bsb":
        J, h = instances.gaussian(n, seed=1234)
    else:
        J, h = instances.complete_pm1(n, seed=1234), None
    return J, h


def cpu_sample(name, J, h, budget_s=12.0, threads=None, max_steps=None):
    """Time the CPU port on a bounded sample: all replicas, as many SB steps as fit ~budget_s."""
    from oracle import binding as orc

    variant, n, R, steps, field, desc = WORKLOADS[name]
    vcode = {"asb": 0, "bsb": 1, "dsb": 2}[variant]
    c0 = orc.default_c0(J)
    x, y = orc.init_uniform(n, R, 1234)
    t0 = time.perf_counter()
    nthreads = orc.cpu_run(vcode, J, h, x, y, 1, 1.0, c0, 1.25, threads=threads)
    t1 = time.perf_counter() - t0
    k = max(1, int(budget_s / max(t1, 1e-6)))
    k = min(k, steps if max_steps is None else max_steps)
    t0 = time.perf_counter()
    orc.cpu_run(vcode, J, h, x, y, k, 1.0, c0, 1.25, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n * R * k / dt, "unit": "spin-updates/s", "cores": nthreads, "kind": "port",
            "sample": f"{k} SB steps x {R} replicas of the workload (N={n}), FP32, {nthreads} threads",
            "seconds": dt, "steps": k}


def reference_gpu_plain(sb_steps=1000):
    """The reference SB program on this GPU, as the plain method: m2_opt.cu's kernels (compiled from
    its sources into oracle/_ref/m2_opt.cubin by oracle/build_ref.py) and cuBLAS SGEMV, driven as its
    main loop does (m2_opt.cu:152-187) on the default instance (2000 spins, padded to its N = 2048,
    one trial = one replica). Returns None when the cubin was not built (no reference checkout)."""
    from annealing_gb300 import instances
    from oracle import ref_gpu

    if not os.path.exists(ref_gpu.M2OPT_CUBIN):
        return None
    spins, N = 2000, 2048
    Jh = np.zeros((N, N), np.float32)
    Jh[:spins, :spins] = instances.complete_pm1(spins, seed=1234)
    ref = ref_gpu.M2opt(Jh)
    try:
        prog_ms, dev_ms = ref.time_steps(sb_steps)
    finally:
        ref.close()
    return {"instance": f"complete +-1 graph, {spins} spins (the program's N = {N}, zero padding), 1 replica, "
                        f"{sb_steps} SB steps (aSB, the reference's update)",
            "ms_per_sb_step_as_program": prog_ms, "ms_per_sb_step_device_only": dev_ms,
            "spin_updates_per_s_as_program": spins / (prog_ms * 1e-3),
            "spin_updates_per_s_device_only": spins / (dev_ms * 1e-3),
            "divergence": "on this instance the aSB update overflows x to NaN after ~300 steps (as the CPU "
                          "restatement of it does): a timing figure",
            "note": "as_program: an event pair and an event synchronize around every step, as m2_opt.cu:159-185 "
                    "(host wall time); device_only: the same launches back to back under one event pair"}


def run_reference(args, rank, world):
    """The CPU port of the reference step loop, timed per bench step on a bounded sample."""
    if rank != 0:
        return
    if args.workload == "sqa":
        return run_reference_sqa(args, world)
    if args.workload == "nmfa":
        return run_reference_nmfa(args, world)
    J, h = make_problem(args.workload)
    variant, n, R, steps, field, desc = WORKLOADS[args.workload]
    budget = args.cpu_budget or max(1.0, min(12.0, 40.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample(args.workload, J, h, budget_s=budget / 4)
    samples = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        samples.append(cpu_sample(args.workload, J, h, budget_s=budget))
    wall = time.perf_counter() - t0
    value = float(sum(n * R * s["steps"] for s in samples) / sum(s["seconds"] for s in samples))
    line = {
        "impl": "reference", "metric": "SB spin-updates/s", "value": value, "unit": "spin-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        # the wall time of one timed bench step: one bounded sample of the workload
        "ms_per_step": 1e3 * sum(s["seconds"] for s in samples) / len(samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": desc, "n": n, "replicas": R, "sb_steps": steps, "variant": variant,
                   "field": "f32", "parallelism": f"replicas-only x{world}",
                   "l2": "host CPU (no device caches)",
                   "sb_steps_timed": int(statistics.median(s["steps"] for s in samples))},
        "cpu_baseline": {"value": value, "unit": "spin-updates/s", "cores": samples[0]["cores"],
                         "kind": "port", "sample": samples[0]["sample"]},
        "e2e": {"value": value, "unit": "spin-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "timed_wall_s": wall,
        "note": "the reference ships no CPU implementation of the SB step loop; this is the C port "
                "of its loop (UpdateTwice + dense matrix-vector field, and the bSB/dSB update) with "
                "POSIX threads; each bench step is a bounded sample of the workload (all replicas, "
                "config.sb_steps_timed SB steps), value = the samples' spin-updates over their time",
    }
    if variant == "dsb" and not args.no_reference_gpu:
        try:
            line["reference_gpu_plain"] = reference_gpu_plain()
        except Exception as exc:  # the GPU leg is informational; the CPU line stands
            line["reference_gpu_plain"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)


def plain_fp32_comparison(sb, ctx, prob, plan, vcode, n, R, sb_steps, value, stream):
    """The plain FP32 fused kernel (one launch per SB step) on the same instance, replicas and steps:
    its spin-updates/s, the tensor-core path's ratio to it, and whether both return the same
    replica energies for the same seed (equal mean best energy: integer fields are exact on both)."""
    import torch

    prm_f = sb.Params.default(vcode, steps=sb_steps, replicas=R, field_mode=sb.FIELD_FP32, seed=4242)
    plan_f = ctx.plan(prob, prm_f)
    plan_f.run(seed=4242)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rf = plan_f.run(seed=4243)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    plan_f.close()
    rt = plan.run(seed=4243)
    plain = float(n) * R * sb_steps / (ms * 1e-3)
    return {"plain_fp32_value": plain, "unit": "spin-updates/s", "ratio": value / plain, "plain_ms_per_solve": ms,
            "replica_energies_identical": bool(np.array_equal(rf.replica_energies, rt.replica_energies)),
            "mean_best_energy": {"tensor_core": float(rt.best_energy), "plain_fp32": float(rf.best_energy)},
            "mean_replica_energy": {"tensor_core": float(np.mean(rt.replica_energies)),
                                    "plain_fp32": float(np.mean(rf.replica_energies))},
            "note": "same instance, replicas, SB steps and seed; one solve each"}


def plain_same_instance(sb, ctx, stream, sb_steps=1000, runs=7):
    """This library's plain FP32 path on the instance `reference_gpu_plain` times the reference
    program on (complete +-1 graph of 2000 spins, seed 1234, one replica, 1000 SB steps): aSB (the
    reference's update, its initial state) and dSB, each a whole solve from a plan (init, every
    step, final energies), CUDA events on the launching stream, the median of `runs` after one
    warm-up run."""
    import torch

    from annealing_gb300 import instances

    spins = 2000
    prob = sb.Problem.from_dense(instances.complete_pm1(spins, seed=1234))
    out = {"instance": f"complete +-1 graph, {spins} spins, 1 replica, {sb_steps} SB steps (as reference_gpu_plain)",
           "note": "a timing figure: on this instance aSB's x overflows to NaN after ~300 steps (the CPU "
                   "restatement of the reference's update does the same; its default is 100 steps)"}
    for name, vcode, init in (("asb", sb.ASB, sb.INIT_REFERENCE), ("dsb", sb.DSB, sb.INIT_UNIFORM)):
        prm = sb.Params.default(vcode, steps=sb_steps, replicas=1, field_mode=sb.FIELD_FP32, init_mode=init)
        plan = ctx.plan(prob, prm)
        try:
            plan.run(seed=1)
            ts = []
            for k in range(runs):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r = plan.run(seed=2 + k)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
        finally:
            plan.close()
        ms = float(np.median(ts))
        out[name] = {"ms_per_solve": ms, "ms_per_sb_step": ms / sb_steps,
                     "spin_updates_per_s": spins * sb_steps / (ms * 1e-3),
                     "sb_steps_per_launch": int(r.steps_per_launch), "kernel_launches": int(r.kernel_launches)}
    return out


def run_ours(args, rank, world, local_rank):
    import torch

    import annealing_gb300 as sb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    variant, n, R, sb_steps, field, desc = WORKLOADS[args.workload]
    vcode = {"asb": sb.ASB, "bsb": sb.BSB, "dsb": sb.DSB}[variant]
    fmode = sb.FIELD_TC if field == "tc" else sb.FIELD_FP32
    J, h = make_problem(args.workload)
    stream = torch.cuda.current_stream(dev)
    ctx = sb.Context(local_rank, stream=stream.cuda_stream)
    prob = sb.Problem.from_dense(J, h)
    odt = {"auto": sb.OPERAND_AUTO, "fp4": sb.OPERAND_FP4, "fp6": sb.OPERAND_FP6, "fp8": sb.OPERAND_FP8,
           "bf16": sb.OPERAND_BF16, "bf16x2": sb.OPERAND_BF16X2, "fp16x2": sb.OPERAND_FP16X2}[args.operand]
    prm = sb.Params.default(vcode, steps=sb_steps, replicas=R, field_mode=fmode, seed=1234 + rank, operand_dtype=odt)
    plan = ctx.plan(prob, prm)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # ---- value: J resident ----
    for k in range(args.warmup):
        plan.run(seed=1000 + k)
    barrier()
    times, launches, results = [], 0, []
    with ClockSampler(local_rank) as clk:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = plan.run(seed=2000 + k)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            launches += r.kernel_launches
            results.append(r)
        barrier()
        wall = time.perf_counter() - wall0
    total_ms = reduce_max(float(sum(times)), world)
    value = weak_scaling_value(float(n) * R * sb_steps, world, args.steps, total_ms)

    # ---- roofline of the dominant kernel: one profiled solve (event pair around each launch) ----
    prm_p = sb.Params.default(vcode, steps=sb_steps, replicas=R, field_mode=fmode, seed=77, profile=1,
                              operand_dtype=odt)
    plan_p = ctx.plan(prob, prm_p)
    plan_p.run()
    rp = plan_p.run(seed=78)
    plan_p.close()
    hbm, bf16, src = peaks()
    flops_per_launch = 2.0 * n * n * R * rp.steps_per_launch
    if field == "tc":
        fdt = results[0].field_dtype
        # FP8 and E2M1 peaks from the measured BF16 burst by the nominal dense ratios
        # (BF16 2.25, FP8 4.5, E2M1 13.5 PFLOP/s)
        scale, label = {"fp4e2m1": (6.0, "6 x {} dense BF16 burst (E2M1 rate, nominal 13.5 / 2.25)"),
                        "fp8e4m3": (2.0, "2 x {} dense BF16 burst (FP8 E4M3 rate)")}.get(fdt, (1.0, "{} dense BF16 burst"))
        tc_peak = scale * bf16
        achieved = flops_per_launch / (rp.kernel_ms_avg * 1e-3) / 1e12
        if fdt == "fp4e2m1" and n == 2000 and R == 1024:
            traffic = NCU_TRAFFIC["batched-dsb"]
        elif fdt in ("bf16x2", "fp16x2") and n == 8192 and R == 256:
            traffic = (NCU_TRAFFIC["batched-bsb"][0] * rp.steps_per_launch, NCU_TRAFFIC["batched-bsb"][1])
        else:
            traffic = (None, None)
        roof = {"bound": "tensor", "achieved": achieved, "peak": tc_peak, "unit": "TFLOP/s",
                "frac": achieved / tc_peak, "traffic": traffic[0], "traffic_source": traffic[1],
                "kernel": ("tc_fp4_kernel" if fdt == "fp4e2m1" else "tc_sb_kernel") + " (persistent, one launch per solve)",
                "launch_ms": rp.kernel_ms_avg, "sb_steps_per_launch": rp.steps_per_launch,
                "flops_per_launch": flops_per_launch, "peak_source": label.format(src),
                "frac_of_bf16_burst": achieved / bf16}
        if results[0].field_dtype in ("bf16x2", "fp16x2"):
            roof["note"] = "split operands run 3 products per field; achieved counts the algorithmic 2N^2R"
    else:
        # algorithmic bytes of one SB step (J, and x, y read and written) x the steps of a launch
        spl = max(1, rp.steps_per_launch)
        bytes_per_launch = (4.0 * n * n + 16.0 * n * R) * spl
        achieved = bytes_per_launch / (rp.kernel_ms_avg * 1e-3) / 1e9
        limiter = None
        if spl > 1:
            traffic = NCU_TRAFFIC.get("plain-dsb-persist", (None, None)) if n == 2000 and R == 1 else (None, None)
            kernel = "plain_persist_kernel (one cooperative launch per solve)"
            note = ("achieved counts the algorithmic 4 N^2 bytes of J per SB step, but J lives in registers for "
                    "the whole launch and is read from HBM once (traffic); the kernel is not HBM-bound, see "
                    "limiter")
            us = 1e3 * rp.kernel_ms_avg / spl
            limiter = {"kind": "latency of the per-step sign exchange through L2",
                       "us_per_sb_step": us,
                       "serial_l2_trips_per_step": 2,
                       "us_per_l2_trip": us / 2,
                       "exchange": "each CTA stores one tagged sign word on its own 128-byte line; thread q of "
                                   "every CTA polls CTA q's line until the tag of the step appears",
                       "hbm_bytes_per_launch": 4.0 * n * n + 16.0 * n * R,
                       "hbm_frac_of_launch": (4.0 * n * n + 16.0 * n * R) / (rp.kernel_ms_avg * 1e-3) / 1e9 / hbm}
        else:
            traffic = NCU_TRAFFIC["plain-dsb"] if n == 2000 and R == 1 else (None, None)
            kernel = "plain_step_kernel"
            note = "J (16 MB) is L2-resident between steps; the fraction is of HBM bandwidth"
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic[0],
                "traffic_source": traffic[1], "kernel": kernel, "launch_ms": rp.kernel_ms_avg,
                "sb_steps_per_launch": spl, "peak_source": f"{src} HBM copy", "note": note}
        if limiter:
            roof["limiter"] = limiter

    # ---- e2e: host buffers through the public calls: sb_problem_wrap (the coupling scan that
    # decides the operand type and c0) and sb_solve (H2D of J, the solve, D2H of the results) ----
    Jp = torch.from_numpy(J).pin_memory()
    hp = torch.from_numpy(h).pin_memory() if h is not None else None

    def wrap():
        return sb.Problem.wrap(n, Jp.data_ptr(), hp.data_ptr() if hp is not None else 0, keepalive=(Jp, hp))

    for k in range(max(1, args.warmup)):
        ctx.solve(wrap(), prm)
    barrier()
    e2e_ms = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r = ctx.solve(wrap(), prm)  # scan, H2D of J, solve, D2H of spins / energies; returns when done
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = reduce_max(float(sum(e2e_ms)), world)
    e2e_value = weak_scaling_value(float(n) * R * sb_steps, world, args.steps, e2e_total)
    h2d = J.nbytes + (h.nbytes if h is not None else 0)
    d2h = n + 8 * R + 4  # best spins (int8), replica energies (f64), status word

    if rank != 0:
        plan.close()
        ctx.close()
        return
    line = {
        "metric": "SB spin-updates/s", "value": value, "unit": "spin-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp4e2m1": "e2m1 x e2m1 field (f32 accumulate, exact for |J| <= 4), f32 state",
                  "fp8e4m3": "fp8e4m3 field (f32 accumulate), f32 state",
                  "bf16x2": "bf16 hi+lo field (f32 accumulate), f32 state",
                  "fp16x2": "fp16 hi+lo field, power-of-two scaled (f32 accumulate), f32 state",
                  "bf16": "bf16 field (f32 accumulate), f32 state",
                  "f32": "f32"}[results[0].field_dtype],
        "data": "synthetic (seeded; the reference's WK2000_1.rud is not shipped)",
        "config": {"workload": desc, "n": n, "replicas": R, "sb_steps": sb_steps,
                   "variant": variant, "field": results[0].field_dtype,
                   "parallelism": f"replicas-only x{world}",
                   "l2": "flushed between timed solves (256 MB write outside the timed events)",
                   "sb_steps_timed": sb_steps},
        "e2e": {"value": e2e_value, "unit": "spin-updates/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_total / args.steps,
                "includes": "sb_problem_wrap of pinned host J (coupling scan), sb_solve (H2D, solve, D2H)"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk.summary(),
        "quality": {"best_energy": min(r.best_energy for r in results),
                    "mean_best_energy": float(np.mean([r.best_energy for r in results])),
                    "mean_replica_energy": float(np.mean(results[0].replica_energies)),
                    "energy_check_ok": all(r.energy_check_ok for r in results)},
        "wall_s": wall,
    }
    if field == "tc" and variant == "dsb" and world == 1:
        line["vs_plain_fp32"] = plain_fp32_comparison(sb, ctx, prob, plan, vcode, n, R, sb_steps, value, stream)
    if args.workload == "batched-dsb" and world == 1:
        # the plain path next to the reference program's GPU timing (the reference arm's reference_gpu_plain)
        try:
            line["plain_same_instance_as_reference_gpu"] = plain_same_instance(sb, ctx, stream)
        except Exception as exc:  # a side figure: the line's own numbers stand without it
            line["plain_same_instance_as_reference_gpu"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_sample(args.workload, J, h).items()
                                if k in ("value", "unit", "cores", "kind", "sample")}
    plan.close()
    if args.workload == "batched-dsb" and world == 1 and not args.no_latency:
        # latency: a bounded run of the serving workload's request stream, after the timed region
        lat_ctx = sb.Context(local_rank)
        try:
            out = serve_stream(sb, lat_ctx, count=200, rate=200.0, pool_size=16, R=32, seed=4321,
                               device=local_rank, warmup=2)
            line["latency"] = {k: v for k, v in out.items() if not k.startswith("_")}
            line["latency"]["workload"] = ("serving stream, bounded: 200 Poisson requests at 200/s, N log-uniform "
                                           "in [128,16384], density ~ U[0.01,1], J ~ U{-8..8}, R=32, step budget "
                                           "~ U[500,4000]; couplings from a pool of 16 distinct instances")
        finally:
            lat_ctx.close()
    print(json.dumps(line), flush=True)
    ctx.close()


def batch_instances(seed_base=1234, count=512):
    """The uneven-batch instances (library generator, seeded 1234 + k)."""
    import annealing_gb300 as sb
    from annealing_gb300 import instances

    spec = instances.uneven_batch(count, seed=seed_base)
    return [sb.Problem.random(n, d, 1, 0, seed=s) for n, d, s in spec]


def run_batch(args, rank, world, local_rank):
    import torch

    import annealing_gb300 as sb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    variant, _, R, sb_steps, field, desc = WORKLOADS[args.workload]
    probs = batch_instances(count=args.instances)
    if args.instances != 512:
        desc = desc.replace("512 instances", f"{args.instances} instances")
    n_sum = sum(p.n for p in probs)
    stream = torch.cuda.current_stream(dev)
    ctx = sb.Context(local_rank, stream=stream.cuda_stream)
    odt = {"auto": sb.OPERAND_AUTO, "fp4": sb.OPERAND_FP4, "fp8": sb.OPERAND_FP8, "fp6": sb.OPERAND_FP6,
           "bf16": sb.OPERAND_BF16}[args.operand]
    prm = sb.Params.default(sb.DSB, steps=sb_steps, replicas=R, seed=1234 + 1000 * rank, field_mode=sb.FIELD_TC,
                            operand_dtype=odt)
    t0 = time.perf_counter()
    batch = ctx.batch(probs, prm)
    setup_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    for k in range(args.warmup):
        batch.run(seed=10 + k)
    barrier()
    times, launches, quality = [], 0, []
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = batch.run(seed=100 + k)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            launches += res[0].kernel_launches
            quality.append(all(r.energy_check_ok for r in res))
        barrier()
    total_ms = reduce_max(float(sum(times)), world)
    updates = float(n_sum) * R * sb_steps
    value = weak_scaling_value(updates, world, args.steps, total_ms)
    # roofline: one profiled run, event pair around every grouped step launch
    prm_p = sb.Params.default(sb.DSB, steps=24, replicas=R, seed=7, field_mode=sb.FIELD_TC, profile=1,
                              operand_dtype=odt)
    bp = ctx.batch(probs, prm_p)
    bp.run()
    rp = bp.run(seed=8)
    bp.close()
    hbm, bf16, src = peaks()
    dts = [r.field_dtype for r in rp]  # each instance's operand bucket
    fp4 = all(d == "fp4e2m1" for d in dts)
    np_kp = sum(operand_row_bytes(p.n, d) * ((p.n + 127) // 128 * 128) for p, d in zip(probs, dts))
    # J + per spin-replica: x, y read and written (16 B) and the next sign operand (1 B, 3/4 or 1/2)
    bytes_per_launch = np_kp + sum(p.n * R * (16.0 + SIGN_BYTES[d]) for p, d in zip(probs, dts))
    achieved = bytes_per_launch / (rp[0].kernel_ms_avg * 1e-3) / 1e9
    tkey = {"fp4e2m1": "uneven-batch-e2m1", "fp6e2m3": "uneven-batch-e2m3"}.get(dts[0], "uneven-batch") \
        if len(set(dts)) == 1 else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": NCU_TRAFFIC[tkey][0] * bytes_per_launch if tkey else None,
            "traffic_source": (NCU_TRAFFIC[tkey][1] + " (48-instance capture, scaled by algorithmic bytes)")
            if tkey else None,
            "kernel": "grouped_kernel (one launch per SB step)",
            "launch_ms": rp[0].kernel_ms_avg, "bytes_per_launch": bytes_per_launch,
            "peak_source": f"{src} HBM copy",
            # the timed solves replay the step launches from a CUDA graph: per SB step, their time
            # (init and final energies included) against the event-timed launch above bounds what a
            # multi-step persistent launch could save (launch gaps and step-boundary tails)
            "graph_ms_per_sb_step": total_ms / args.steps / sb_steps,
            "gap_frac_bound": 1.0 - rp[0].kernel_ms_avg / (total_ms / args.steps / sb_steps)}
    # e2e: from host couplings every step through the public calls: sb_problem_wrap of each
    # instance (its coupling scan), then the batch (upload, convert, run, results back)
    import ctypes

    def addr(ptr):
        return ctypes.cast(ptr, ctypes.c_void_p).value or 0

    from concurrent.futures import ThreadPoolExecutor

    host = [(p.n, addr(p.s.J), addr(p.s.h)) for p in probs]
    pool = ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4))  # the scans run in C, GIL released
    e2e_ms = []
    for k in range(args.steps):
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        wrapped = list(pool.map(lambda a: sb.Problem.wrap(a[0], a[1], a[2], keepalive=probs), host))
        ctx.batch(wrapped, prm).run(seed=200 + k)
        e2e_ms.append(1e3 * (time.perf_counter() - t1))
    pool.shutdown()
    e2e_total = reduce_max(float(sum(e2e_ms)), world)
    if rank != 0:
        return
    line = {
        "metric": "SB spin-updates/s", "value": value, "unit": "spin-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("e2m1 x e2m1 field (f32 accumulate, exact for |J| <= 4), f32 state" if fp4
                  else "/".join(sorted(set(dts))) + " field (f32 accumulate, exact), f32 state"),
        "data": "synthetic (seeded)",
        "config": {"workload": desc, "instances": len(probs), "sum_n": n_sum, "replicas": R,
                   "sb_steps": sb_steps, "parallelism": f"replicas-only x{world}",
                   "l2": f"inputs ({np_kp / 1e9:.2f} GB of {'/'.join(sorted(set(dts)))} J) "
                   + ("larger than L2" if np_kp > 129e6 else "smaller than L2") + "; 256 MB flush between runs"},
        "e2e": {"value": world * updates * args.steps / (e2e_total * 1e-3), "unit": "spin-updates/s",
                "h2d_bytes_per_step": int(np_kp),  # couplings packed on the host, then copied
                "d2h_bytes_per_step": int(sum(p.n + 8 * R for p in probs)),
                "ms_per_step": e2e_total / args.steps,
                "includes": "sb_problem_wrap of every instance's host couplings (coupling scans, 16 at a "
                            "time), batch creation (packing, upload), the run, results back"},
        "gpu_launches": int(launches), "roofline": roof, "clocks": clk.summary(),
        "quality": {"energy_check_ok": all(quality)}, "setup_s": setup_s,
    }
    print(json.dumps(line), flush=True)


def serve_stream(sb, ctx, count, rate, pool_size, R, seed, device, warmup=2):
    """The serving workload's request stream through sb_submit / sb_poll: Poisson arrivals at
    `rate`, N log-uniform in [128, 16384], density U[0.01, 1], J ~ U{-8..8}, R replicas, step budget
    U[500, 4000]. A pool of distinct instances drawn from the same size distribution stands in for
    the couplings (each request takes the pool instance nearest its own N), which keeps host memory
    bounded. Latency = submit to result (the library's per-request total_ms). The stream's HBM
    fraction counts the algorithmic bytes the resident requests' steps read and write (FP8 couplings
    Np x Kp per step, x and y read and written and the next sign operand, 17 B per spin and replica)
    over the worker's busy time."""
    import threading as th

    from annealing_gb300 import instances

    stream = instances.serving_stream(count=count, rate=rate, seed=seed)
    rng = np.random.default_rng(99)
    pool_n = sorted(set(int(v) for v in np.exp(rng.uniform(np.log(128), np.log(16384), size=pool_size))))
    pool = [sb.Problem.random(n, float(rng.uniform(0.01, 1.0)), 8, 0, seed=5000 + i) for i, n in enumerate(pool_n)]
    pool_arr = np.array(pool_n)
    # warm-up: a few requests through the server (kernels, allocator)
    for k in range(warmup):
        p = pool[0]
        prm = sb.Params.default(sb.DSB, steps=100, replicas=R, seed=k, field_mode=sb.FIELD_TC)
        ctx.poll(ctx.submit(p, prm), p.n, prm, wait_ms=-1)
    stats0 = ctx.serving_stats()
    reqs = []
    for (arr, n, dens, steps, sd) in stream:
        i = int(np.argmin(np.abs(pool_arr - n)))
        reqs.append((arr, pool[i], sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=sd,
                                                     field_mode=sb.FIELD_TC)))
    tickets = [None] * len(reqs)
    t_start = time.perf_counter()

    def producer():
        for k, (arr, p, prm) in enumerate(reqs):
            now = time.perf_counter() - t_start
            if arr > now:
                time.sleep(arr - now)
            tickets[k] = ctx.submit(p, prm)

    with ClockSampler(device) as clk:
        pt = th.Thread(target=producer)
        pt.start()
        results = [None] * len(reqs)
        done_at = np.zeros(len(reqs))
        for k in range(len(reqs)):
            while tickets[k] is None:
                time.sleep(0.001)
            arr, p, prm = reqs[k]
            results[k] = ctx.poll(tickets[k], p.n, prm, wait_ms=-1)
            done_at[k] = time.perf_counter() - t_start
        pt.join()
        makespan = time.perf_counter() - t_start
    lat = np.array([r.total_ms for r in results])
    updates = float(sum(p.n * R * prm.steps for _, p, prm in reqs))
    stats = ctx.serving_stats()
    busy_ms = stats["busy_ms"] - stats0["busy_ms"]
    # per request and step: its couplings as stored (the grouped path's operand type), x and y read
    # and written, the next sign operand
    algo_bytes = 0.0
    for (_, p, prm), r in zip(reqs, results):
        d = r.field_dtype if r.field_dtype in SIGN_BYTES else "fp8e4m3"
        algo_bytes += (operand_row_bytes(p.n, d) * ((p.n + 127) // 128 * 128) + (16.0 + SIGN_BYTES[d]) * p.n * R) * prm.steps
    hbm, _, src = peaks()
    span = reqs[-1][0]
    # a queue that keeps up finishes the last request about one latency after its arrival; a
    # growing queue shows as latency rising along the stream
    half = len(reqs) // 2
    return {"requests": len(reqs), "offered_rate_per_s": rate, "arrival_span_s": span,
            "served_rate_per_s": len(reqs) / makespan, "makespan_s": makespan,
            "p50_ms": float(np.percentile(lat, 50)), "p90_ms": float(np.percentile(lat, 90)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "p50_ms_first_half": float(np.percentile(lat[:half], 50)),
            "p50_ms_second_half": float(np.percentile(lat[half:], 50)),
            "spin_updates_per_s": updates / makespan, "busy_ms": busy_ms,
            "admit_ms": stats["admit_ms"] - stats0["admit_ms"],
            "hbm_fraction": (algo_bytes / (busy_ms * 1e-3) / 1e9) / hbm if busy_ms > 0 else None,
            "hbm_bytes": algo_bytes, "peak_source": f"{src} HBM copy",
            "pool_instances": len(pool), "replicas": R,
            "energy_check_ok": all(r.energy_check_ok for r in results), "clocks": clk.summary(),
            "_updates": updates, "_results": results, "_reqs": reqs, "_stats": stats}


def run_serving(args, rank, world, local_rank):
    import torch

    import annealing_gb300 as sb

    torch.cuda.set_device(local_rank)
    variant, _, R, _, field, desc = WORKLOADS[args.workload]
    ctx = sb.Context(local_rank)
    out = serve_stream(sb, ctx, count=args.requests, rate=args.rate, pool_size=args.pool, R=R, seed=1234 + rank,
                       device=local_rank, warmup=args.warmup)
    reqs, results, updates, stats = out.pop("_reqs"), out.pop("_results"), out.pop("_updates"), out.pop("_stats")
    makespan = out["makespan_s"]
    if rank != 0:
        ctx.close()
        return
    if args.rate != 200.0:
        desc = desc.replace("at 200/s", f"at {args.rate:g}/s")
    line = {
        "metric": "SB spin-updates/s (serving stream)", "value": updates / makespan,
        "unit": "spin-updates/s", "n_gpus": world, "steps": len(reqs), "warmup": args.warmup,
        "ms_per_step": 1e3 * makespan / len(reqs), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp6e2m3 field (J / 4 in six bits, f32 accumulate, exact), f32 state",
        "data": "synthetic (seeded Poisson stream; sizes from a pool of distinct instances)",
        "config": {"workload": desc, "requests": len(reqs), "rate_per_s": args.rate,
                   "pool_instances": out["pool_instances"], "replicas": R},
        "latency_ms": {"p50": out["p50_ms"], "p90": out["p90_ms"], "p99": out["p99_ms"], "max": out["max_ms"]},
        "latency": {k: v for k, v in out.items() if k != "clocks"},
        "makespan_s": makespan, "arrival_span_s": out["arrival_span_s"],
        "requests_per_s": len(reqs) / makespan, "serving": stats,
        "quality": {"energy_check_ok": out["energy_check_ok"]},
        "clocks": out["clocks"],
        "e2e": {"value": updates / makespan, "unit": "spin-updates/s",
                # couplings packed to FP8 on the host before the copy
                "h2d_bytes_per_step": int(np.mean([((p.n + 127) // 128 * 128) ** 2 for _, p, _ in reqs])),
                "d2h_bytes_per_step": int(np.mean([p.n + 8 * R for _, p, _ in reqs]))},
    }
    print(json.dumps(line), flush=True)
    ctx.close()


SQA_TROTTER = 64


def sqa_cpu_sample(J, M, budget_s=10.0):
    """The SQA oracle (single-threaded C restatement of pre_calculate.cu) on whole annealing steps
    of one replica, as many as fit ~budget_s (at least one)."""
    from oracle import binding as orc

    n = J.shape[0]
    s, _ = orc.sqa_init(n, M, 1, 1, 1234)
    b, jp = orc.sqa_schedule(100, M)
    k, t0 = 0, time.perf_counter()
    while True:
        orc.sqa_run(J, s, 1, 1, seed=1234, beta=b[k % 100:k % 100 + 1], jperp=jp[k % 100:k % 100 + 1])
        k += 1
        if time.perf_counter() - t0 >= budget_s or k >= 100:
            break
    dt = time.perf_counter() - t0
    return {"value": M * (n + M - 1) * k / dt, "unit": "spin-updates/s", "cores": 1, "kind": "port",
            "sample": f"{k} annealing steps x 1 replica (N={n}, M={M}), single thread", "seconds": dt}


def run_reference_sqa(args, world):
    from annealing_gb300 import instances

    _, n, R, steps, _, desc = WORKLOADS["sqa"]
    J = instances.complete_pm1(n, seed=1234)
    budget = args.cpu_budget or max(2.0, min(10.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        sqa_cpu_sample(J, SQA_TROTTER, budget_s=budget / 4)
    samples = [sqa_cpu_sample(J, SQA_TROTTER, budget_s=budget) for _ in range(args.steps)]
    value = float(statistics.median(s["value"] for s in samples))
    line = {
        "impl": "reference", "metric": "SQA spin-updates/s", "value": value, "unit": "spin-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(s["seconds"] for s in samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int",
        "data": "synthetic", "config": {"workload": desc, "n": n, "trotter": SQA_TROTTER, "replicas": R,
                                        "anneal_steps": steps, "rng": "hash", "parallelism": f"replicas-only x{world}",
                                        "l2": "host CPU (no device caches)"},
        "cpu_baseline": {"value": value, "unit": "spin-updates/s", "cores": 1, "kind": "port",
                         "sample": samples[0]["sample"]},
        "e2e": {"value": value, "unit": "spin-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the C restatement of pre_calculate.cu's wavefront (oracle/sqa_oracle.c), one thread; each "
                "bench step is a bounded sample (whole annealing steps of one replica)",
    }
    print(json.dumps(line), flush=True)


def run_sqa(args, rank, world, local_rank):
    import torch

    import annealing_gb300 as sb
    from annealing_gb300 import instances

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    _, n, R, steps, _, desc = WORKLOADS["sqa"]
    M = SQA_TROTTER
    J = instances.complete_pm1(n, seed=1234)
    prob = sb.Problem.from_dense(J)
    stream = torch.cuda.current_stream(dev)
    ctx = sb.Context(local_rank, stream=stream.cuda_stream)
    prm = sb.SqaParams.default(trotter=M, steps=steps, replicas=R, seed=1234 + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    for k in range(args.warmup):
        ctx.sqa_solve(prob, prm)
    barrier()
    dev_ms, tot_ms, results = [], [], []
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize(dev)
            prm.seed = 5000 + k
            t0 = time.perf_counter()
            r = ctx.sqa_solve(prob, prm)  # H2D of J, anneal, D2H of energies and spins
            tot_ms.append(1e3 * (time.perf_counter() - t0))
            dev_ms.append(r.device_ms)
            results.append(r)
        barrier()
    updates = float(R) * M * (n + M - 1) * steps
    total_dev = reduce_max(float(sum(dev_ms)), world)
    total_e2e = reduce_max(float(sum(tot_ms)), world)
    value = weak_scaling_value(updates, world, args.steps, total_dev)
    e2e = weak_scaling_value(updates, world, args.steps, total_e2e)
    if rank != 0:
        ctx.close()
        return
    # couplings evaluated per second: every update's field covers N couplings of one row
    coupling_evals = updates * n / (total_dev / args.steps * 1e-3)
    line = {
        "metric": "SQA spin-updates/s", "value": value, "unit": "spin-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int (bit-plane couplings, popcount fields), f32 acceptance test",
        "data": "synthetic (seeded +-1 complete graph)",
        "config": {"workload": desc, "n": n, "trotter": M, "replicas": R, "anneal_steps": steps,
                   "rng": "hash", "parallelism": f"replicas-only x{world}",
                   "l2": "flushed between timed solves (256 MB write outside the timed region)"},
        "e2e": {"value": e2e, "unit": "spin-updates/s", "h2d_bytes_per_step": int(J.nbytes),
                "d2h_bytes_per_step": int(R * 8 + n)},
        "gpu_launches": int(sum(r.kernel_launches for r in results)),
        "throughput": {"coupling_evals_per_s": coupling_evals,
                       "note": "each Metropolis update evaluates its spin's N couplings against its slice"},
        "clocks": clk.summary(),
        "quality": {"best_energy": min(r.best_energy for r in results),
                    "energy_check_ok": all(r.energy_check_ok for r in results)},
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = sqa_cpu_sample(J, M)
    print(json.dumps(line), flush=True)
    ctx.close()


def nmfa_cpu_sample(J, budget_s=10.0):
    """The NMFA oracle (single-threaded C restatement of gpu_nmfa_kernel with the library's sweep
    semantics) on whole anneals of one sample, as many as fit ~budget_s (at least one)."""
    from oracle import binding as orc

    n = J.shape[0]
    betas = orc.nmfa_schedule(100)
    k, t0 = 0, time.perf_counter()
    while True:
        orc.nmfa_run(J, 1, betas, 0.15, 0.15, 1234 + k)
        k += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": n * 2 * 100 * k / dt, "unit": "spin-updates/s", "cores": 1, "kind": "port",
            "sample": f"{k} anneals (100 stages x 2 sweeps) x 1 sample (N={n}), single thread", "seconds": dt}


def run_reference_nmfa(args, world):
    from annealing_gb300 import instances

    _, n, R, stages, _, desc = WORKLOADS["nmfa"]
    J = instances.nmfa_fully(n, seed=1234)
    budget = args.cpu_budget or max(2.0, min(10.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        nmfa_cpu_sample(J, budget_s=budget / 4)
    samples = [nmfa_cpu_sample(J, budget_s=budget) for _ in range(args.steps)]
    value = float(statistics.median(s["value"] for s in samples))
    line = {
        "impl": "reference", "metric": "NMFA spin-updates/s", "value": value, "unit": "spin-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(s["seconds"] for s in samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": desc, "n": n, "samples": R, "stages": stages,
                                        "sweeps_per_stage": 2, "parallelism": f"samples-only x{world}",
                                        "l2": "host CPU (no device caches)"},
        "cpu_baseline": {"value": value, "unit": "spin-updates/s", "cores": 1, "kind": "port",
                         "sample": samples[0]["sample"]},
        "e2e": {"value": value, "unit": "spin-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the C restatement of NMFA/CUDA_GPU/src/nmfa.cu (oracle/nmfa_oracle.c), one thread; each "
                "bench step is a bounded sample (whole anneals of one sample)",
    }
    if not args.no_reference_gpu:
        try:
            line["reference_gpu_kernel"] = reference_gpu_nmfa(J, R, stages)
        except Exception as exc:  # the GPU leg is informational; the CPU line stands
            line["reference_gpu_kernel"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)


def reference_gpu_nmfa(J, samples, stages):
    """The reference NMFA kernel on this GPU (gpu_nmfa_kernel of NMFA/CUDA_GPU/src/nmfa.cu, compiled
    from its sources into oracle/_ref/nmfa_states_n{N}.cubin by oracle/build_ref.py), launched as
    gpu_nmfa does on the workload's instance and schedule: event time of the one launch, best of 3.
    Returns None when the cubin was not built."""
    from oracle import ref_gpu

    n = J.shape[0]
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", f"nmfa_states_n{n}.cubin")):
        return None
    k = ref_gpu.NmfaKernel(n)
    betas = ref_gpu.nmfa_schedule(stages)
    try:
        k.run(J, betas, 8)  # warm-up
        ms = min(k.run(J, betas, samples, timed=True)[1] for _ in range(3))
    finally:
        k.close()
    return {"samples": samples, "stages": stages, "ms_per_anneal": ms,
            "spin_updates_per_s": float(n) * samples * 2 * stages / (ms * 1e-3),
            "note": "one launch anneals every sample (one CTA of N threads each); event-timed, best of 3"}


def run_nmfa(args, rank, world, local_rank):
    import torch

    import annealing_gb300 as sb
    from annealing_gb300 import instances

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    _, n, R, stages, _, desc = WORKLOADS["nmfa"]
    J = instances.nmfa_fully(n, seed=1234)
    prob = sb.Problem.from_dense(J)
    betas = sb.nmfa_schedule(stages)
    stream = torch.cuda.current_stream(dev)
    ctx = sb.Context(local_rank, stream=stream.cuda_stream)
    prm = sb.NmfaParams.default(samples=R, stages=stages, seed=1234 + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    for k in range(args.warmup):
        ctx.nmfa_solve(prob, prm)
        ctx.gpu_nmfa(J, betas, R, 0.15, 0.15, 1234 + k)
    barrier()
    dev_ms, tot_ms, results = [], [], []
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize(dev)
            prm.seed = 7000 + k
            results.append(ctx.nmfa_solve(prob, prm))
            dev_ms.append(results[-1].device_ms)
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            ctx.gpu_nmfa(J, betas, R, 0.15, 0.15, 9000 + k)  # H2D of J, anneal, D2H of the samples
            tot_ms.append(1e3 * (time.perf_counter() - t0))
        barrier()
    updates = float(n) * R * 2 * stages
    total_dev = reduce_max(float(sum(dev_ms)), world)
    total_e2e = reduce_max(float(sum(tot_ms)), world)
    value = weak_scaling_value(updates, world, args.steps, total_dev)
    e2e = weak_scaling_value(updates, world, args.steps, total_e2e)
    if rank != 0:
        ctx.close()
        return
    flops = 2.0 * n * n * R * 2 * stages / (total_dev / args.steps * 1e-3)
    tc = results[-1].field_mode_used == sb.FIELD_TC
    _, bf16_peak, peak_kind = peaks()
    line = {
        "metric": "NMFA spin-updates/s", "value": value, "unit": "spin-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("bf16 hi+lo states x bf16 couplings on tensor cores (f32 accumulate), f32 states" if tc
                  else "f32 (field, mean-field states)"),
        "data": "synthetic (seeded graph)",
        "config": {"workload": desc, "n": n, "samples": R, "stages": stages, "sweeps_per_stage": 2,
                   "parallelism": f"samples-only x{world}",
                   "l2": "flushed between timed solves (256 MB write outside the timed region)"},
        "e2e": {"value": e2e, "unit": "spin-updates/s", "h2d_bytes_per_step": int(J.nbytes + betas.nbytes),
                "d2h_bytes_per_step": int(R * n * 4), "entry_point": "sb_gpu_nmfa (the reference's gpu_nmfa)"},
        "gpu_launches": int(sum(r.kernel_launches for r in results)),
        "throughput": {"field_flops_per_s": flops,
                       "note": ("tensor-core field, 2 N^2 FLOPs per sample and sweep (the hi+lo operand runs "
                                "twice that on the tensor pipe); all sweeps in one persistent launch" if tc else
                                "FP32 CUDA-core field, 2 N^2 FLOPs per sample and sweep; one fused launch per sweep")},
        "clocks": clk.summary(),
        "quality": {"best_energy": min(r.best_energy for r in results),
                    "mean_energy": float(np.mean([r.energies.mean() for r in results])),
                    "energy_check_ok": all(r.energy_check_ok for r in results)},
    }
    if tc:
        pipe = 2 * flops / 1e12  # two products (hi, lo) per coupling and sample on the tensor pipe
        line["roofline"] = {"bound": "tensor", "achieved": pipe, "peak": bf16_peak, "unit": "TFLOP/s",
                            "frac": pipe / bf16_peak, "traffic": None,
                            "kernel": "tc_sb_kernel<BF16, NMFA> (persistent, all 200 sweeps)",
                            "timing": "solve device time (seeding, operand, persistent launch, samples, energies)",
                            "peak_source": f"{peak_kind} dense BF16 burst"}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = nmfa_cpu_sample(J)
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed bench steps (one step = one solve); default per workload, about half a "
                         "second to a few seconds of timed work (40 solves of the default workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="batched-dsb")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip the reference program's GPU timing")
    ap.add_argument("--no-latency", action="store_true",
                    help="default workload: skip the bounded serving run that reports latency")
    ap.add_argument("--rate", type=float, default=200.0, help="serving workload: offered requests per second")
    ap.add_argument("--requests", type=int, default=2000, help="serving workload: stream length")
    ap.add_argument("--cpu-budget", type=float, default=0.0,
                    help="seconds of CPU work per reference-arm step (default: fit the run in ~1 min)")
    ap.add_argument("--pool", type=int, default=64, help="serving workload: distinct instances")
    ap.add_argument("--sb-steps", type=int, default=0,
                    help="smaller case for profiling: SB steps per solve (default: the workload's)")
    ap.add_argument("--operand", choices=["auto", "fp4", "fp6", "fp8", "bf16", "bf16x2", "fp16x2"], default="auto",
                    help="tensor-core operand type of the single-instance workloads (default: narrowest exact)")
    ap.add_argument("--instances", type=int, default=512,
                    help="uneven-batch workload: instance count (smaller cases for profiling)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"batched-dsb": 40, "plain-dsb": 40, "batched-bsb": 10, "uneven-batch": 5, "serving": 1,
                      "sqa": 5, "nmfa": 50}[args.workload] if args.impl == "ours" else 5
    if args.sb_steps > 0 and args.workload != "serving":
        v, n, R, _, field, desc = WORKLOADS[args.workload]
        WORKLOADS[args.workload] = (v, n, R, args.sb_steps, field,
                                    desc.replace(f"{_} steps", f"{args.sb_steps} steps"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "uneven-batch":
        run_batch(args, rank, world, local_rank)
    elif args.workload == "serving":
        run_serving(args, rank, world, local_rank)
    elif args.workload == "sqa":
        run_sqa(args, rank, world, local_rank)
    elif args.workload == "nmfa":
        run_nmfa(args, rank, world, local_rank)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
