"""Time the reference's own NMFA kernel on a GPU, next to this library's NMFA path.

The reference (NMFA/CUDA_GPU/src/nmfa.cu) anneals every sample in one launch of gpu_nmfa_kernel, one
CTA of N threads per sample with its row of J in registers (:54-140, launched by gpu_nmfa :180). This
script loads oracle/_ref/nmfa_states_n1024.cubin (that kernel, template expanded for N = 1024 by
oracle/build_ref.py) and times that launch with CUDA events for several sample counts on a seeded
N = 1024 graph with the distribution of NMFA/CUDA_GPU/tests/fully.py and the 100-stage schedule of
Ising.cpp; then the same instance, schedule and sample counts through sb_nmfa_solve (device time)
with the FP32 field (seeding, 200 fused sweep launches, the energy pass) and the tensor-core field
(seeding, one persistent launch for all sweeps, the samples and the energy pass; 32 samples and
more). Rates count N x samples x 200 spin updates.

Usage (on a machine with a GB300):  python tests/golden/time_ref_nmfa.py
Prints one JSON line.
"""
import json
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import annealing_gb300 as sb  # noqa: E402
from annealing_gb300 import instances  # noqa: E402
from make_nmfa_golden import RefKernel, schedule  # noqa: E402

N, STAGES = 1024, 100
COUNTS = (1, 8, 152, 1024)


def main():
    J = instances.nmfa_fully(N, 1234)
    betas = schedule(STAGES)
    ref = RefKernel(N)
    ref.run(J, betas, 8)  # warm-up
    out = {"instance": f"N={N}, fully.py distribution (seed 1234), {STAGES} stages x 2 sweeps",
           "gpu": torch.cuda.get_device_name(0), "reference_kernel": {}, "ours": {}}
    for R in COUNTS:
        ms = min(ref.run(J, betas, R, timed=True)[1] for _ in range(3))
        out["reference_kernel"][str(R)] = {"ms": ms, "spin_updates_per_s": N * R * 2 * STAGES / (ms * 1e-3)}
    ctx = sb.Context(0)
    prob = sb.Problem.from_dense(J)
    for field, mode in (("fp32", sb.FIELD_FP32), ("tc", sb.FIELD_TC)):
        out["ours_" + field] = {}
        for R in COUNTS:
            if mode == sb.FIELD_TC and R < 32:
                continue
            p = sb.NmfaParams.default(samples=R, field_mode=mode)
            ctx.nmfa_solve(prob, p, betas=betas)
            ms = min(ctx.nmfa_solve(prob, p, betas=betas).device_ms for _ in range(3))
            out["ours_" + field][str(R)] = {"ms": ms, "spin_updates_per_s": N * R * 2 * STAGES / (ms * 1e-3)}
    ctx.close()
    # the library's default (SB_FIELD_AUTO): the tensor-core field from 32 samples on
    out["ours"] = {k: out["ours_tc"].get(k, v) for k, v in out["ours_fp32"].items()}
    out["speedup"] = {k: out["reference_kernel"][k]["ms"] / out["ours"][k]["ms"] for k in out["ours"]}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
