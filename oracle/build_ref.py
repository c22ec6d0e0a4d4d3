"""Build the reference's own SB and SQA kernels for the oracle pin — TEST INFRASTRUCTURE ONLY.

Compiles the device code of SB/CUDA_GPU/m2_opt.cu (prepare_points, UpdateTwice; the kernels do
not depend on its compile-time N) from the reference checkout, with the flags of its Makefile
(SB/CUDA_GPU/Makefile:9: -use_fast_math, -O3) retargeted to sm_103a, into oracle/_ref/m2_opt.cubin.
tests/golden/make_ref_golden.py loads that cubin on a GPU, drives it the way m2_opt.cu:main does
(with cuBLAS SGEMV for the field) and records golden trajectories.

SQA: SQA_fully/fully_test/pre_calculate.cu sets N and M (spins, Trotter slices) as #defines that its
kernels depend on; the recipe writes a copy with those two lines changed into a temporary directory
(deleted after the build) and compiles its device code, with the flags of its Makefile
(SQA_fully/fully_test/Makefile:6-7: nvcc defaults), into oracle/_ref/sqa_pre_calculate_n{N}_m{M}.cubin
for the pin cases below; tests/golden/make_sqa_golden.py drives those cubins the way its main does.
Nothing is copied into the repository: the sources are read where they lie.
Usage: python oracle/build_ref.py [reference checkout root]
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


SQA_CASES = ((256, 8), (512, 16))  # (N, M) of the SQA pin


def build_sqa(root, nvcc, out_dir):
    src = os.path.join(root, "SQA_fully", "fully_test", "pre_calculate.cu")
    if not os.path.exists(src):
        return 0
    text = open(src).read()
    rc = 0
    for N, M in SQA_CASES:
        out = os.path.join(out_dir, f"sqa_pre_calculate_n{N}_m{M}.cubin")
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        patched = re.sub(r"^#define N .*$", f"#define N {N}", text, flags=re.M)
        patched = re.sub(r"^#define M .*$", f"#define M {M}", patched, flags=re.M)
        with tempfile.TemporaryDirectory() as td:
            tmp = os.path.join(td, f"sqa_pre_calculate_n{N}_m{M}.cu")
            with open(tmp, "w") as f:
                f.write(patched)
            rc |= subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", tmp, "-o", out]).returncode
    return rc


def main(root="/root/reference"):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    rc = build_sqa(root, nvcc, out_dir)
    return rc | build_sb(root, nvcc, out_dir)


def build_sb(root, nvcc, out_dir):
    src = os.path.join(root, "SB", "CUDA_GPU", "m2_opt.cu")
    if not os.path.exists(src):
        print("reference source not present; skipping", src)
        return 0
    out = os.path.join(out_dir, "m2_opt.cubin")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return 0
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-use_fast_math",
           "-Xptxas", "-O3", src, "-o", out]
    return subprocess.run(cmd).returncode


if __name__ == "__main__":
    sys.exit(main(*sys.argv[1:]))
