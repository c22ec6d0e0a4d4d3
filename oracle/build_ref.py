"""Build the reference's own SB kernels for the oracle pin — TEST INFRASTRUCTURE ONLY.

Compiles the device code of SB/CUDA_GPU/m2_opt.cu (prepare_points, UpdateTwice; the kernels do
not depend on its compile-time N) from the reference checkout, with the flags of its Makefile
(SB/CUDA_GPU/Makefile:9: -use_fast_math, -O3) retargeted to sm_103a, into oracle/_ref/m2_opt.cubin.
tests/golden/make_ref_golden.py loads that cubin on a GPU, drives it the way m2_opt.cu:main does
(with cuBLAS SGEMV for the field) and records golden trajectories.
Nothing is copied from the reference: the source is read where it lies.
Usage: python oracle/build_ref.py [reference checkout root]
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root="/root/reference"):
    src = os.path.join(root, "SB", "CUDA_GPU", "m2_opt.cu")
    if not os.path.exists(src):
        print("reference source not present; skipping", src)
        return 0
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "m2_opt.cubin")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return 0
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-use_fast_math",
           "-Xptxas", "-O3", src, "-o", out]
    return subprocess.run(cmd).returncode


if __name__ == "__main__":
    sys.exit(main(*sys.argv[1:]))
