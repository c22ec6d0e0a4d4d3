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
NMFA: NMFA/CUDA_GPU/src/nmfa.cu is a template (its Makefile expands `for @i from A to B ... endfor`
blocks between START_PYTHON_PREPROCESS / END_PYTHON_PREPROCESS lines and the size __N__ with a
generator script before nvcc). The recipe below does that expansion itself on a copy in a temporary
directory, changes the kernel's last line to store the final mean-field state (the float's bits)
instead of its sign, and compiles the device code with the flags of NMFA/CUDA_GPU/Makefile:2
(-use_fast_math --fmad=true -prec-div=false) into oracle/_ref/nmfa_states_n{N}.cubin;
tests/golden/make_nmfa_golden.py drives those cubins the way gpu_nmfa (nmfa.cu:142-199) does.
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


NMFA_SIZES = (32, 128, 1024)  # spins of the NMFA pin (one warp; four warps; the reference's Ising.cpp size)


def expand_nmfa_template(text, n):
    """The size and the unrolled loops of nmfa.cu: every __N__ becomes n, and each block between
    START_PYTHON_PREPROCESS and END_PYTHON_PREPROCESS, of the form `for VAR from A to B`, body lines,
    `endfor`, becomes the body repeated for VAR = A .. B-1 with VAR replaced by its value."""
    text = text.replace("__N__", str(n))
    out, block = [], None
    for line in text.split("\n"):
        if "START_PYTHON_PREPROCESS" in line:
            block = []
        elif "END_PYTHON_PREPROCESS" in line:
            head = block[0].split()
            if len(head) != 6 or head[0] != "for" or head[2] != "from" or head[4] != "to" or block[-1] != "endfor":
                raise ValueError("unexpected template block: %r" % block[0])
            var, lo, hi = head[1], int(head[3]), int(head[5])
            for v in range(lo, hi):
                out.extend(b.replace(var, str(v)) for b in block[1:-1])
            block = None
        elif block is not None:
            block.append(line.strip())
        else:
            out.append(line)
    return "\n".join(out)


def build_nmfa(root, nvcc, out_dir):
    src = os.path.join(root, "NMFA", "CUDA_GPU", "src", "nmfa.cu")
    if not os.path.exists(src):
        return 0
    text = open(src).read()
    final = "samples[blockIdx.x*__N__ + threadIdx.x] = current_st > 0 ? 1 : -1;"
    if final not in text:
        print("nmfa.cu: final store not found; skipping")
        return 1
    text = text.replace(final, "samples[blockIdx.x*__N__ + threadIdx.x] = __float_as_int(current_st);")
    rc = 0
    for n in NMFA_SIZES:
        out = os.path.join(out_dir, f"nmfa_states_n{n}.cubin")
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        with tempfile.TemporaryDirectory() as td:
            tmp = os.path.join(td, f"nmfa_states_n{n}.cu")
            with open(tmp, "w") as f:
                f.write(expand_nmfa_template(text, n))
            shutil.copy(os.path.join(os.path.dirname(src), "cuda_nmfa.h"), os.path.join(td, "cuda_nmfa.h"))
            rc |= subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-use_fast_math",
                                  "--fmad=true", "-prec-div=false", tmp, "-o", out]).returncode
    return rc


def main(root="/root/reference"):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    rc = build_sqa(root, nvcc, out_dir)
    rc |= build_nmfa(root, nvcc, out_dir)
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
