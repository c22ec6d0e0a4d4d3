"""In-tree build of the native parts: the solver library, its CLI, and the CPU oracle.

Everything is compiled with plain nvcc / gcc calls (no cmake), object files in parallel:
  annealing_gb300/libsbsolve.so   CUDA kernels (sm_103a) + C ABI (include/sb.h)
  annealing_gb300/sb              command-line drop-in for the reference's `./opt <graph>`
  annealing_gb300/_checked/libsbsolve.so
                                  the same library with device bounds checks (-DSB_CHECKS), built
                                  on request (build_library(checks=True)) for the checked test run
  oracle/libsboracle.so           CPU oracle + multithreaded CPU baseline (test infrastructure)
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "annealing_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
CHECKED = os.path.join(PKG, "_checked")
ORACLE = os.path.join(ROOT, "oracle")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["sb_plain.cu", "sb_tc.cu", "sb_tc_fp8.cu", "sb_tc_bf16.cu", "sb_tc_split.cu", "sb_tc_split16.cu", "sb_tc_fp4.cu", "sb_grouped.cu", "sb_noalloc.cu",
               "sb_api.cpp", "sb_batch.cpp", "sb_problem.cpp", "sb_serve.cpp", "sb_analysis.cpp", "sb_sqa.cu",
               "sb_nmfa.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "sb.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def build_library(force: bool = False, checks: bool = False) -> str:
    """The solver library (and its CLI); checks=True: the bounds-checked library only, in _checked/."""
    bdir = os.path.join(CHECKED, "_build") if checks else BUILD
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + (["-DSB_CHECKS"] if checks else [])
    hdrs = _headers()
    objs, jobs = [], []
    for src in LIB_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            if src.endswith(".cu"):
                cmd = [nvcc, *GENCODE, "-lineinfo", *common, "-c", s, "-o", o]
            else:
                cmd = [nvcc, *common, "-c", s, "-o", o]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = os.path.join(CHECKED if checks else PKG, "libsbsolve.so")
    if force or jobs or not os.path.exists(lib):
        _run([nvcc, *GENCODE, "-shared", "-o", lib, *objs, "-lpthread"])
    if checks:
        return lib
    cli = os.path.join(PKG, "sb")
    cli_src = os.path.join(CSRC, "sb_cli.cpp")
    if force or not _newer(cli, [cli_src, lib] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", cli,
              "-L" + PKG, "-lsbsolve", "-Wl,-rpath,$ORIGIN"])
    return lib


def build_oracle(force: bool = False) -> str:
    out_dir = os.path.join(ORACLE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    exact = os.path.join(ORACLE, "sb_oracle.c")
    base = os.path.join(ORACLE, "sb_cpu_baseline.c")
    sqa = os.path.join(ORACLE, "sqa_oracle.c")
    nmfa = os.path.join(ORACLE, "nmfa_oracle.c")
    math_h = os.path.join(ORACLE, "sb_math_oracle.h")
    o1 = os.path.join(out_dir, "sb_oracle.o")
    o2 = os.path.join(out_dir, "sb_cpu_baseline.o")
    o3 = os.path.join(out_dir, "sqa_oracle.o")
    o4 = os.path.join(out_dir, "nmfa_oracle.o")
    lib = os.path.join(ORACLE, "libsboracle.so")
    jobs = []
    if force or not _newer(o1, [exact]):
        jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-c", exact, "-o", o1])
    if force or not _newer(o2, [base]):
        jobs.append(["gcc", "-O3", "-std=gnu11", "-fPIC", "-ffp-contract=fast", "-pthread",
                     "-c", base, "-o", o2])
    if force or not _newer(o3, [sqa, math_h]):
        jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-c", sqa, "-o", o3])
    if force or not _newer(o4, [nmfa, math_h]):
        jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-c", nmfa, "-o", o4])
    with ThreadPoolExecutor(max_workers=4) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or not os.path.exists(lib):
        _run(["gcc", "-shared", "-o", lib, o1, o2, o3, o4, "-lm", "-pthread"])
    return lib


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fl = ex.submit(build_library, force)
        fo = ex.submit(build_oracle, force)
        fl.result()
        fo.result()


if __name__ == "__main__":
    build_all(force=True)
    print("built", os.path.join(PKG, "libsbsolve.so"))
