"""Drivers of the reference's own GPU kernels — TEST AND BENCHMARK INFRASTRUCTURE ONLY.

The kernels are compiled from the reference's sources by oracle/build_ref.py into oracle/_ref/
(git-ignored; the files travel with the working tree). Used by the golden-vector generators in
tests/golden/ and by bench.py's reference arm, which times the reference SB program on the GPU next
to its CPU port. The solver package never imports this module.

  M2opt       SB/CUDA_GPU/m2_opt.cu: prepare_points and UpdateTwice from oracle/_ref/m2_opt.cubin,
              the field by cuBLAS SGEMV, driven as m2_opt.cu:main drives them (:130-187)
  NmfaKernel  NMFA/CUDA_GPU/src/nmfa.cu: gpu_nmfa_kernel from oracle/_ref/nmfa_states_n{N}.cubin,
              launched as gpu_nmfa does (nmfa.cu:161-184)
"""
import ctypes as C
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
M2OPT_CUBIN = os.path.join(HERE, "_ref", "m2_opt.cubin")
XI, DELTA_T = 0.01565, 1.0  # m2_opt.cu:18, :20
NMFA_KERNEL = b"_Z15gpu_nmfa_kernelPfPiS_iffj"
NMFA_NOISE, NMFA_RECOMB, NMFA_SEED = 0.15, 0.15, 1234  # Ising.cpp:11-13


def cublas():
    """The cuBLAS library torch has loaded (one small matrix-vector product loads it)."""
    import torch

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


def _driver():
    import torch

    cu = C.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")
    if cu.cuInit(0) != 0:
        raise RuntimeError("cuInit failed")
    return cu


def _args(args):
    return (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])


class M2opt:
    """The reference SB program's kernels and field call on an N x N matrix (N a multiple of 64,
    m2_opt.cu's launch shape N/64 x 64). `J` holds the instance in its first rows and columns, as the
    reference stores a graph with fewer spins than its compile-time N."""

    def __init__(self, J: np.ndarray):
        import torch

        self.N = J.shape[0]
        if self.N % 64 or J.shape != (self.N, self.N):
            raise ValueError("the reference's N is a square size that is a multiple of 64")
        if not os.path.exists(M2OPT_CUBIN):
            raise FileNotFoundError(M2OPT_CUBIN + " (built by oracle/build_ref.py)")
        self.cu = _driver()
        self.mod = C.c_void_p()
        rc = self.cu.cuModuleLoad(C.byref(self.mod), M2OPT_CUBIN.encode())
        if rc != 0:
            raise RuntimeError(f"cuModuleLoad failed: {rc}")
        self.f_prep, self.f_upd = C.c_void_p(), C.c_void_p()
        assert self.cu.cuModuleGetFunction(C.byref(self.f_prep), self.mod, b"_Z14prepare_pointsPfS_Pj") == 0
        assert self.cu.cuModuleGetFunction(C.byref(self.f_upd), self.mod, b"_Z11UpdateTwicePfS_f") == 0
        self.cb = cublas()
        self.handle = C.c_void_p()
        assert self.cb.cublasCreate_v2(C.byref(self.handle)) == 0
        self.J = torch.from_numpy(np.ascontiguousarray(J, np.float32)).cuda()
        self.rand = torch.arange(self.N, dtype=torch.int32, device="cuda")  # initRand[i] = i
        self.x = torch.zeros(self.N, device="cuda")
        self.y = torch.zeros(self.N, device="cuda")
        self.coeff1 = C.c_float(np.float32(DELTA_T * XI))
        self.coeff2 = C.c_float(1.0)
        self.px, self.py = C.c_void_p(self.x.data_ptr()), C.c_void_p(self.y.data_ptr())
        self.pr = C.c_void_p(self.rand.data_ptr())

    def _launch(self, fn, args):
        rc = self.cu.cuLaunchKernel(fn, self.N // 64, 1, 1, 64, 1, 1, 0, None, _args(args), None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel: {rc}")

    def prepare(self):
        """prepare_points<<<N/64, 64>>> (m2_opt.cu:48-56, launched at :152): one trial's x, y."""
        self._launch(self.f_prep, [self.px, self.py, self.pr])

    def step(self, s, steps):
        """One SB step (m2_opt.cu:158-169): UpdateTwice with amplitude s/STEP, then
        y += DeltaT*xi * J x by cublasSgemv."""
        self._launch(self.f_upd, [self.px, self.py, C.c_float(np.float32(s) / np.float32(steps))])
        rc = self.cb.cublasSgemv_v2(self.handle, 0, self.N, self.N, C.byref(self.coeff1),
                                    C.c_void_p(self.J.data_ptr()), self.N, self.px, 1, C.byref(self.coeff2),
                                    self.py, 1)
        if rc != 0:
            raise RuntimeError(f"cublasSgemv: {rc}")

    def time_steps(self, steps, warmup=20):
        """Milliseconds per SB step, two ways: as the program runs it (an event pair and an event
        synchronize around every step, m2_opt.cu:159-185; host wall time) and with the same
        launches back to back (one event pair around all steps)."""
        import torch

        self.prepare()
        for s in range(warmup):
            self.step(s, steps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            self.step(s, steps)
            b.record()
            b.synchronize()
            a.elapsed_time(b)
        as_program = 1e3 * (time.perf_counter() - t0) / steps
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for s in range(steps):
            self.step(s, steps)
        b.record()
        b.synchronize()
        return as_program, a.elapsed_time(b) / steps

    def close(self):
        self.cb.cublasDestroy_v2(self.handle)
        self.cu.cuModuleUnload(self.mod)


def nmfa_schedule(stages):
    """Ising.cpp:37-43 in FP32."""
    inc = np.float32((np.float32(8) - np.float32(1) / np.float32(16)) / np.float32(stages))
    b, out = np.float32(1) / np.float32(16), []
    for _ in range(stages):
        out.append(b)
        b = np.float32(b + inc)
    return np.array(out, np.float32)


class NmfaKernel:
    """gpu_nmfa_kernel for N spins: one CTA of N threads per sample, N floats of dynamic shared
    memory; as oracle/build_ref.py expands it, its last store writes the final mean-field state
    instead of its sign."""

    def __init__(self, n):
        self.cu = _driver()
        self.n = n
        self.mod = C.c_void_p()
        path = os.path.join(HERE, "_ref", f"nmfa_states_n{n}.cubin")
        if self.cu.cuModuleLoad(C.byref(self.mod), path.encode()) != 0:
            raise RuntimeError("cuModuleLoad failed: build " + path + " with oracle/build_ref.py")
        self.fn = C.c_void_p()
        assert self.cu.cuModuleGetFunction(C.byref(self.fn), self.mod, NMFA_KERNEL) == 0

    def run(self, J, betas, samples, timed=False):
        """Final states [samples, n] (and the kernel's event time in ms)."""
        import torch

        n = self.n
        dJ = torch.from_numpy(np.ascontiguousarray(J, np.float32)).cuda()
        db = torch.from_numpy(np.ascontiguousarray(betas, np.float32)).cuda()
        out = torch.zeros(samples * n, dtype=torch.int32, device="cuda")
        args = [C.c_void_p(dJ.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(db.data_ptr()),
                C.c_int(len(betas)), C.c_float(NMFA_NOISE), C.c_float(NMFA_RECOMB), C.c_uint32(NMFA_SEED)]
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        if self.cu.cuLaunchKernel(self.fn, samples, 1, 1, n, 1, 1, n * 4, None, _args(args), None) != 0:
            raise RuntimeError("cuLaunchKernel failed")
        b.record()
        b.synchronize()
        states = out.cpu().numpy().view(np.float32).reshape(samples, n).copy()
        return (states, a.elapsed_time(b)) if timed else states

    def close(self):
        self.cu.cuModuleUnload(self.mod)
