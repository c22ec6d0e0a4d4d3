"""ctypes binding of the solver's C ABI (include/sb.h).

This mirrors the reference program's contract (SB/CUDA_GPU/m2_opt.cu): read a graph, run SB
trials, report one energy per trial and the best spin vector. There is no CPU fallback: if
libsbsolve.so is missing this module raises on import of the library, and every solve runs the
CUDA kernels in that library.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# SB_LIBRARY selects another build of the same ABI (the bounds-checked one in _checked/)
LIB_PATH = os.environ.get("SB_LIBRARY") or os.path.join(_HERE, "libsbsolve.so")

# enums (sb.h)
SB_OK, SB_ERR_PENDING = 0, 12
ASB, BSB, DSB = 0, 1, 2
FIELD_AUTO, FIELD_FP32, FIELD_TC = 0, 1, 2
INIT_UNIFORM, INIT_REFERENCE = 0, 1
DTYPE_NAMES = {0: "f32", 1: "fp8e4m3", 2: "bf16", 3: "bf16x2", 4: "fp4e2m1", 5: "fp16x2", 6: "fp6e2m3"}
OPERAND_AUTO, OPERAND_FP8, OPERAND_BF16, OPERAND_BF16X2, OPERAND_FP4, OPERAND_FP16X2, OPERAND_FP6 = 0, 1, 2, 3, 4, 5, 6
VARIANTS = {"asb": ASB, "bsb": BSB, "dsb": DSB}


class GraphOpts(C.Structure):
    _fields_ = [("index_base", C.c_int32), ("n_override", C.c_int32), ("strict", C.c_int32)]


class ProblemStruct(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("J", C.POINTER(C.c_float)),
        ("h", C.POINTER(C.c_float)),
        ("integer_valued", C.c_int32),
        ("max_abs_j", C.c_int32),
        ("n_edges", C.c_int64),
        ("lib_owned", C.c_int32),
        ("stats_valid", C.c_int32),
        ("sum_j", C.c_int64),
        ("sum_j2", C.c_int64),
    ]


class Params(C.Structure):
    _fields_ = [
        ("variant", C.c_int32),
        ("field_mode", C.c_int32),
        ("init_mode", C.c_int32),
        ("steps", C.c_int32),
        ("replicas", C.c_int32),
        ("seed", C.c_uint64),
        ("dt", C.c_float),
        ("a0", C.c_float),
        ("c0", C.c_float),
        ("mts_m", C.c_int32),
        ("mts_dt", C.c_float),
        ("coupling_dt", C.c_float),
        ("xi", C.c_float),
        ("detune", C.c_float),
        ("kerr", C.c_float),
        ("trace", C.c_int32),
        ("trace_all", C.c_int32),
        ("profile", C.c_int32),
        ("operand_dtype", C.c_int32),
    ]

    @classmethod
    def default(cls, variant: int = DSB, **kw) -> "Params":
        p = cls()
        lib().sb_params_default(C.byref(p), variant)
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p


class ResultStruct(C.Structure):
    _fields_ = [
        ("best_spins", C.POINTER(C.c_int8)),
        ("replica_energies", C.POINTER(C.c_double)),
        ("energy_trace", C.POINTER(C.c_double)),
        ("energy_trace_all", C.POINTER(C.c_double)),
        ("final_x", C.POINTER(C.c_float)),
        ("final_y", C.POINTER(C.c_float)),
        ("best_energy", C.c_double),
        ("best_energy_i64", C.c_int64),
        ("best_replica", C.c_int32),
        ("field_mode_used", C.c_int32),
        ("field_dtype_used", C.c_int32),
        ("energy_check_ok", C.c_int32),
        ("device_ms", C.c_double),
        ("kernel_ms_avg", C.c_double),
        ("steps_per_launch", C.c_int32),
        ("kernel_launches", C.c_int64),
        ("total_ms", C.c_double),
        ("spin_updates_per_s", C.c_double),
    ]


class DeviceOpts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("stream", C.c_void_p),
        ("hbm_budget_bytes", C.c_int64),
        ("max_inflight", C.c_int32),
    ]


class ServingStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64),
        ("finished", C.c_int64),
        ("cancelled", C.c_int64),
        ("inflight", C.c_int64),
        ("queued", C.c_int64),
        ("grouped_launches", C.c_int64),
        ("busy_ms", C.c_double),
        ("peak_inflight", C.c_int64),
        ("ticks", C.c_int64),
        ("admit_ms", C.c_double),
    ]


SQA_RNG_REFERENCE, SQA_RNG_HASH = 0, 1


class SqaParams(C.Structure):
    _fields_ = [
        ("trotter", C.c_int32),
        ("steps", C.c_int32),
        ("replicas", C.c_int32),
        ("rng_mode", C.c_int32),
        ("seed", C.c_uint64),
        ("trace", C.c_int32),
    ]

    @classmethod
    def default(cls, **kw) -> "SqaParams":
        p = cls()
        lib().sb_sqa_params_default(C.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p


class SqaResultStruct(C.Structure):
    _fields_ = [
        ("best_spins", C.POINTER(C.c_int8)),
        ("replica_energies", C.POINTER(C.c_double)),
        ("energy_trace", C.POINTER(C.c_double)),
        ("final_spins", C.POINTER(C.c_int8)),
        ("best_energy", C.c_double),
        ("best_energy_i64", C.c_int64),
        ("best_replica", C.c_int32),
        ("energy_check_ok", C.c_int32),
        ("device_ms", C.c_double),
        ("total_ms", C.c_double),
        ("spin_updates_per_s", C.c_double),
        ("kernel_launches", C.c_int64),
    ]


@dataclass
class SqaResult:
    best_spins: np.ndarray
    replica_energies: np.ndarray
    best_energy: float
    best_energy_i64: int
    best_replica: int
    energy_check_ok: bool
    device_ms: float
    total_ms: float
    spin_updates_per_s: float
    kernel_launches: int
    energy_trace: Optional[np.ndarray] = None   # [replicas, steps]
    final_spins: Optional[np.ndarray] = None    # [replicas, trotter, n]


class NmfaParams(C.Structure):
    _fields_ = [
        ("samples", C.c_int32),
        ("stages", C.c_int32),
        ("betas", C.POINTER(C.c_float)),
        ("noise", C.c_float),
        ("recombination", C.c_float),
        ("seed", C.c_uint32),
        ("field_mode", C.c_int32),
    ]

    @classmethod
    def default(cls, **kw) -> "NmfaParams":
        p = cls()
        lib().sb_nmfa_params_default(C.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p


class NmfaResultStruct(C.Structure):
    _fields_ = [
        ("samples", C.POINTER(C.c_int8)),
        ("states", C.POINTER(C.c_float)),
        ("energies", C.POINTER(C.c_double)),
        ("best_spins", C.POINTER(C.c_int8)),
        ("best_energy", C.c_double),
        ("best_sample", C.c_int32),
        ("energy_check_ok", C.c_int32),
        ("device_ms", C.c_double),
        ("total_ms", C.c_double),
        ("spin_updates_per_s", C.c_double),
        ("kernel_launches", C.c_int64),
        ("field_mode_used", C.c_int32),
    ]


@dataclass
class NmfaResult:
    samples: np.ndarray          # [samples, n] int8 +-1
    energies: np.ndarray         # [samples] E = sum_{i<j} J_ij s_i s_j
    best_spins: np.ndarray
    best_energy: float
    best_sample: int
    energy_check_ok: bool
    device_ms: float
    total_ms: float
    spin_updates_per_s: float
    kernel_launches: int
    field_mode_used: int = 0                   # FIELD_FP32 or FIELD_TC
    states: Optional[np.ndarray] = None   # [samples, n] final mean-field states


class TtsStruct(C.Structure):
    _fields_ = [
        ("trials", C.c_int32),
        ("reached", C.c_int32),
        ("succeeded", C.c_int32),
        ("best_ms", C.c_double),
        ("mean_ms", C.c_double),
        ("worst_ms", C.c_double),
        ("success_rate", C.c_double),
        ("tts_ms", C.c_double),
    ]


# Every symbol include/sb.h declares, with its ctypes signature.
_SIGS = {
    "sb_status_string": (C.c_char_p, [C.c_int]),
    "sb_abi_version": (C.c_int32, []),
    "sb_params_default": (None, [C.POINTER(Params), C.c_int32]),
    "sb_graph_opts_default": (None, [C.POINTER(GraphOpts)]),
    "sb_load_graph": (C.c_int, [C.c_char_p, C.POINTER(ProblemStruct)]),
    "sb_load_graph_ex": (C.c_int, [C.c_char_p, C.POINTER(GraphOpts), C.POINTER(ProblemStruct)]),
    "sb_problem_init": (C.c_int, [C.POINTER(ProblemStruct), C.c_int32, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
    "sb_problem_wrap": (C.c_int, [C.POINTER(ProblemStruct), C.c_int32, C.c_void_p, C.c_void_p]),
    "sb_problem_free": (None, [C.POINTER(ProblemStruct)]),
    "sb_problem_random": (C.c_int, [C.POINTER(ProblemStruct), C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                    C.c_uint64]),
    "sb_coupling_std": (C.c_double, [C.POINTER(ProblemStruct)]),
    "sb_default_c0": (C.c_float, [C.POINTER(ProblemStruct)]),
    "sb_pump": (C.c_float, [C.c_float, C.c_int32, C.c_int32]),
    "sb_energy_i64": (C.c_int, [C.POINTER(ProblemStruct), C.POINTER(C.c_int8),
                                C.POINTER(C.c_int64)]),
    "sb_energy_f64": (C.c_double, [C.POINTER(ProblemStruct), C.POINTER(C.c_int8)]),
    "sb_energies_i64": (C.c_int, [C.POINTER(ProblemStruct), C.POINTER(C.c_int8), C.c_int32,
                                  C.POINTER(C.c_int64)]),
    "sb_sqa_params_default": (None, [C.POINTER(SqaParams)]),
    "sb_sqa_schedule": (None, [C.c_int32, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sb_sqa_solve": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.POINTER(SqaParams),
                               C.POINTER(SqaResultStruct)]),
    "sb_nmfa_params_default": (C.c_int, [C.POINTER(NmfaParams)]),
    "sb_nmfa_schedule": (C.c_int, [C.c_int32, C.POINTER(C.c_float)]),
    "sb_nmfa_solve": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.POINTER(NmfaParams),
                                C.POINTER(NmfaResultStruct)]),
    "sb_gpu_nmfa": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                              C.c_int32, C.POINTER(C.c_int32), C.c_float, C.c_float, C.c_uint32,
                              C.POINTER(C.c_float)]),
    "sb_time_to_target": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32, C.c_int32,
                                    C.c_int32, C.c_double, C.c_double, C.c_double, C.POINTER(TtsStruct)]),
    "sb_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(DeviceOpts)]),
    "sb_destroy": (C.c_int, [C.c_void_p]),
    "sb_last_error": (C.c_char_p, [C.c_void_p]),
    "sb_solve": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.POINTER(Params),
                           C.POINTER(ResultStruct)]),
    "sb_plan_create": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.POINTER(Params),
                                 C.POINTER(C.c_void_p)]),
    "sb_plan_run": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(ResultStruct)]),
    "sb_plan_destroy": (C.c_int, [C.c_void_p]),
    "sb_plan_footprint": (C.c_int64, [C.POINTER(ProblemStruct), C.POINTER(Params)]),
    "sb_submit": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.POINTER(Params),
                            C.POINTER(C.c_uint64)]),
    "sb_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(ResultStruct), C.c_int32]),
    "sb_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "sb_serving_stats_get": (C.c_int, [C.c_void_p, C.POINTER(ServingStats)]),
    "sb_batch_create": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.c_int32, C.POINTER(Params),
                                  C.POINTER(C.c_void_p)]),
    "sb_batch_run": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(ResultStruct)]),
    "sb_batch_destroy": (C.c_int, [C.c_void_p]),
    "sb_solve_batch": (C.c_int, [C.c_void_p, C.POINTER(ProblemStruct), C.c_int32, C.POINTER(Params),
                                 C.POINTER(ResultStruct)]),
    "sb_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int64]),
    "sb_debug_skip_publish": (C.c_int, [C.c_void_p, C.c_int32]),
    "sb_dsb_solve_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Load libsbsolve.so (built in-tree by __graft_entry__.build()). Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class SBError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        name = lib().sb_status_string(status).decode()
        super().__init__(f"{name} ({status}): {msg}")


def _check(status: int, ctx=None) -> None:
    if status != SB_OK:
        raise SBError(status, (lib().sb_last_error(ctx) or b"").decode())


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Problem:
    """A dense symmetric Ising instance: H(s) = -sum_{i<j} J_ij s_i s_j - sum_i h_i s_i."""

    def __init__(self, struct: ProblemStruct, owner=None):
        self.s = struct
        self._owner = owner

    @classmethod
    def from_dense(cls, J: np.ndarray, h: Optional[np.ndarray] = None) -> "Problem":
        J = np.ascontiguousarray(J, dtype=np.float32)
        n = J.shape[0]
        if J.shape != (n, n):
            raise ValueError("J must be square")
        hh = None if h is None else np.ascontiguousarray(h, dtype=np.float32)
        st = ProblemStruct()
        _check(lib().sb_problem_init(C.byref(st), n, _fp(J), _fp(hh) if hh is not None else None))
        return cls(st)

    @classmethod
    def wrap(cls, n: int, J_ptr: int, h_ptr: int = 0, keepalive=None) -> "Problem":
        """Refer to caller-owned host memory (e.g. pinned buffers) without copying."""
        st = ProblemStruct()
        _check(lib().sb_problem_wrap(C.byref(st), n, J_ptr, h_ptr or None))
        return cls(st, owner=keepalive)

    @classmethod
    def random(cls, n: int, density: float = 1.0, jmax: int = 1, field_max: int = 0,
               seed: int = 1234) -> "Problem":
        """Seeded G(n, density) instance: couplings +-1 (jmax = 1) or uniform in [-jmax, jmax]."""
        st = ProblemStruct()
        _check(lib().sb_problem_random(C.byref(st), n, density, jmax, field_max, seed))
        return cls(st)

    @classmethod
    def load(cls, path: str, index_base: int = -1, n: int = 0, strict: bool = False) -> "Problem":
        o = GraphOpts(index_base, n, 1 if strict else 0)
        st = ProblemStruct()
        _check(lib().sb_load_graph_ex(path.encode(), C.byref(o), C.byref(st)))
        return cls(st)

    @property
    def n(self) -> int:
        return self.s.n

    @property
    def J(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.s.J, shape=(self.n, self.n))

    @property
    def h(self) -> Optional[np.ndarray]:
        return np.ctypeslib.as_array(self.s.h, shape=(self.n,)) if self.s.h else None

    @property
    def integer_valued(self) -> bool:
        return bool(self.s.integer_valued)

    def default_c0(self) -> float:
        return lib().sb_default_c0(C.byref(self.s))

    def energy(self, spins: np.ndarray) -> float:
        sp = np.ascontiguousarray(spins, dtype=np.int8)
        if self.integer_valued:
            out = C.c_int64()
            _check(lib().sb_energy_i64(C.byref(self.s), sp.ctypes.data_as(C.POINTER(C.c_int8)),
                                       C.byref(out)))
            return int(out.value)
        return lib().sb_energy_f64(C.byref(self.s), sp.ctypes.data_as(C.POINTER(C.c_int8)))

    def energies(self, spins: np.ndarray) -> np.ndarray:
        """Exact int64 energies of several spin vectors (rows of `spins`, int8 +-1); couplings
        in {-1, 0, +1} or |J| <= 127 are read from a compact copy (sb_energies_i64)."""
        sp = np.ascontiguousarray(np.atleast_2d(spins), dtype=np.int8)
        if sp.shape[1] != self.n:
            raise ValueError("spins must have n columns")
        out = np.zeros(sp.shape[0], np.int64)
        _check(lib().sb_energies_i64(C.byref(self.s), sp.ctypes.data_as(C.POINTER(C.c_int8)), sp.shape[0],
                                     out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def close(self) -> None:
        if self.s.J:
            lib().sb_problem_free(C.byref(self.s))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Result:
    best_spins: np.ndarray
    replica_energies: np.ndarray
    best_energy: float
    best_energy_i64: int
    best_replica: int
    field_mode: int
    field_dtype: str
    energy_check_ok: bool
    device_ms: float
    kernel_ms_avg: float
    steps_per_launch: int
    kernel_launches: int
    total_ms: float
    spin_updates_per_s: float
    energy_trace: Optional[np.ndarray] = None
    energy_trace_all: Optional[np.ndarray] = None
    final_x: Optional[np.ndarray] = None
    final_y: Optional[np.ndarray] = None


class _ResultBuffers:
    def __init__(self, n: int, params: Params, want_state: bool):
        R, T = params.replicas, params.steps
        self.spins = np.zeros(n, np.int8)
        self.energies = np.zeros(R, np.float64)
        self.trace = np.zeros(T + 1, np.float64) if params.trace else None
        self.trace_all = np.zeros((T + 1, R), np.float64) if params.trace_all else None
        self.x = np.zeros((R, n), np.float32) if want_state else None
        self.y = np.zeros((R, n), np.float32) if want_state else None
        r = ResultStruct()
        r.best_spins = self.spins.ctypes.data_as(C.POINTER(C.c_int8))
        r.replica_energies = self.energies.ctypes.data_as(C.POINTER(C.c_double))
        if self.trace is not None:
            r.energy_trace = self.trace.ctypes.data_as(C.POINTER(C.c_double))
        if self.trace_all is not None:
            r.energy_trace_all = self.trace_all.ctypes.data_as(C.POINTER(C.c_double))
        if want_state:
            r.final_x = _fp(self.x)
            r.final_y = _fp(self.y)
        self.r = r

    def result(self) -> Result:
        r = self.r
        return Result(
            best_spins=self.spins, replica_energies=self.energies, best_energy=r.best_energy,
            best_energy_i64=r.best_energy_i64, best_replica=r.best_replica,
            field_mode=r.field_mode_used, field_dtype=DTYPE_NAMES.get(r.field_dtype_used, "?"),
            energy_check_ok=bool(r.energy_check_ok), device_ms=r.device_ms,
            kernel_ms_avg=r.kernel_ms_avg, steps_per_launch=r.steps_per_launch,
            kernel_launches=r.kernel_launches, total_ms=r.total_ms,
            spin_updates_per_s=r.spin_updates_per_s, energy_trace=self.trace,
            energy_trace_all=self.trace_all, final_x=self.x, final_y=self.y)


class Plan:
    """J resident on the device; each run() is one solve (init, steps, final energy)."""

    def __init__(self, ctx: "Context", problem: Problem, params: Params, want_state: bool):
        self.ctx, self.problem, self.params, self.want_state = ctx, problem, params, want_state
        h = C.c_void_p()
        _check(lib().sb_plan_create(ctx.h, C.byref(problem.s), C.byref(params), C.byref(h)), ctx.h)
        self.h = h

    def run(self, seed: Optional[int] = None) -> Result:
        buf = _ResultBuffers(self.problem.n, self.params, self.want_state)
        sd = self.params.seed if seed is None else seed
        _check(lib().sb_plan_run(self.h, sd, C.byref(buf.r)), self.ctx.h)
        return buf.result()

    def close(self) -> None:
        if self.h:
            lib().sb_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many instances solved together by the grouped tensor-core kernel (sb_batch_*)."""

    def __init__(self, ctx: "Context", problems, params: Params, want_state: bool = False):
        self.ctx, self.problems, self.params, self.want_state = ctx, list(problems), params, want_state
        self._arr = (ProblemStruct * len(self.problems))(*[p.s for p in self.problems])
        h = C.c_void_p()
        _check(lib().sb_batch_create(ctx.h, self._arr, len(self.problems), C.byref(params), C.byref(h)), ctx.h)
        self.h = h

    def run(self, seed: Optional[int] = None):
        bufs = [_ResultBuffers(p.n, self.params, self.want_state) for p in self.problems]
        arr = (ResultStruct * len(bufs))(*[b.r for b in bufs])
        sd = self.params.seed if seed is None else seed
        _check(lib().sb_batch_run(self.h, sd, arr), self.ctx.h)
        out = []
        for b, r in zip(bufs, arr):
            b.r = r
            out.append(b.result())
        return out

    def close(self) -> None:
        if self.h:
            lib().sb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One device, one stream (cudaStream_t as an integer handle, or None for an owned one)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None, hbm_budget: int = 0,
                 max_inflight: int = 0):
        o = DeviceOpts(device, stream or None, hbm_budget, max_inflight)
        h = C.c_void_p()
        _check(lib().sb_create(C.byref(h), C.byref(o)))
        self.h = h

    def solve(self, problem: Problem, params: Params, want_state: bool = False) -> Result:
        buf = _ResultBuffers(problem.n, params, want_state)
        _check(lib().sb_solve(self.h, C.byref(problem.s), C.byref(params), C.byref(buf.r)), self.h)
        return buf.result()

    def sqa_solve(self, problem: Problem, params: SqaParams, want_spins: bool = False) -> SqaResult:
        """Simulated quantum annealing (sb_sqa_solve)."""
        n, R, M, T = problem.n, params.replicas, params.trotter, params.steps
        spins = np.zeros(n, np.int8)
        energies = np.zeros(R, np.float64)
        trace = np.zeros((R, T), np.float64) if params.trace else None
        allsp = np.zeros((R, M, n), np.int8) if want_spins else None
        r = SqaResultStruct()
        r.best_spins = spins.ctypes.data_as(C.POINTER(C.c_int8))
        r.replica_energies = energies.ctypes.data_as(C.POINTER(C.c_double))
        if trace is not None:
            r.energy_trace = trace.ctypes.data_as(C.POINTER(C.c_double))
        if allsp is not None:
            r.final_spins = allsp.ctypes.data_as(C.POINTER(C.c_int8))
        _check(lib().sb_sqa_solve(self.h, C.byref(problem.s), C.byref(params), C.byref(r)), self.h)
        return SqaResult(best_spins=spins, replica_energies=energies, best_energy=r.best_energy,
                         best_energy_i64=r.best_energy_i64, best_replica=r.best_replica,
                         energy_check_ok=bool(r.energy_check_ok), device_ms=r.device_ms,
                         total_ms=r.total_ms, spin_updates_per_s=r.spin_updates_per_s,
                         kernel_launches=r.kernel_launches, energy_trace=trace, final_spins=allsp)

    def nmfa_solve(self, problem: Problem, params: Optional[NmfaParams] = None, betas=None,
                   want_states: bool = False) -> NmfaResult:
        """Noisy mean-field annealing (sb_nmfa_solve); betas (stages,) overrides the schedule."""
        params = params if params is not None else NmfaParams.default()
        keep = None
        if betas is not None:
            keep = np.ascontiguousarray(betas, np.float32)
            params.stages = len(keep)
            params.betas = keep.ctypes.data_as(C.POINTER(C.c_float))
        n, R = problem.n, params.samples
        samples = np.zeros((R, n), np.int8)
        energies = np.zeros(R, np.float64)
        best = np.zeros(n, np.int8)
        states = np.zeros((R, n), np.float32) if want_states else None
        r = NmfaResultStruct()
        r.samples = samples.ctypes.data_as(C.POINTER(C.c_int8))
        r.energies = energies.ctypes.data_as(C.POINTER(C.c_double))
        r.best_spins = best.ctypes.data_as(C.POINTER(C.c_int8))
        if states is not None:
            r.states = states.ctypes.data_as(C.POINTER(C.c_float))
        try:
            _check(lib().sb_nmfa_solve(self.h, C.byref(problem.s), C.byref(params), C.byref(r)), self.h)
        finally:
            if keep is not None:
                params.betas = None
        return NmfaResult(samples=samples, energies=energies, best_spins=best, best_energy=r.best_energy,
                          best_sample=r.best_sample, energy_check_ok=bool(r.energy_check_ok), device_ms=r.device_ms,
                          total_ms=r.total_ms, spin_updates_per_s=r.spin_updates_per_s,
                          kernel_launches=r.kernel_launches, field_mode_used=r.field_mode_used, states=states)

    def gpu_nmfa(self, J: np.ndarray, betas, num_samples: int, noise: float = 0.15, recombination: float = 0.15,
                 seed: int = 1234):
        """The reference's entry point gpu_nmfa (sb_gpu_nmfa): (samples [num_samples, n] int32, elapsed ms)."""
        J = np.ascontiguousarray(J, np.float32)
        b = np.ascontiguousarray(betas, np.float32)
        n = J.shape[0]
        out = np.zeros((num_samples, n), np.int32)
        ms = C.c_float()
        _check(lib().sb_gpu_nmfa(self.h, n, J.ctypes.data_as(C.POINTER(C.c_float)), b.ctypes.data_as(C.POINTER(C.c_float)),
                                 len(b), num_samples, out.ctypes.data_as(C.POINTER(C.c_int32)), noise, recombination,
                                 seed, C.byref(ms)), self.h)
        return out, ms.value

    def plan(self, problem: Problem, params: Params, want_state: bool = False) -> Plan:
        return Plan(self, problem, params, want_state)

    def batch(self, problems, params: Params, want_state: bool = False) -> Batch:
        return Batch(self, problems, params, want_state)

    def submit(self, problem: Problem, params: Params) -> int:
        t = C.c_uint64()
        _check(lib().sb_submit(self.h, C.byref(problem.s), C.byref(params), C.byref(t)), self.h)
        return t.value

    def poll(self, ticket: int, n: int, params: Params, wait_ms: int = 0,
             want_state: bool = False) -> Optional[Result]:
        buf = _ResultBuffers(n, params, want_state)
        st = lib().sb_poll(self.h, ticket, C.byref(buf.r), wait_ms)
        if st == SB_ERR_PENDING:
            return None
        _check(st, self.h)
        return buf.result()

    def cancel(self, ticket: int) -> None:
        _check(lib().sb_cancel(self.h, ticket), self.h)

    def set_wait_limit(self, cycles: int) -> None:
        """Limit of every bounded wait in the tensor-core kernels, in SM clock cycles (0: default)."""
        _check(lib().sb_set_wait_limit(self.h, cycles), self.h)

    def debug_skip_publish(self, step: int) -> None:
        """Test hook: the next tensor-core solve runs with unit 0 leaving out its step `step` flag."""
        _check(lib().sb_debug_skip_publish(self.h, step), self.h)

    def serving_stats(self) -> dict:
        s = ServingStats()
        _check(lib().sb_serving_stats_get(self.h, C.byref(s)), self.h)
        return {k: getattr(s, k) for k, _ in ServingStats._fields_}

    def close(self) -> None:
        if self.h:
            lib().sb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pump(a0: float, t: int, steps: int) -> float:
    return lib().sb_pump(a0, t, steps)


def sqa_schedule(steps: int, trotter: int):
    """beta[p], J_perp[p] of the SQA schedule (sb_sqa_schedule)."""
    b = np.zeros(steps, np.float32)
    j = np.zeros(steps, np.float32)
    lib().sb_sqa_schedule(steps, trotter, b.ctypes.data_as(C.POINTER(C.c_float)), j.ctypes.data_as(C.POINTER(C.c_float)))
    return b, j


def nmfa_schedule(stages: int = 100) -> np.ndarray:
    """The NMFA inverse temperatures of NMFA/CUDA_GPU/Ising.cpp:37-43 (sb_nmfa_schedule)."""
    b = np.zeros(stages, np.float32)
    _check(lib().sb_nmfa_schedule(stages, b.ctypes.data_as(C.POINTER(C.c_float))))
    return b


def time_to_target(energies: np.ndarray, times_ms: np.ndarray, threshold: float, run_ms: float,
                   p_target: float = 0.99) -> dict:
    """Time-to-target summary of an energy trace (sb_time_to_target).

    energies: [rows, trials] (a Result's energy_trace_all, row = step). times_ms: [rows] (time at
    which each row was reached, shared by replicas that run together) or [rows, trials]. run_ms:
    the time of one run, used for the success-probability time.
    """
    e = np.ascontiguousarray(energies, dtype=np.float64)
    if e.ndim != 2:
        raise ValueError("energies must be [rows, trials]")
    t = np.ascontiguousarray(times_ms, dtype=np.float64)
    per_trial = 1 if t.ndim == 2 else 0
    if t.shape != (e.shape if per_trial else (e.shape[0],)):
        raise ValueError("times_ms must be [rows] or [rows, trials]")
    out = TtsStruct()
    dp = C.POINTER(C.c_double)
    _check(lib().sb_time_to_target(e.ctypes.data_as(dp), t.ctypes.data_as(dp), e.shape[0], e.shape[1],
                                   per_trial, threshold, run_ms, p_target, C.byref(out)))
    return {k: getattr(out, k) for k, _ in TtsStruct._fields_}


def success_threshold(final_energies: np.ndarray, divisor: int = 5) -> float:
    """Success cut of SA_naive/CUDA_GPU/tests/test.sh:26-28: the best energy plus 1/divisor of
    the spread between the worst and the best (divisor 5: "80% --> success"). Integer energies use
    the script's integer division."""
    e = np.asarray(final_energies, dtype=np.float64)
    small, big = float(e.min()), float(e.max())
    if np.all(e == np.round(e)):
        return small + float(int(big - small) // divisor)
    return small + (big - small) / divisor


def result_time_to_target(res: "Result", threshold: float, p_target: float = 0.99) -> dict:
    """time_to_target of a solve's energy_trace_all: row t is reached at t / steps of the solve's
    device time, every replica is a run and the run time is the solve's device time."""
    if res.energy_trace_all is None:
        raise ValueError("solve with trace_all=1 to get per-replica traces")
    rows = res.energy_trace_all.shape[0]
    steps = max(rows - 1, 1)
    times = np.arange(rows, dtype=np.float64) * (res.device_ms / steps)
    return time_to_target(res.energy_trace_all, times, threshold, res.device_ms, p_target)
