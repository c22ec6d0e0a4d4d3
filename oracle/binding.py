"""ctypes binding of oracle/libsboracle.so (the CPU oracle and the multithreaded CPU baseline).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline, never by the solver.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsboracle.so")
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        sig = {
            "oracle_xorshift32": (C.c_uint32, [C.POINTER(C.c_uint32)]),
            "oracle_init_reference": (None, [C.c_int, C.c_int, f32p, f32p]),
            "oracle_uniform_value": (C.c_float, [C.c_uint64, C.c_uint64]),
            "oracle_init_uniform": (None, [C.c_int, C.c_int, C.c_uint64, f32p, f32p]),
            "oracle_pump": (C.c_float, [C.c_float, C.c_int, C.c_int]),
            "oracle_coupling_std": (C.c_double, [C.c_int, f32p]),
            "oracle_default_c0": (C.c_float, [C.c_int, f32p]),
            "oracle_field_f32": (None, [C.c_int, C.c_int, f32p, f32p, f32p]),
            "oracle_field_f64": (None, [C.c_int, C.c_int, f32p, f64p, f64p]),
            "oracle_sb_update_f32": (None, [C.c_int, C.c_int, f32p, C.c_void_p, f32p, f32p,
                                            C.c_float, C.c_float, C.c_float, C.c_float]),
            "oracle_sb_run_f32": (None, [C.c_int, C.c_int, C.c_int, f32p, C.c_void_p, f32p, f32p,
                                         C.c_int, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                         C.c_void_p]),
            "oracle_sb_run_f64": (None, [C.c_int, C.c_int, C.c_int, f32p, C.c_void_p, f32p, f32p,
                                         f64p, f64p, C.c_int, C.c_double, C.c_double,
                                         C.c_double]),
            "oracle_asb_local": (None, [C.c_size_t, f32p, f32p, C.c_float, C.c_int, C.c_float,
                                        C.c_float, C.c_float]),
            "oracle_asb_coeff": (C.c_float, [C.c_float, C.c_float]),
            "oracle_asb_run": (None, [C.c_int, C.c_int, f32p, f32p, f32p, C.c_int, C.c_int,
                                      C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.c_void_p, C.c_void_p]),
            "oracle_energy_i64": (C.c_int, [C.c_int, f32p, C.c_void_p, i8p,
                                            C.POINTER(C.c_int64)]),
            "oracle_energy_f64": (C.c_double, [C.c_int, f32p, C.c_void_p, i8p]),
            "oracle_energies_of_x": (None, [C.c_int, C.c_int, f32p, C.c_void_p, f32p, f64p]),
            "oracle_cpu_run": (C.c_int, [C.c_int, C.c_int, C.c_int, f32p, C.c_void_p, f32p, f32p,
                                         C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                         C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.c_int]),
            "oracle_sqa_log": (C.c_float, [C.c_float]),
            "oracle_sqa_schedule": (None, [C.c_int, C.c_int, f32p, f32p]),
            "oracle_sqa_init_reference": (None, [C.c_int, C.c_int, C.c_int, i8p, u32p]),
            "oracle_sqa_init_hash": (None, [C.c_int, C.c_int, C.c_int, C.c_uint64, i8p]),
            "oracle_sqa_energy": (C.c_int64, [C.c_int, i8p, i8p]),
            "oracle_sqa_run": (C.c_int, [C.c_int, i8p, C.c_int, C.c_int, f32p, f32p, C.c_int, C.c_int,
                                         C.c_void_p, C.c_uint64, i8p, C.c_void_p]),
            "oracle_nmfa_schedule": (None, [C.c_int, f32p]),
            "oracle_nmfa_seed": (None, [C.c_int, C.c_int, C.c_uint32, u32p]),
            "oracle_nmfa_xorwow": (C.c_uint32, [u32p]),
            "oracle_nmfa_gauss": (None, [u32p, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "oracle_nmfa_tanh": (C.c_float, [C.c_float]),
            "oracle_nmfa_sincos": (None, [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "oracle_nmfa_run": (C.c_int, [C.c_int, f32p, C.c_int, f32p, C.c_int, C.c_float, C.c_float, C.c_uint32,
                                          f32p, i32p, C.c_void_p]),
        }
        for k, (r, a) in sig.items():
            fn = getattr(L, k)
            fn.restype = r
            fn.argtypes = a
        _lib = L
    return _lib


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def init_reference(n, R):
    x = np.zeros((R, n), np.float32)
    y = np.zeros((R, n), np.float32)
    lib().oracle_init_reference(n, R, x, y)
    return x, y


def init_uniform(n, R, seed):
    x = np.zeros((R, n), np.float32)
    y = np.zeros((R, n), np.float32)
    lib().oracle_init_uniform(n, R, seed, x, y)
    return x, y


def pump(a0, t, steps):
    return lib().oracle_pump(a0, t, steps)


def default_c0(J):
    J = np.ascontiguousarray(J, np.float32)
    return lib().oracle_default_c0(J.shape[0], J)


def coupling_std(J):
    J = np.ascontiguousarray(J, np.float32)
    return lib().oracle_coupling_std(J.shape[0], J)


def field_f32(J, v):
    J = np.ascontiguousarray(J, np.float32)
    v = np.ascontiguousarray(v, np.float32)
    f = np.zeros_like(v)
    lib().oracle_field_f32(J.shape[0], v.shape[0], J, v, f)
    return f


def sb_run_f32(variant, J, h, x, y, steps, a0, c0, dt, trace=False, trace_all=False):
    """bSB (1) / dSB (2) in FP32 with the device's operation order. x, y updated in place."""
    J = np.ascontiguousarray(J, np.float32)
    R = x.shape[0]
    tr = np.zeros(steps + 1) if trace else None
    tra = np.zeros((steps + 1, R)) if trace_all else None
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    lib().oracle_sb_run_f32(variant, J.shape[0], R, J, _vp(hh), x, y, steps, a0, c0, dt,
                            _vp(tr), _vp(tra))
    return tr, tra


def sb_run_f64(variant, J, h, x0, y0, steps, a0, c0, dt):
    J = np.ascontiguousarray(J, np.float32)
    R, n = x0.shape
    xd = np.zeros((R, n))
    yd = np.zeros((R, n))
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    lib().oracle_sb_run_f64(variant, n, R, J, _vp(hh), np.ascontiguousarray(x0),
                            np.ascontiguousarray(y0), xd, yd, steps, a0, c0, dt)
    return xd, yd


def asb_run(J, x, y, steps, m=2, mts_dt=0.5, coupling_dt=1.0, xi=0.01565, detune=1.0, kerr=1.0,
            want_trace=False):
    J = np.ascontiguousarray(J, np.float32)
    R, n = x.shape
    xt = np.zeros((steps, R, n), np.float32) if want_trace else None
    yt = np.zeros((steps, R, n), np.float32) if want_trace else None
    lib().oracle_asb_run(n, R, J, x, y, steps, m, mts_dt, coupling_dt, xi, detune, kerr, _vp(xt),
                         _vp(yt))
    return xt, yt


def asb_local(x, y, amp, m=2, mts_dt=0.5, detune=1.0, kerr=1.0):
    lib().oracle_asb_local(x.size, x, y, amp, m, mts_dt, detune, kerr)


def energy_i64(J, h, s):
    J = np.ascontiguousarray(J, np.float32)
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    out = C.c_int64()
    rc = lib().oracle_energy_i64(J.shape[0], J, _vp(hh), np.ascontiguousarray(s, np.int8),
                                 C.byref(out))
    if rc != 0:
        raise ValueError("non-integer couplings")
    return int(out.value)


def energy_f64(J, h, s):
    J = np.ascontiguousarray(J, np.float32)
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    return lib().oracle_energy_f64(J.shape[0], J, _vp(hh), np.ascontiguousarray(s, np.int8))


def energies_of_x(J, h, x):
    J = np.ascontiguousarray(J, np.float32)
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    e = np.zeros(x.shape[0])
    lib().oracle_energies_of_x(J.shape[0], x.shape[0], J, _vp(hh), x, e)
    return e


def cpu_run(variant, J, h, x, y, steps, a0=1.0, c0=0.0, dt=1.25, m=2, mts_dt=0.5,
            coupling_dt=1.0, xi=0.01565, detune=1.0, kerr=1.0, threads=None):
    """Multithreaded FP32 port (the timed CPU baseline). x, y (R, n) updated in place."""
    J = np.ascontiguousarray(J, np.float32)
    R, n = x.shape
    hh = None if h is None else np.ascontiguousarray(h, np.float32)
    threads = threads or (os.cpu_count() or 1)
    rc = lib().oracle_cpu_run(variant, n, R, J, _vp(hh), x, y, steps, a0, c0, dt, m, mts_dt,
                              coupling_dt, xi, detune, kerr, threads)
    if rc != 0:
        raise RuntimeError(f"oracle_cpu_run failed: {rc}")
    return threads


# ---- SQA (oracle/sqa_oracle.c) ----

def sqa_log(u):
    return lib().oracle_sqa_log(u)


def sqa_schedule(steps, M):
    beta = np.zeros(steps, np.float32)
    jp = np.zeros(steps, np.float32)
    lib().oracle_sqa_schedule(steps, M, beta, jp)
    return beta, jp


def sqa_init(n, M, R, rng, seed=0):
    """Initial slices [R, M, n] int8 and (reference mode) the per-spin random words [R, n]."""
    s = np.zeros((R, M, n), np.int8)
    rnd = np.zeros((R, n), np.uint32)
    if rng == 0:
        lib().oracle_sqa_init_reference(n, M, R, s, rnd)
    else:
        lib().oracle_sqa_init_hash(n, M, R, seed, s)
    return s, (rnd if rng == 0 else None)


def sqa_run(J, spins, steps, rng, rnd=None, seed=0, beta=None, jperp=None):
    """SQA on spins [R, M, n] int8 (updated in place); returns the slice-0 energy trace [R, steps]."""
    J8 = np.ascontiguousarray(J, np.float32).astype(np.int8)
    R, M, n = spins.shape
    if beta is None:
        beta, jperp = sqa_schedule(steps, M)
    trace = np.zeros((R, steps), np.int64)
    rc = lib().oracle_sqa_run(n, J8, M, steps, np.ascontiguousarray(beta, np.float32),
                              np.ascontiguousarray(jperp, np.float32), R, rng,
                              _vp(None if rnd is None else np.ascontiguousarray(rnd, np.uint32)), seed,
                              spins, _vp(trace))
    if rc != 0:
        raise ValueError("bad SQA sizes")
    return trace


def sqa_energy(J, s):
    J8 = np.ascontiguousarray(J, np.float32).astype(np.int8)
    return int(lib().oracle_sqa_energy(J8.shape[0], J8, np.ascontiguousarray(s, np.int8)))


def nmfa_schedule(stages):
    b = np.zeros(stages, np.float32)
    lib().oracle_nmfa_schedule(stages, b)
    return b


def nmfa_seed(n, R, seed):
    """XORWOW words [R, n, 5] of every (sample, spin)."""
    w = np.zeros((R, n, 5), np.uint32)
    lib().oracle_nmfa_seed(n, R, seed, w)
    return w


def nmfa_gauss(words, noise):
    """One stage's two Gaussian samples from a (5,) uint32 state, advanced in place."""
    z0, z1 = C.c_float(), C.c_float()
    lib().oracle_nmfa_gauss(words, noise, C.byref(z0), C.byref(z1))
    return z0.value, z1.value


def nmfa_tanh(x):
    return lib().oracle_nmfa_tanh(x)


def nmfa_sincos(t):
    s, c = C.c_float(), C.c_float()
    lib().oracle_nmfa_sincos(t, C.byref(s), C.byref(c))
    return s.value, c.value


def nmfa_run(J, samples, betas, noise=0.15, recombination=0.15, seed=1234, trace=False):
    """NMFA on J [n, n]: (states [R, n] float32, samples [R, n] int32, trace [stages, R, n] or None)."""
    J = np.ascontiguousarray(J, np.float32)
    n = J.shape[0]
    betas = np.ascontiguousarray(betas, np.float32)
    st = np.zeros((samples, n), np.float32)
    sp = np.zeros((samples, n), np.int32)
    tr = np.zeros((len(betas), samples, n), np.float32) if trace else None
    rc = lib().oracle_nmfa_run(n, J, samples, betas, len(betas), noise, recombination, seed, st, sp, _vp(tr))
    if rc != 0:
        raise ValueError("bad NMFA sizes")
    return st, sp, tr
