"""NMFA oracle and host logic (no GPU): the oracle pinned to the reference's own kernel, its random
streams restated independently from NMFA/CUDA_GPU/src/nmfa.cu, its FP32 functions against libm, and
the library's schedule against NMFA/CUDA_GPU/Ising.cpp."""
import math
import os

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
M32 = 0xFFFFFFFF


def _xorshift32(t):
    """nmfa.cu:43-47"""
    t ^= (t << 13) & M32
    t ^= t >> 17
    t ^= (t << 5) & M32
    return t


def _xorwow(s):
    """nmfa.cu:29-40 on s = [s0, s1, s2, s3, s4]; returns the draw."""
    t = s[3]
    t ^= t >> 2
    t ^= (t << 1) & M32
    s[3], s[2], s[1] = s[2], s[1], s[0]
    t ^= s[0]
    t ^= (s[0] << 4) & M32
    s[0] = t
    s[4] = (s[4] + 362437) & M32
    return (t + s[4]) & M32


def test_random_streams_match_the_reference_macros():
    """Seeding (nmfa.cu:62-76: seed + blockDim.x * blockIdx.x + threadIdx.x, four xorshift32 steps)
    and XORWOW draws, restated here in Python, equal the oracle's words."""
    n, R, seed = 7, 3, 4294967290  # the seed wraps around 2^32 within the first sample
    w = orc.nmfa_seed(n, R, seed)
    for r in range(R):
        for i in range(n):
            t = (seed + n * r + i) & M32
            ref = []
            for _ in range(4):
                t = _xorshift32(t)
                ref.append(t)
            assert list(w[r, i, :4]) == ref and w[r, i, 4] == 0
    s = [int(v) for v in w[1, 2]]
    ws = w[1, 2].copy()
    for _ in range(50):
        assert orc.lib().oracle_nmfa_xorwow(ws) == _xorwow(s)
    assert list(ws) == s


def test_gaussian_noise():
    """Box-Muller from the XORWOW words: the radius and angle use the words as nmfa.cu:106-107 does;
    20000 draws have mean 0 and standard deviation sigma."""
    w = orc.nmfa_seed(1, 1, 77)[0, 0].copy()
    z = np.array([orc.nmfa_gauss(w, 0.5) for _ in range(10000)]).ravel()
    assert abs(z.mean()) < 0.02 and abs(z.std() - 0.5) < 0.01
    w = orc.nmfa_seed(1, 1, 77)[0, 0].copy()
    s = [int(v) for v in w]
    z0, z1 = orc.nmfa_gauss(w, 1.0)
    a, b = _xorwow(s), _xorwow(s)
    rad = math.sqrt(-2.0 * math.log(a / 2**32))
    ang = b / 2**32 * 2 * math.pi
    assert abs(z0 - math.sin(ang) * rad) < 1e-5 * (1 + rad) and abs(z1 - math.cos(ang) * rad) < 1e-5 * (1 + rad)


def test_own_functions_against_libm():
    xs = np.concatenate([np.linspace(-12, 12, 20001), np.float32([1e-30, 1e-7, -1e-5, 1e-3, 0.25, 9.9, 10.1])])
    err = max(abs(orc.nmfa_tanh(float(x)) - math.tanh(float(np.float32(x)))) for x in xs)
    assert err < 3e-7
    for x in (1e-6, 1e-3, 0.1, 0.6):
        assert abs(orc.nmfa_tanh(x) / math.tanh(x) - 1) < 3e-7
    assert orc.nmfa_tanh(0.0) == 0.0 and orc.nmfa_tanh(50.0) == 1.0 and orc.nmfa_tanh(-50.0) == -1.0
    assert math.isnan(orc.nmfa_tanh(float("nan")))
    ts = np.linspace(0.0, 2 * math.pi, 20001)
    e = max(max(abs(s - math.sin(float(np.float32(t)))), abs(c - math.cos(float(np.float32(t)))))
            for t in ts for (s, c) in [orc.nmfa_sincos(float(t))])
    assert e < 2e-7


def test_schedule_matches_ising_cpp():
    """Ising.cpp:37-43 in FP32; the library's sb_nmfa_schedule and the oracle's agree."""
    inc = np.float32((np.float32(8) - np.float32(1) / np.float32(16)) / np.float32(100))
    b, ref = np.float32(1) / np.float32(16), []
    for _ in range(100):
        ref.append(b)
        b = np.float32(b + inc)
    assert np.array_equal(orc.nmfa_schedule(100), np.array(ref, np.float32))
    assert np.array_equal(sb.nmfa_schedule(100), orc.nmfa_schedule(100))


def test_oracle_against_reference_one_warp():
    """N = 32 (one warp, race-free in the reference): the oracle's states after the first K stages
    against the reference kernel's (tests/golden/ref_nmfa_n32.npz); the bounds of the GPU test."""
    g = np.load(os.path.join(GOLDEN, "ref_nmfa_n32.npz"))
    J = g["J"].astype(np.float32)
    full = orc.nmfa_schedule(100)
    R = int(g["samples"])
    _, _, trace = orc.nmfa_run(J, R, full, 0.15, 0.15, 1234, trace=True)
    for K in g["ks"]:
        d = np.abs(trace[K - 1] - g[f"states_k{K}"])
        if K <= 2:
            assert d.max() <= 2e-3
        assert np.quantile(d, 0.99) <= 2e-3
    assert np.mean((trace[-1] > 0) == (g["states_k100"] > 0)) >= 0.99


def test_oracle_energy_mean_four_warps():
    """N = 128: 300 oracle samples' mean energy within 4 standard errors of the reference kernel's
    1000 (the full two-sample test runs on the GPU path, which equals the oracle bit for bit)."""
    g = np.load(os.path.join(GOLDEN, "ref_nmfa_n128.npz"))
    J = instances.nmfa_fully(128, int(g["seed"]))
    _, sp, _ = orc.nmfa_run(J, 300, orc.nmfa_schedule(100), 0.15, 0.15, 555)
    s = sp.astype(np.int64)
    e = np.einsum("ri,ij,rj->r", s, J.astype(np.int64), s) // 2
    ref = g["energies"].astype(np.float64)
    se = math.sqrt(e.var() / len(e) + ref.var() / len(ref))
    assert abs(e.mean() - ref.mean()) <= 4 * se


def test_oracle_rejects_bad_sizes():
    with pytest.raises(ValueError):
        orc.nmfa_run(np.zeros((4, 4), np.float32), 0, orc.nmfa_schedule(3))
