"""The CPU oracle against independent restatements of the reference and against itself (CPU)."""
import json
import os

import numpy as np
import pytest

from annealing_gb300 import instances
from oracle import binding as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def xorshift32(v):
    # SB/CUDA_GPU/m2_opt.cu:38-46
    v ^= (v << 13) & 0xFFFFFFFF
    v ^= v >> 17
    v ^= (v << 5) & 0xFFFFFFFF
    return v


def ref_value(u):
    # m2_opt.cu:54 — (u / (float)MAX) / 10.0 ; (float)4294967295.0 == 2**32
    q = np.float32(np.float32(u) / np.float32(4294967296.0))
    return np.float32(np.float64(q) / 10.0)


def test_reference_init_matches_prepare_points():
    n, R = 300, 3
    x, y = orc.init_reference(n, R)
    for i in range(n):
        st = i
        for r in range(R):
            st = xorshift32(st)
            ux = st
            st = xorshift32(st)
            uy = st
            assert x[r, i] == ref_value(ux)
            assert y[r, i] == ref_value(uy)
    assert np.all(x[:, 0] == 0) and np.all(y[:, 0] == 0)  # xorshift32(0) == 0
    assert np.all((x >= 0) & (x < 0.1))


def _mix64(z):
    M = (1 << 64) - 1
    z ^= z >> 30
    z = (z * 0xBF58476D1CE4E5B9) & M
    z ^= z >> 27
    z = (z * 0x94D049BB133111EB) & M
    z ^= z >> 31
    return z


def test_uniform_init_hash_restated():
    n, R, seed = 37, 4, 99
    x, y = orc.init_uniform(n, R, seed)
    for r in range(R):
        for i in range(n):
            for which, arr in ((0, x), (1, y)):
                e = 2 * (r * n + i) + which
                z = _mix64((seed + 0x9E3779B97F4A7C15 * (e + 1)) & ((1 << 64) - 1))
                u = z >> 40
                f = np.float32(u) * np.float32(2.0 ** -24)
                v = np.float32(np.float32(f * np.float32(2.0) - np.float32(1.0)) * np.float32(0.1))
                assert arr[r, i] == v
    assert np.all((x >= -0.1) & (x < 0.1))
    x2, _ = orc.init_uniform(n, R, seed + 1)
    assert not np.array_equal(x, x2)


def test_pump_schedule_is_linear_and_below_one():
    steps = 1000
    p = np.array([orc.pump(1.0, t, steps) for t in range(steps)], np.float32)
    assert p[0] == 1.0
    assert np.all(np.diff(p) < 0)
    assert abs(p[-1] - 1.0 / steps) < 1e-6  # a(t) never reaches a0 (m2_opt.cu:158 form)


def test_c0_definition():
    J = instances.complete_pm1(64, seed=3)
    off = J[~np.eye(64, dtype=bool)].astype(np.float64)
    sd = off.std()
    assert abs(orc.coupling_std(J) - sd) < 1e-12
    assert orc.default_c0(J) == np.float32(0.5 / (np.sqrt(64) * sd))


def test_energy_int64_and_f64_agree_with_bruteforce():
    rng = np.random.default_rng(0)
    n = 50
    J = instances.erdos_renyi(n, 0.6, seed=5, jmax=8, allow_zero=True)
    h = rng.integers(-3, 4, size=n).astype(np.float32)
    s = (rng.integers(0, 2, size=n) * 2 - 1).astype(np.int8)
    ss = s.astype(np.int64)
    brute = -int(np.sum(np.triu(J.astype(np.int64), 1) * np.outer(ss, ss))) - int(np.dot(h.astype(np.int64), ss))
    assert orc.energy_i64(J, h, s) == brute
    assert orc.energy_f64(J, h, s) == brute
    Jb = J.copy()
    Jb[0, 1] = Jb[1, 0] = 0.5
    with pytest.raises(ValueError):
        orc.energy_i64(Jb, None, s)


def test_asb_local_restated_in_double():
    n = 64
    x, y = orc.init_reference(n, 2)
    x2, y2 = x.copy(), y.copy()
    orc.asb_local(x, y, 0.35)
    for k in np.ndindex(x2.shape):
        lx, ly = x2[k], y2[k]
        for _ in range(2):
            lx = np.float32(np.float64(lx) + 1.0 * np.float64(ly) * 0.5)
            ly = np.float32(np.float64(ly) - 0.5 * (1.0 * np.float64(lx) * np.float64(lx) * np.float64(lx)
                                                   + (1.0 - np.float64(np.float32(0.35))) * np.float64(lx)))
        assert x[k] == lx and y[k] == ly


def test_dsb_fp32_tracks_fp64_for_first_steps():
    n, R, steps = 128, 4, 40
    J = instances.complete_pm1(n, seed=9)
    c0 = orc.default_c0(J)
    x0, y0 = orc.init_uniform(n, R, 5)
    x, y = x0.copy(), y0.copy()
    orc.sb_run_f32(2, J, None, x, y, steps, 1.0, c0, 1.25)
    xd, yd = orc.sb_run_f64(2, J, None, x0, y0, steps, 1.0, float(c0), 1.25)
    # 40 steps of dSB stay within FP32 rounding of the FP64 trajectory
    assert np.max(np.abs(x - xd)) < 1e-4


def test_bsb_energy_trace_decreases():
    n, R, steps = 200, 8, 300
    J = instances.complete_pm1(n, seed=2)
    x, y = orc.init_uniform(n, R, 1)
    tr, _ = orc.sb_run_f32(1, J, None, x, y, steps, 1.0, orc.default_c0(J), 1.25, trace=True)
    assert tr[-1] < tr[0] and tr[-1] < -0.6 * n ** 1.5  # SK-type instance: E0 ~ -0.763 N^1.5


def test_cpu_baseline_matches_oracle_for_integer_dsb():
    n, R, steps = 100, 12, 25
    J = instances.erdos_renyi(n, 0.7, seed=4, jmax=3, allow_zero=True)
    c0 = orc.default_c0(J)
    x0, y0 = orc.init_uniform(n, R, 8)
    xa, ya = x0.copy(), y0.copy()
    orc.sb_run_f32(2, J, None, xa, ya, steps, 1.0, c0, 1.25)
    xb, yb = x0.copy(), y0.copy()
    orc.cpu_run(2, J, None, xb, yb, steps, 1.0, c0, 1.25, threads=3)
    assert np.array_equal(xa, xb) and np.array_equal(ya, yb)


def test_cpu_baseline_asb_close_to_oracle():
    n, R, steps = 96, 3, 10
    J = instances.complete_pm1(n, seed=6)
    x0, y0 = orc.init_reference(n, R)
    xa, ya = x0.copy(), y0.copy()
    orc.asb_run(J, xa, ya, steps)
    xb, yb = x0.copy(), y0.copy()
    orc.cpu_run(0, J, None, xb, yb, steps, threads=2)
    assert np.max(np.abs(xa - xb)) < 1e-4


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "ref_energy_band.json")),
                    reason="energy band fixture not generated")
def test_asb_energy_distribution_matches_reference_band():
    """The reference's published 20-step results (100 trials, N=2048 build, a 2000-spin complete
    +-1 instance) as a statistical band for the oracle on a synthetic instance of the same class."""
    band = json.load(open(os.path.join(GOLDEN, "ref_energy_band.json")))["opt"]
    n_build, n_spins, steps, trials = 2048, 2000, 20, 100
    J = np.zeros((n_build, n_build), np.float32)
    J[:n_spins, :n_spins] = instances.complete_pm1(n_spins, seed=1234)
    x, y = orc.init_reference(n_build, trials)
    orc.cpu_run(0, J, None, x, y, steps)
    s = np.where(x[:, :n_spins] > 0, 1, -1).astype(np.int8)
    e = np.array([orc.energy_i64(J[:n_spins, :n_spins], None, s[r]) for r in range(trials)])
    assert abs(e.mean() - band["mean"]) < 0.02 * abs(band["mean"])
    assert 0.5 * band["std"] < e.std() < 2.0 * band["std"]
