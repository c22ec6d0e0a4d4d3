"""SQA oracle (oracle/sqa_oracle.c): its own log, the schedule, the reference initial state, and the
pin against the reference's own SQA kernels (tests/golden/ref_sqa_*.npz, made by
tests/golden/make_sqa_golden.py from SQA_fully/fully_test/pre_calculate.cu run on a GB300).
CPU only."""
import math
import os

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_own_log_accuracy_and_edges():
    rng = np.random.default_rng(0)
    us = np.concatenate([rng.random(4000), np.float32(2.0) ** -np.arange(1, 33), [1.0, 0.5, 0.75]])
    for u in us.astype(np.float32):
        if u <= 0:
            continue
        got = orc.sqa_log(float(u))
        assert abs(got - math.log(float(u))) <= 3e-7 * max(1.0, abs(math.log(float(u))))
    assert orc.sqa_log(0.0) == -math.inf
    assert orc.sqa_log(1.0) == 0.0


def test_schedule_matches_the_library_and_the_reference_formula():
    for steps, M in ((100, 16), (10, 8), (7, 64)):
        b, j = orc.sqa_schedule(steps, M)
        bl, jl = sb.sqa_schedule(steps, M)
        assert np.array_equal(b, bl) and np.array_equal(j, jl)
        assert b[0] == np.float32(1 / 16)
        inc = np.float32((8 - np.float32(1 / 16)) / np.float32(steps))
        for p in range(1, steps):
            assert b[p] == np.float32(b[p - 1] + inc)  # beta += increase, in float
        for p in range(steps):
            gamma = 8.0 * (1.0 - p / steps)
            ref = -0.5 * math.log(math.tanh(gamma / M * float(b[p]))) / float(b[p])
            assert abs(float(j[p]) - ref) <= 1e-5 * abs(ref)


def _xorshift32(x):
    x ^= (x << 13) & 0xFFFFFFFF
    x ^= x >> 17
    x ^= (x << 5) & 0xFFFFFFFF
    return x


def test_reference_initial_state():
    n, M, R = 40, 6, 3
    s, rnd = orc.sqa_init(n, M, R, 0)
    for i in (0, 1, 17, 39):
        st = i
        for r in range(R):
            for m in range(M):
                st = _xorshift32(st)
                assert s[r, m, i] == ((st & 1) << 1) - 1
            assert rnd[r, i] == st
    assert (s[:, :, 0] == -1).all() and (rnd[:, 0] == 0).all()  # xorshift32(0) = 0


def test_oracle_anneal_lowers_the_energy():
    n, M, R, steps = 96, 8, 2, 30
    J = instances.complete_pm1(n, seed=3)
    s, _ = orc.sqa_init(n, M, R, 1, seed=9)
    e0 = [orc.sqa_energy(J, s[r, 0]) for r in range(R)]
    tr = orc.sqa_run(J, s, steps, 1, seed=9)
    assert all(tr[r, -1] == orc.sqa_energy(J, s[r, 0]) for r in range(R))
    assert all(tr[r, -1] < e0[r] - 100 for r in range(R))


@pytest.mark.parametrize("N,M", [(256, 8), (512, 16)])
def test_oracle_matches_the_reference_kernels(N, M):
    d = np.load(os.path.join(GOLDEN, f"ref_sqa_n{N}_m{M}.npz"))
    J = d["J"].astype(np.float32)
    trials, steps = d["energy"].shape
    s, rnd = orc.sqa_init(N, M, trials, 0)
    # the reference stores spin-major s[i * M + m]; the oracle slice-major [r][m][i]
    assert np.array_equal(s, d["init"].transpose(0, 2, 1))
    assert np.array_equal(rnd, d["rnd"])
    b, j = orc.sqa_schedule(steps, M)
    assert np.array_equal(b, d["beta"]) and np.array_equal(j, d["jperp"])
    for p in range(steps):  # one step at a time, compared after every step
        tr = orc.sqa_run(J, s, 1, 0, rnd=rnd, beta=d["beta"][p:p + 1], jperp=d["jperp"][p:p + 1])
        assert np.array_equal(s, d["spins"][:, p].transpose(0, 2, 1)), f"step {p}"
        assert np.array_equal(tr[:, 0], d["energy"][:, p])
