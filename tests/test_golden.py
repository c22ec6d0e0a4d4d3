"""Oracle pinned to the reference's own execution.

tests/golden/ref_m2opt_n{256,2048}.npz were produced by tests/golden/make_ref_golden.py on a GB300:
the reference's prepare_points and UpdateTwice kernels (compiled from SB/CUDA_GPU/m2_opt.cu by
oracle/build_ref.py) driven as m2_opt.cu:main drives them, with cuBLAS SGEMV for the field.
"""
import os

import numpy as np
import pytest

from annealing_gb300 import instances
from oracle import binding as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [256, 2048]


def load(N):
    d = np.load(os.path.join(GOLDEN, f"ref_m2opt_n{N}.npz"))
    n = int(d["n_spins"])
    J = np.zeros((N, N), np.float32)
    J[:n, :n] = instances.complete_pm1(n, seed=int(d["seed"]))
    return d, J, n


@pytest.mark.parametrize("N", CASES)
def test_reference_init_bit_exact(N):
    d, _, _ = load(N)
    x, y = orc.init_reference(N, d["x0"].shape[0])
    np.testing.assert_array_equal(x, d["x0"])
    np.testing.assert_array_equal(y, d["y0"])


@pytest.mark.parametrize("N", CASES)
def test_update_twice_bit_exact_and_kick_within_sum_order(N):
    """From every recorded reference state, one oracle step reproduces the next recorded state:
    the local MTS update (UpdateTwice) bit for bit, the coupling kick up to cuBLAS's summation
    order (|dy| <= 1e-5 absolute)."""
    d, J, _ = load(N)
    x0, y0, xs, ys = d["x0"], d["y0"], d["xs"], d["ys"]
    T, S = xs.shape[0], xs.shape[1]
    coeff = orc.lib().oracle_asb_coeff(1.0, 0.01565)
    for t in range(T):
        for s in range(S):
            xp = (x0[t] if s == 0 else xs[t, s - 1]).copy()[None, :]
            yp = (y0[t] if s == 0 else ys[t, s - 1]).copy()[None, :]
            orc.asb_local(xp, yp, float(np.float32(s) / np.float32(S)))
            np.testing.assert_array_equal(xp[0], xs[t, s])
            f = orc.field_f32(J, xp)
            ynew = (yp.astype(np.float64) + np.float64(coeff) * f.astype(np.float64)).astype(np.float32)
            assert np.max(np.abs(ynew[0] - ys[t, s])) <= 1e-5


@pytest.mark.parametrize("N", CASES)
def test_trajectory_tracks_reference(N):
    """20 reference steps: positions within 2e-4 of the reference, identical spin signs, hence
    identical reported energies."""
    d, J, n = load(N)
    x, y = d["x0"].copy(), d["y0"].copy()
    xt, _ = orc.asb_run(J, x, y, d["xs"].shape[1], want_trace=True)
    for s in range(xt.shape[0]):
        assert np.max(np.abs(xt[s] - d["xs"][:, s])) <= 2e-4
        assert np.array_equal(xt[s] > 0, d["xs"][:, s] > 0)
    for t in range(x.shape[0]):
        s_ours = np.where(x[t, :n] > 0, 1, -1).astype(np.int8)
        s_ref = np.where(d["xs"][t, -1, :n] > 0, 1, -1).astype(np.int8)
        assert orc.energy_i64(J[:n, :n], None, s_ours) == orc.energy_i64(J[:n, :n], None, s_ref)
