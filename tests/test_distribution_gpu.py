"""Best-energy distributions over 1000 seeds (replicas / trials).

* The plain aSB path against the reference's own program: 1000 trials of m2_opt.cu run on a GB300
  through its own kernels and cuBLAS (tests/golden/ref_m2opt_energies_n2000.npz, made by
  tests/golden/make_ref_energy_dist.py) against 1000 replicas here with the reference's initial
  states (replica r = trial r) on the same instance and schedule. Stated test: two-sample
  Kolmogorov-Smirnov, p >= 0.01, and means within 3 standard errors.
* Batched tensor-core dSB against the plain FP32 kernel over 1000 seeds: integer fields are exact on
  both, so the distributions are identical (equal mean best energy by construction).
"""
import os

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = sb.Context(0)
    yield c
    c.close()


def test_asb_energy_distribution_matches_the_reference_program(ctx):
    stats = pytest.importorskip("scipy.stats")
    d = np.load(os.path.join(GOLDEN, "ref_m2opt_energies_n2000.npz"))
    ref = d["energies"].astype(np.float64)
    J = instances.complete_pm1(int(d["spins"]), seed=int(d["seed"]))
    prm = sb.Params.default(sb.ASB, steps=int(d["steps"]), replicas=int(d["trials"]), field_mode=sb.FIELD_FP32)
    assert prm.init_mode == sb.INIT_REFERENCE
    ours = ctx.solve(sb.Problem.from_dense(J), prm).replica_energies
    ks = stats.ks_2samp(ours, ref)
    assert ks.pvalue >= 0.01, (ks, ours.mean(), ref.mean())
    se = np.sqrt(ours.var() / ours.size + ref.var() / ref.size)
    assert abs(ours.mean() - ref.mean()) <= 3 * se


def test_tensor_core_and_plain_fp32_dsb_distributions_are_identical(ctx):
    J = instances.complete_pm1(2000, seed=11)
    prob = sb.Problem.from_dense(J)
    e = {}
    for mode in (sb.FIELD_TC, sb.FIELD_FP32):
        prm = sb.Params.default(sb.DSB, steps=200, replicas=1000, seed=77, field_mode=mode)
        e[mode] = ctx.solve(prob, prm).replica_energies
    np.testing.assert_array_equal(e[sb.FIELD_TC], e[sb.FIELD_FP32])
    assert e[sb.FIELD_TC].mean() == e[sb.FIELD_FP32].mean()
